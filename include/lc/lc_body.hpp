/* lc_body.hpp — Physics::CudaDeformableBody on the licenta_gb300 engine, for
 * C++ hosts.
 *
 * A header-only adapter over the C ABI of lc.h with the reference body's
 * constructor arguments and methods (Physics/CudaDeformableBody.h:23-28):
 *
 *   CudaDeformableBody(std::vector<VertexT> *verts, std::vector<unsigned> *indices,
 *                      const lc_cloth_params params, std::vector<bool> &fixedVerts)
 *   FixedUpdate()  — one cloth step (Physics/CudaDeformableBody.cpp:550-627)
 *   Update()       — publishes the positions into *verts
 *                    (Physics/CudaDeformableBody.cpp:629-638, 473-495)
 *   SetSpherePos(pos, radius)   (Physics/CudaDeformableBody.cpp:640-643)
 *   Autotune(steps, warmup, allow_variants) — picks the launch shapes with
 *                    the library's autotuner (no counterpart in the reference)
 *
 * and lc::CollisionMethod<Id>, Collision::ICollisionMethod over the engine's
 * object-level broadphase (lc_broadphase_*).
 *
 * VertexT is any vertex record with a `m_position` member that has float x,
 * y, z fields — Rendering::VertexFormat (glm::vec3 m_position) qualifies.
 * As in the reference, the caller owns *verts and *indices and the body keeps
 * the pointer to *verts, writing the published positions (the previous
 * positions after the step, as the reference's FinalVertUpdate does) back
 * into it on Update().  Errors throw lc::Error with the engine's message
 * (the reference exits the process instead).
 *
 * The body steps on the default stream and waits for the step in Update();
 * several bodies are better stepped together through lc_batch_* directly.
 */
#pragma once

#include <algorithm>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "lc.h"

namespace lc {

struct Error : std::runtime_error {
    lc_status status;
    Error(lc_status s, const std::string &where)
        : std::runtime_error(where + ": " + lc_status_string(s) + " (" + lc_last_error_string() + ")"), status(s) {}
};

inline void check(lc_status s, const char *where) {
    if (s != LC_OK) throw Error(s, where);
}

template <class VertexT>
class CudaDeformableBody {
public:
    CudaDeformableBody(std::vector<VertexT> *verts, std::vector<unsigned int> *indices, const lc_cloth_params params,
                       std::vector<bool> &fixedVerts)
        : m_verts(verts) {
        if (!verts || !indices || indices->size() % 3 != 0 || fixedVerts.size() != verts->size())
            throw std::invalid_argument("CudaDeformableBody: inconsistent vertices / indices / fixedVerts");
        const size_t V = verts->size();
        std::vector<float> pos(3 * V);
        for (size_t i = 0; i < V; ++i) {
            pos[3 * i] = (*verts)[i].m_position.x;
            pos[3 * i + 1] = (*verts)[i].m_position.y;
            pos[3 * i + 2] = (*verts)[i].m_position.z;
        }
        std::vector<uint8_t> pinned(V);
        for (size_t i = 0; i < V; ++i) pinned[i] = fixedVerts[i] ? 1 : 0;
        lc_cloth_desc d;
        d.num_vertices = (int32_t)V;
        d.num_triangles = (int32_t)(indices->size() / 3);
        d.positions = pos.data();
        d.indices = reinterpret_cast<const uint32_t *>(indices->data());
        d.pinned = pinned.data();
        d.params = params;
        lc_batch_options o;
        lc_default_options(&o);
        check(lc_batch_create(&d, 1, &o, &m_batch), "lc_batch_create");
        m_published.resize(3 * V);
    }

    CudaDeformableBody(const CudaDeformableBody &) = delete;
    CudaDeformableBody &operator=(const CudaDeformableBody &) = delete;

    virtual ~CudaDeformableBody() {
        if (m_batch) lc_batch_destroy(m_batch);
    }

    virtual void FixedUpdate() { check(lc_batch_step(m_batch, 1, nullptr), "lc_batch_step"); }

    virtual void Update() {
        check(lc_batch_sync(m_batch), "lc_batch_sync");
        check(lc_batch_read_positions(m_batch, m_published.data(), 1, nullptr), "lc_batch_read_positions");
        check(lc_batch_sync(m_batch), "lc_batch_sync");
        for (size_t i = 0; i < m_verts->size(); ++i) {
            (*m_verts)[i].m_position.x = m_published[3 * i];
            (*m_verts)[i].m_position.y = m_published[3 * i + 1];
            (*m_verts)[i].m_position.z = m_published[3 * i + 2];
        }
    }

    template <class Vec3>
    void SetSpherePos(const Vec3 &pos, float radius) {
        const float p[3] = {pos.x, pos.y, pos.z};
        check(lc_batch_set_sphere(m_batch, 0, p, radius), "lc_batch_set_sphere");
    }

    // Times the library's default space of launch shapes on the body's
    // current state (lc_batch_autotune; the state is restored) and keeps the
    // fastest.  With allow_variants false the solver variant stays, and the
    // body's trajectory is bit-identical to the untuned one.
    lc_tuning Autotune(int steps = 3, int warmup = 1, bool allow_variants = false) {
        lc_tuning best;
        float ms = 0.f;
        check(lc_batch_autotune(m_batch, nullptr, steps, warmup, allow_variants ? 1 : 0, nullptr, &best, &ms,
                                nullptr, 0, nullptr),
              "lc_batch_autotune");
        return best;
    }

    lc_batch *batch() { return m_batch; }

private:
    std::vector<VertexT> *m_verts;
    lc_batch *m_batch = nullptr;
    std::vector<float> m_published;
};

// Collision::ICollisionMethod (Collision/ICollisionMethod.h:15-87) over an
// lc_broadphase: objects are ids of type Id with an axis-aligned box each.
// ObjectAdded / ObjectMoved / ObjectRemoved edit a host box table, Update()
// copies it to the device and builds the method's structure, TestCollision()
// returns the pairs of ids whose boxes overlap, and GetLastFrameCriteria()
// the reference's per-frame criteria under its keys (Core/Utils.hpp:42-46).
template <class Id>
class CollisionMethod {
public:
    explicit CollisionMethod(const lc_broadphase_desc &desc) : max_(desc.max_objects) {
        check(lc_broadphase_create(&desc, &h_), "lc_broadphase_create");
    }
    ~CollisionMethod() { lc_broadphase_destroy(h_); }
    CollisionMethod(const CollisionMethod &) = delete;
    CollisionMethod &operator=(const CollisionMethod &) = delete;

    void ObjectAdded(const Id &id, const float box_min[3], const float box_max[3]) {
        if (slot_.count(id)) throw std::invalid_argument("ObjectAdded: id already present");
        if ((int)ids_.size() >= max_) throw std::length_error("ObjectAdded: more objects than max_objects");
        slot_[id] = ids_.size();
        ids_.push_back(id);
        lo_.insert(lo_.end(), box_min, box_min + 3);
        hi_.insert(hi_.end(), box_max, box_max + 3);
    }
    void ObjectMoved(const Id &id, const float box_min[3], const float box_max[3]) {
        const size_t s = slot_.at(id);
        std::copy(box_min, box_min + 3, lo_.begin() + 3 * s);
        std::copy(box_max, box_max + 3, hi_.begin() + 3 * s);
    }
    void ObjectRemoved(const Id &id) {
        const size_t s = slot_.at(id), last = ids_.size() - 1;
        slot_.erase(id);
        if (s != last) {  // the last object takes the freed slot
            ids_[s] = ids_[last];
            slot_[ids_[s]] = s;
            std::copy(lo_.begin() + 3 * last, lo_.begin() + 3 * last + 3, lo_.begin() + 3 * s);
            std::copy(hi_.begin() + 3 * last, hi_.begin() + 3 * last + 3, hi_.begin() + 3 * s);
        }
        ids_.pop_back();
        lo_.resize(3 * last);
        hi_.resize(3 * last);
    }
    void Update() {
        check(lc_broadphase_update_host(h_, lo_.data(), hi_.data(), (int32_t)ids_.size(), nullptr),
              "lc_broadphase_update_host");
    }
    std::vector<std::pair<Id, Id>> TestCollision() {
        uint64_t n = 0;
        lc_status s = lc_broadphase_test_host(h_, host_.data(), host_.size() / 2, &n, nullptr);
        if (s == LC_ERR_CAPACITY_OVERFLOW) {  // grow to the count and ask again
            host_.resize(2 * n);
            s = lc_broadphase_test_host(h_, host_.data(), n, &n, nullptr);
        }
        check(s, "lc_broadphase_test_host");
        std::vector<std::pair<Id, Id>> out(n);
        for (uint64_t k = 0; k < n; ++k) out[k] = {ids_[host_[2 * k]], ids_[host_[2 * k + 1]]};
        lc_broadphase_criteria c{};
        check(lc_broadphase_get_criteria(h_, &c), "lc_broadphase_get_criteria");
        criteria_ = {{"Time Spent - Collisions", c.collision_ms},
                     {"Time Spent - Structure Update", c.structure_ms},
                     {"Intersection Tests", (float)c.intersection_tests},
                     {"Memory Used (KB)", (float)c.memory_bytes / 1024.f}};
        return out;
    }
    std::unordered_map<std::string, float> GetLastFrameCriteria() const { return criteria_; }

private:
    lc_broadphase *h_ = nullptr;
    int max_;
    std::vector<Id> ids_;
    std::unordered_map<Id, size_t> slot_;
    std::vector<float> lo_, hi_;
    std::vector<uint32_t> host_;
    std::unordered_map<std::string, float> criteria_;
};

}  // namespace lc
