// lc_oracle.hpp — CPU oracle of the reference's GPU cloth step.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++, the algorithm
// of the reference's GPU cloth body (Tureyz/Licenta; paths relative to
// LicentaV2/LicentaV2/) so that tests, smoke() and the CPU-baseline leg of
// bench.py can check the CUDA engine against it.  Nothing in the product
// (licenta_gb300/) includes, links or calls it.
//
// Parity status.  The collision stages (Morton codes, stable sort, Karras
// topology, refit boxes and rightmost leaves, traversal pairs, candidate
// generation, feature AABB cull, CCD contacts) are PINNED against the
// reference's own kernels: oracle/ref_pin/build_ref.py compiles the
// reference's CUDA sources for sm_103a, oracle/ref_pin/refchain.py runs its
// collision chain on a GPU, and the outputs are committed as golden vectors
// under tests/golden/ (generator: tests/golden/make_golden.py), which this
// restatement reproduces bit for bit.  The pin settled two points where the
// reference's source alone is ambiguous: its refit races (see refit()) and
// its unset critical point reads as the first root (see critical_points()).
// The PBD solver half is checked FP32 against FP64 (same scheme, teacher
// forced); it is not pinned against the reference's solver kernels.
//
// The class is templated on the real type R.  R = float is the FP32 mirror:
// the same operation order as the reference kernels (no FMA contraction, the
// build uses -ffp-contract=off), so integer/contact results are bit-exact for
// identical inputs.  R = double is the FP64 oracle the positions are compared
// against.  The vector length is sqrt(x*x+y*y+z*z) in both modes (the
// reference's norm3df is CUDA library code and is not reproduced).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <utility>
#include <vector>

#include "../include/lc/lc.h"

namespace lco {

using u8 = uint8_t;
using u32 = uint32_t;
using u64 = uint64_t;

// ---------------------------------------------------------------------------
// float3 algebra — Core/CudaUtils.cu:32-107, 139-276 (operation order kept).
// ---------------------------------------------------------------------------
template <class R> struct V3 {
    R x, y, z;
};
template <class R> inline V3<R> mk(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> inline V3<R> operator-(V3<R> a) { return mk(-a.x, -a.y, -a.z); }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return mk(a.x * s, a.y * s, a.z * s); }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return mk(a.x / s, a.y / s, a.z / s); }
template <class R> inline V3<R> addc(V3<R> a, R s) { return mk(a.x + s, a.y + s, a.z + s); }
template <class R> inline V3<R> subc(V3<R> a, R s) { return mk(a.x - s, a.y - s, a.z - s); }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> inline R len(V3<R> a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <class R> inline R dist(V3<R> a, V3<R> b) { return len(a - b); }
template <class R> inline V3<R> normalize(V3<R> a) { return a / len(a); }
template <class R> inline bool is_zero(V3<R> a) { return a.x == R(0) && a.y == R(0) && a.z == R(0); }
template <class R> inline V3<R> vmin(V3<R> a, V3<R> b) { return mk(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
template <class R> inline V3<R> vmax(V3<R> a, V3<R> b) { return mk(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
template <class R> inline V3<R> min3(V3<R> a, V3<R> b, V3<R> c) { return vmin(a, vmin(b, c)); }
template <class R> inline V3<R> max3(V3<R> a, V3<R> b, V3<R> c) { return vmax(a, vmax(b, c)); }
template <class R> inline R clampf(R v, R lo, R hi) { return std::fmin(std::fmax(lo, v), hi); }
template <class R> inline bool between(R v, R lo, R hi) { return v >= lo && v <= hi; }
// Core/CudaUtils.cu:364-371 — closed-interval overlap.
template <class R> inline bool overlap(V3<R> amin, V3<R> amax, V3<R> bmin, V3<R> bmax) {
    bool a = amax.x < bmin.x || amin.x > bmax.x;
    bool b = amax.y < bmin.y || amin.y > bmax.y;
    bool c = amax.z < bmin.z || amin.z > bmax.z;
    return !(a || b || c);
}

// Constants of the reference.
static const double kEpsPbd = 0.00000001;      // Physics/CudaPBD.cu:33 (and Core/CudaUtils.cu:4)
static const double kEpsCubic = 1.0 / 1000000;  // Physics/CudaCubicSolver.cuh:12
static const double kEpsEE = 0.000000001;       // Collision/CudaPrimitiveTests.cu:124
static const float kPi = 3.14159265359f;        // Physics/CudaPBD.cu:35

// ---------------------------------------------------------------------------
// Morton codes — Core/CudaUtils.cu:278-325 (REF63 live encoder) and the
// commented-out 30-bit encoder at :289-308 (K30).  Bit k of each axis lands
// at bit 3k (+2 for x, +1 for y), the interleave of ExpandBy2.
// ---------------------------------------------------------------------------
inline u64 spread_bits(u64 v, int nbits) {
    u64 r = 0;
    for (int k = 0; k < nbits; ++k)
        if ((v >> k) & 1u) r |= u64(1) << (3 * k);
    return r;
}
inline u64 quantize(float x, int mode) {
    if (mode == LC_MORTON_K30) {
        float q = std::fmin(std::fmax(x * 1024.f, 0.0f), 1023.0f);
        return (u64)q;
    }
    float q = std::fmin(std::fmax(x * 2097152.f, 0.0f), 2097151.0f);
    return (u64)q;
}
inline u64 morton3d(float x, float y, float z, int mode) {
    int nb = mode == LC_MORTON_K30 ? 10 : 21;
    return (spread_bits(quantize(x, mode), nb) << 2) + (spread_bits(quantize(y, mode), nb) << 1) +
           spread_bits(quantize(z, mode), nb);
}

inline int clz64(u64 v) { return v ? __builtin_clzll(v) : 64; }

// Core/CudaUtils.cu:338-351
inline int delta(const u64 *m, int i, int j, int maxi) {
    if (j < 0 || j > maxi) return -1;
    u64 x = m[i] ^ m[j];
    return x ? clz64(x) : clz64(u64(i) ^ u64(j)) + 64;
}
// Core/CudaUtils.cu:353-362 — sgn(0) = +1.
inline int sgn(int a) { return std::signbit((float)a) ? -1 : 1; }

// Collision/CudaBVH.cu:190-212
inline void find_range(const u64 *m, int count, int id, int &first, int &last) {
    int d = sgn(delta(m, id, id + 1, count) - delta(m, id, id - 1, count));
    int delmin = delta(m, id, id - d, count);
    int lmax = 2;
    while (delta(m, id, id + lmax * d, count) > delmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(m, id, id + (l + t) * d, count) > delmin) l += t;
    int j = id + l * d;
    first = std::min(id, j);
    last = std::max(id, j);
}
// Collision/CudaBVH.cu:214-242 — code-only prefix, no index tiebreak.
inline int find_split(const u64 *m, int first, int last) {
    u64 fc = m[first], lc = m[last];
    if (fc == lc) return (first + last) >> 1;
    int com = clz64(fc ^ lc);
    int split = first, step = last - first;
    do {
        step = (step + 1) >> 1;
        int ns = split + step;
        if (ns < last) {
            if (clz64(fc ^ m[ns]) > com) split = ns;
        }
    } while (step > 1);
    return split;
}

// ---------------------------------------------------------------------------
// Topology built once per cloth (constructor work).
// ---------------------------------------------------------------------------
struct Topology {
    int V = 0, T = 0;
    std::vector<u32> idx;        // 3T, original triangle order
    std::vector<u8> pinned;      // V
    std::vector<u8> features;    // T, per original triangle (bits 5..0)
    std::vector<int> s1, s2;     // stretch constraints
    std::vector<double> sl0;
    std::vector<int> b1, b2, b3, b4;  // bend constraints (p1,p2 shared, p3,p4 opposite)
    std::vector<int> soff;       // V+1 static CSR offsets (Physics/CudaPBD.cu:146-186)
    std::vector<int> sent;       // entries: kind<<30 | role<<28 | constraint
    std::vector<int> fixed;      // pinned ids (Physics/CudaPBD.cu:48-58)
    std::vector<double> lra_l0;  // V*F
    std::vector<double> kst, kbd;  // per-constraint stiffness
    bool tri_bend = false;       // bends are triangle bends (b1, b2, b3 = b0, b1, v; th0 rest heights)
    std::vector<double> th0;
    double vmass = 0;
};

enum { ENT_STRETCH = 0, ENT_BEND = 1 };

// Rendering/VisualBodyFactory.cpp:343-391 topology (used by tests through
// the C API); positions are supplied by the caller.
inline void grid_indices(int rows, int cols, std::vector<u32> &out) {
    out.clear();
    for (int i = 0; i < rows - 1; ++i)
        for (int j = 0; j < cols - 1; ++j) {
            if ((i + j) % 2 == 0) {
                u32 t[6] = {u32(rows * i + j), u32(rows * (i + 1) + j), u32(rows * i + j + 1),
                            u32(rows * i + j + 1), u32(rows * (i + 1) + j), u32(rows * (i + 1) + j + 1)};
                out.insert(out.end(), t, t + 6);
            } else {
                u32 t[6] = {u32(rows * i + j), u32(rows * (i + 1) + j), u32(rows * (i + 1) + j + 1),
                            u32(rows * (i + 1) + j + 1), u32(rows * i + j + 1), u32(rows * i + j)};
                out.insert(out.end(), t, t + 6);
            }
        }
}

inline double ddist(const float *p, int a, int b) {
    double dx = (double)p[3 * a] - p[3 * b], dy = (double)p[3 * a + 1] - p[3 * b + 1],
           dz = (double)p[3 * a + 2] - p[3 * b + 2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// Physics/CudaPBD.cu:289-370 — shared pair (p1,p2) and the opposite vertices.
inline void bend_ids(const int t1[3], const int t2[3], int &p1, int &p2, int &p3, int &p4) {
    p1 = p2 = p3 = p4 = -1;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (t1[i] == t2[j]) { p1 = t1[i]; break; }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (t1[i] == t2[j] && t1[i] != p1) { p2 = t1[i]; break; }
    for (int i = 0; i < 3; ++i)
        if (t1[i] != p1 && t1[i] != p2) { p3 = t1[i]; break; }
    for (int i = 0; i < 3; ++i)
        if (t2[i] != p1 && t2[i] != p2) { p4 = t2[i]; break; }
}

inline void build_topology(const lc_cloth_desc &d, Topology &tp) {
    tp.V = d.num_vertices;
    tp.T = d.num_triangles;
    tp.idx.assign(d.indices, d.indices + 3 * tp.T);
    tp.pinned.assign(tp.V, 0);
    if (d.pinned)
        for (int i = 0; i < tp.V; ++i) tp.pinned[i] = d.pinned[i] ? 1 : 0;
    const float *P = d.positions;
    // Physics/CudaDeformableBody.cpp:52 — vertex mass = objectMass / vertex count.
    tp.vmass = (double)(d.params.objectMass / (float)tp.V);

    // Physics/CudaPBD.cu:111-142 — first sighting of an undirected edge makes a
    // stretch constraint, the second makes a bend constraint and forgets it.
    std::map<std::pair<int, int>, int> open;  // edge -> triangle index
    for (int t = 0; t < tp.T; ++t) {
        int tri[3] = {(int)tp.idx[3 * t], (int)tp.idx[3 * t + 1], (int)tp.idx[3 * t + 2]};
        for (int j = 0; j < 3; ++j) {
            int a = tri[j], b = tri[(j + 1) % 3];
            std::pair<int, int> key(std::min(a, b), std::max(a, b));
            auto it = open.find(key);
            if (it != open.end()) {
                int o = it->second;
                int t1[3] = {(int)tp.idx[3 * o], (int)tp.idx[3 * o + 1], (int)tp.idx[3 * o + 2]};
                int p1, p2, p3, p4;
                bend_ids(t1, tri, p1, p2, p3, p4);
                tp.b1.push_back(p1); tp.b2.push_back(p2); tp.b3.push_back(p3); tp.b4.push_back(p4);
                open.erase(it);
            } else {
                open[key] = t;
                tp.s1.push_back(a);
                tp.s2.push_back(b);
                tp.sl0.push_back(ddist(P, a, b));
            }
        }
    }
    if (d.params.useTriangleBending) {
        // Physics/CudaPBD.cu:474-509 — triangle bends replace the dihedral
        // ones (:159-178): every three consecutive vertices of a grid row,
        // then of a grid column; h0 = |v - centroid|.
        tp.tri_bend = true;
        tp.b1.clear(); tp.b2.clear(); tp.b3.clear(); tp.b4.clear();
        const int nx = d.params.dims[0], ny = d.params.dims[1];
        auto lin = [&](int i, int j) { return i * nx + j; };
        auto add = [&](int v1, int v3, int v2) {
            double c[3], h2 = 0;
            for (int k = 0; k < 3; ++k) c[k] = ((double)P[3 * v1 + k] + P[3 * v2 + k] + P[3 * v3 + k]) / 3.0;
            for (int k = 0; k < 3; ++k) h2 += ((double)P[3 * v3 + k] - c[k]) * ((double)P[3 * v3 + k] - c[k]);
            tp.b1.push_back(v1); tp.b2.push_back(v2); tp.b3.push_back(v3); tp.b4.push_back(-1);
            tp.th0.push_back((double)(float)std::sqrt(h2));
        };
        if ((long)nx * ny == tp.V) {
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j + 2 < ny; ++j) add(lin(i, j), lin(i, j + 1), lin(i, j + 2));
            for (int i = 0; i + 2 < nx; ++i)
                for (int j = 0; j < ny; ++j) add(lin(i, j), lin(i + 1, j), lin(i + 2, j));
        }
    }
    int E = (int)tp.s1.size(), B = (int)tp.b1.size();
    tp.kst.assign(E, d.params.kStretch);
    tp.kbd.assign(B, d.params.kBend);
    // Physics/CudaPBD.cu:146-233 — per-vertex slots, stretch first then bend.
    std::vector<int> cnt(tp.V, 0);
    for (int i = 0; i < E; ++i) { cnt[tp.s1[i]]++; cnt[tp.s2[i]]++; }
    for (int i = 0; i < B; ++i) {
        cnt[tp.b1[i]]++; cnt[tp.b2[i]]++; cnt[tp.b3[i]]++;
        if (!tp.tri_bend) cnt[tp.b4[i]]++;
    }
    tp.soff.assign(tp.V + 1, 0);
    for (int i = 0; i < tp.V; ++i) tp.soff[i + 1] = tp.soff[i] + cnt[i];
    tp.sent.assign(tp.soff[tp.V], 0);
    std::fill(cnt.begin(), cnt.end(), 0);
    auto put = [&](int v, int kind, int role, int c) {
        tp.sent[tp.soff[v] + cnt[v]++] = (kind << 30) | (role << 28) | c;
    };
    for (int i = 0; i < E; ++i) { put(tp.s1[i], ENT_STRETCH, 0, i); put(tp.s2[i], ENT_STRETCH, 1, i); }
    for (int i = 0; i < B; ++i) {
        put(tp.b1[i], ENT_BEND, 0, i); put(tp.b2[i], ENT_BEND, 1, i);
        put(tp.b3[i], ENT_BEND, 2, i);
        if (!tp.tri_bend) put(tp.b4[i], ENT_BEND, 3, i);
    }
    // Physics/CudaPBD.cu:48-81 — long-range attachments to every pinned vertex.
    tp.fixed.clear();
    for (int i = 0; i < tp.V; ++i)
        if (tp.pinned[i]) tp.fixed.push_back(i);
    int F = (int)tp.fixed.size();
    tp.lra_l0.assign((size_t)tp.V * F, 0.0);
    for (int i = 0; i < tp.V; ++i)
        for (int j = 0; j < F; ++j)
            if (!tp.pinned[i])
                tp.lra_l0[(size_t)i * F + j] = ddist(P, i, tp.fixed[j]) * (1.0 + (double)d.params.strainLimit);
    // Collision/FeatureList.cu:84-132 — feature ownership.  The reference
    // decides it by an atomicExch race; here the lowest original triangle
    // index wins, deterministically.
    tp.features.assign(tp.T, 0);
    std::vector<u8> vt(tp.V, 0);
    std::map<std::pair<int, int>, int> et;
    for (int t = 0; t < tp.T; ++t) {
        int v1 = tp.idx[3 * t], v2 = tp.idx[3 * t + 1], v3 = tp.idx[3 * t + 2];
        u8 f = 0;
        if (!vt[v1]) { vt[v1] = 1; f |= 1 << 5; }
        if (!vt[v2]) { vt[v2] = 1; f |= 1 << 4; }
        if (!vt[v3]) { vt[v3] = 1; f |= 1 << 3; }
        int e[3][2] = {{v1, v2}, {v2, v3}, {v3, v1}};
        for (int k = 0; k < 3; ++k) {
            std::pair<int, int> key(std::min(e[k][0], e[k][1]), std::max(e[k][0], e[k][1]));
            if (!et.count(key)) { et[key] = t; f |= 1 << (2 - k); }
        }
        tp.features[t] = f;
    }
}

// Thickness of Physics/CudaDeformableBody.cpp:86 (|x0 - x1| / 3).
inline float mesh_thickness(const lc_cloth_desc &d) {
    return (float)(ddist(d.positions, 0, 1) / 3.0);
}

struct Contact {
    int v[4];
    float w[4];
};

// Physics::PrimitiveContact (Physics/Structs.h:106-129): ids, weights, time
// of contact and unit normal, as the continuous and discrete tests leave them.
struct ContactFull {
    int v[4];
    float w[4];
    float t;
    float n[3];
};

// CudaDeformableBody::SolveCollisions (Physics/CudaDeformableBody.cpp:523-548):
// DeformableUtils::CreateImpulses then ApplyImpulses
// (Collision/CudaCollisionResponse.cu:11-300), in float as the reference.
// positions = x_prev (the reference passes m_dPrevPositions), velocities v;
// on return v holds the velocities after the impulses and x the new
// positions x_prev + v dt of every vertex that is not fixed (fixed vertices
// keep both).  Each contact writes four impulses (its vertices, weights
// times the impulse along its normal), the VF contacts first; they are
// grouped by vertex with a stable sort (CUB's radix sort, unique result) and
// summed per vertex in that order, then divided by the vertex's impulse
// count.  AccumulateImpulses is launched over the contact count's grid,
// ceil(contacts / 256) * 256 threads, one per run of equal vertex ids: the
// runs past that many (vertices ranked by id) are never accumulated and get
// no impulse (:132-136, the grid is not recomputed for the runs).
inline void solve_collisions(std::vector<V3<float>> &x, const std::vector<V3<float>> &xp, std::vector<V3<float>> &v,
                             const std::vector<u8> &fixed, const std::vector<ContactFull> &vf,
                             const std::vector<ContactFull> &ee, float stiffness, float mass, float dt, float h) {
    using V = V3<float>;
    const size_t Vn = v.size(), C = vf.size() + ee.size();
    std::vector<V> acc(Vn, mk<float>(0, 0, 0));
    if (C) {
        std::vector<std::pair<u32, V>> imp(4 * C);
        for (size_t id = 0; id < C; ++id) {
            const bool isvf = id < vf.size();
            const ContactFull &c = isvf ? vf[id] : ee[id - vf.size()];
            V vr;
            if (isvf) {  // :179-189
                V cv1 = v[c.v[0]] * c.w[0];
                V cv2 = v[c.v[1]] * c.w[1] + v[c.v[2]] * c.w[2] + v[c.v[3]] * c.w[3];
                vr = cv1 + cv2;
            } else {     // :191-201
                V cv1 = v[c.v[0]] * c.w[0] + v[c.v[1]] * c.w[1];
                V cv2 = v[c.v[2]] * c.w[2] + v[c.v[3]] * c.w[3];
                vr = cv1 + cv2;
            }
            // _CreateImpulse, :203-254
            const V n = mk<float>(c.n[0], c.n[1], c.n[2]);
            const V p = xp[c.v[0]] * c.w[0] + xp[c.v[1]] * c.w[1] + xp[c.v[2]] * c.w[2] + xp[c.v[3]] * c.w[3];
            const float d = h - dot(p, n);
            const float vn = dot(vr, n);
            const float dts = (0.1f * d) / dt;
            float i = 0.f;
            if (vn < dts) i = -std::fmin(dt * stiffness * d, mass * (dts - vn));
            if (vn < 0) i += mass * vn * 0.5f;
            i = std::fmin(std::fmax(-mass * 0.1f * h, i), mass * 0.1f * h);
            const float ip = (2 * i) / (c.w[0] * c.w[0] + c.w[1] * c.w[1] + c.w[2] * c.w[2] + c.w[3] * c.w[3]);
            const V ipv = n * ip;
            for (int k = 0; k < 4; ++k) imp[4 * id + k] = {(u32)c.v[k], ipv * c.w[k]};
        }
        std::stable_sort(imp.begin(), imp.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
        const size_t threads = (C + 255) / 256 * 256;
        size_t run = 0;
        for (size_t s = 0; s < imp.size(); ++run) {
            size_t e = s;
            V sum = mk<float>(0, 0, 0);
            while (e < imp.size() && imp[e].first == imp[s].first) sum = sum + imp[e++].second;
            if (run < threads) acc[imp[s].first] = sum / (float)(int)(e - s);
            s = e;
        }
    }
    // ApplyImpulses, :262-300
    for (size_t i = 0; i < Vn; ++i) {
        if (fixed[i]) continue;
        v[i] = v[i] + acc[i] / mass;
        x[i] = xp[i] + v[i] * dt;
    }
}

// ---------------------------------------------------------------------------
// The cloth: state + one FixedUpdate (Physics/CudaDeformableBody.cpp:550-627).
// ---------------------------------------------------------------------------
template <class R> class Cloth {
  public:
    using V = V3<R>;
    Topology tp;
    lc_cloth_params prm;
    float h = 0;  // thickness (float as the reference stores it)
    std::vector<V> x, xp, v, vn;
    std::vector<R> mass, invm;
    std::vector<u32> perm;  // slot -> original triangle
    V wind;                 // m_crtWindDir
    u64 rng = 0;

    // buffers of the last step (debug / parity)
    std::vector<V> pred_x, pred_xp, pred_v;
    std::vector<u32> perm_before;
    std::vector<u64> morton;  // sorted
    std::vector<int> lefts, rights, parents, rmll, rmlr;
    std::vector<V> nmin, nmax;  // node AABBs (2T-1)
    std::vector<u32> pairs;     // (i, j) flattened
    std::vector<Contact> vf, ee;
    std::vector<V> vf_n;          // unit face normal of each VF contact at its hit (friction)
    std::vector<u8> ground_flag;  // ground constraints of the last solve (friction)
    std::vector<V> pmin, pmax;  // particle swept AABBs
    u64 dropped = 0;
    int stack_overflow = 0;

    // Static triangle collider of the engine's lc_batch_set_collider (no
    // counterpart in the reference): its mesh and winding, and per vertex the
    // step's contacts (kCollSlots, ascending triangle; triangle -1 unused; a
    // contact's w holds its plane: unit normal towards the free side, n . a).
    static constexpr int kCollSlots = 8;
    static constexpr float kCollMargin = 4.0f;  // detection reach beyond the contact layer, in thicknesses
    std::vector<V> coll_v;
    std::vector<int> coll_t;
    bool coll_cw = false;  // faces clockwise seen from the free side
    std::vector<int> coll_tri;
    std::vector<Contact> coll_c;
    bool coll_overflow = false;
    bool have_frozen_coll = false;
    std::vector<int> frozen_coll_tri;
    std::vector<Contact> frozen_coll_c;

    bool have_frozen = false;
    std::vector<Contact> frozen_vf, frozen_ee;
    std::vector<V> frozen_vf_n;  // their face normals, for friction (empty: no friction on frozen contacts)

    // Discrete decisions replayed from another implementation for one step
    // (ground / LRA / sphere activation, per-iteration counted terms), so that
    // a comparison measures only the continuous arithmetic.
    struct Forced {
        bool on = false;
        std::vector<u8> ground;     // V
        std::vector<u32> ground_it; // V, bit per iteration
        std::vector<u8> lra;        // V*F
        std::vector<u8> dyn;        // iterations x (4 * contacts)
        std::vector<int8_t> sphere; // V
    } forced;

    // What one step decided and the intermediate states its adjoint needs
    // (filled while `recording`; see backward()).
    struct Record {
        std::vector<Contact> vf, ee;
        std::vector<u8> ground;      // V
        std::vector<u32> ground_it;  // V
        std::vector<u8> lra;         // V*F
        std::vector<u8> dyn;         // iterations x 4*(vf+ee)
        std::vector<int8_t> sphere;  // V: ray-sphere outcome -1 / 0 / 1
        std::vector<V> x_in, v_b;    // damping inputs: state x, velocity after the global damping
        std::vector<std::vector<V>> xk;  // solver iterates x^0 .. x^K
        std::vector<int> coll_tri;       // static-collider contacts of the step (V x kCollSlots) ...
        std::vector<Contact> coll_c;     // ... and their planes
        std::vector<u8> coll_act;        // (iterations + 1) x V: slots projected, [0] before the solver
        double M = 0, xcm[3] = {0, 0, 0}, vcm[3] = {0, 0, 0}, om[3] = {0, 0, 0}, I[3][3] = {};
    };
    bool recording = false;
    Record rec;
    // Smallest 1 - n1.n2 (bend_min) and 1 + n1.n2 (bend_min_neg) over the
    // bends and the solver iterates of the last solve (when track_bend): how
    // close a bend came to a singularity of the reference's formula.  At
    // d -> 1 the correction itself is 0 * inf and rounding alone moves it by
    // a finite amount; at d -> -1 (phi -> phi0 = pi) the correction is a
    // 0 / 0 ratio that goes to zero with a bounded rounding error, but whose
    // derivative grows like (1 + d)^-1/2, so only the reverse pass is
    // ill-conditioned there.  The formula takes raw positions, so every bend
    // of a cloth lying in a plane through the origin (on the ground plane
    // y = 0) sits at d = -1.
    bool track_bend = false;
    double bend_min = 1e300, bend_min_neg = 1e300;
    // Smallest |n| / h over the contacts of the last solve's iterates (when
    // track_bend), n the contact vector of Physics/CudaPBD.cu:1212-1415: the
    // correction's Jacobian I - (h / |n|)(I - n n^T / |n|^2) grows without
    // bound as a vertex comes to lie on its face or two edges cross.
    double contact_min = 1e300;
    std::vector<Record> records;  // one per recorded step of a rollout

    void init(const lc_cloth_desc &d) {
        prm = d.params;
        build_topology(d, tp);
        h = prm.thicknessFromMesh ? mesh_thickness(d) : prm.thickness;
        int Vn = tp.V;
        x.resize(Vn); xp.resize(Vn); v.assign(Vn, mk<R>(0, 0, 0)); vn.assign(Vn, mk<R>(0, 0, 0));
        mass.resize(Vn); invm.resize(Vn);
        for (int i = 0; i < Vn; ++i) {
            x[i] = mk<R>(d.positions[3 * i], d.positions[3 * i + 1], d.positions[3 * i + 2]);
            xp[i] = x[i];
            // Physics/CudaDeformableBody.cpp:80-82
            float vm = prm.objectMass / (float)Vn;
            mass[i] = tp.pinned[i] ? R(1000) : R(vm);
            invm[i] = tp.pinned[i] ? R(0) : R(1.f / vm);
        }
        perm.resize(tp.T);
        std::iota(perm.begin(), perm.end(), 0u);
        // Physics/CudaPBD.cu:42 — current wind.
        wind = prm.windOn ? mk<R>(prm.startWindDir[0], prm.startWindDir[1], prm.startWindDir[2]) : mk<R>(0, 0, 0);
        rng = prm.windSeed ? prm.windSeed : 0x9E3779B97F4A7C15ull;
        // Physics/CudaDeformableBody.cpp:214,269 with Physics/CudaDeformableUtils.cu:37-64
        // and :190-249: initial vertex normals from the unnormalised face normals.
        for (int t = 0; t < tp.T; ++t) {
            V a = x[tp.idx[3 * t]], b = x[tp.idx[3 * t + 1]], c = x[tp.idx[3 * t + 2]];
            V fn = cross(b - a, c - a);
            for (int k = 0; k < 3; ++k) vn[tp.idx[3 * t + k]] = vn[tp.idx[3 * t + k]] + fn;
        }
        for (int i = 0; i < Vn; ++i) vn[i] = normalize(vn[i]);
    }

    R kp_of(double k) const {
        return R(1.0 - std::pow(1.0 - k, 1.0 / (double)prm.solverIterations));
    }

    // Host wind update of Physics/CudaPBD.cu:613-619; the std::rand() draw is
    // replaced by a seeded xorshift so that runs are reproducible.
    double next_uniform() {
        rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
        return (double)(rng >> 11) * (1.0 / 9007199254740992.0);
    }
    void update_wind() {
        if (!prm.windOn) return;
        u64 bit = (rng ^ (rng >> 29)) & 1;
        double u = next_uniform();
        double var = (double)prm.windMinVariation + u * ((double)prm.windMaxVariation - prm.windMinVariation);
        float variation = (bit ? 1.f : -1.f) * (float)var;
        V sw = mk<R>(prm.startWindDir[0], prm.startWindDir[1], prm.startWindDir[2]);
        wind = wind + sw * R(variation);
        wind = mk(clampf(wind.x, R(prm.minWindDir[0]), R(prm.maxWindDir[0])),
                  clampf(wind.y, R(prm.minWindDir[1]), R(prm.maxWindDir[1])),
                  clampf(wind.z, R(prm.minWindDir[2]), R(prm.maxWindDir[2])));
    }

    // ---- 1. PBDStepExternal (Physics/CudaPBD.cu:610-630) -------------------
    void external() {
        int Vn = tp.V;
        update_wind();
        R dt = R(prm.timestep);
        V g = mk<R>(prm.gravity[0], prm.gravity[1], prm.gravity[2]);
        // ApplyExternalForces, Physics/CudaPBD.cu:1992-2003
        for (int i = 0; i < Vn; ++i) {
            if (is_zero(wind))
                v[i] = v[i] + dt * g;
            else
                v[i] = v[i] + dt * (g + vn[i] * dot(normalize(wind), vn[i]) * len(wind));
        }
        // DampVelocities, Physics/CudaPBD.cu:411-458 with kernels :1934-1990.
        R kg = R(prm.globalVelDamp);
        for (int i = 0; i < Vn; ++i) v[i] = v[i] * (R(1) - kg);
        if (recording) { rec.x_in = x; rec.v_b = v; }
        // Reductions in double (the reference reduces float3s with CUB).
        double msum = 0, xm[3] = {0, 0, 0}, vm[3] = {0, 0, 0};
        for (int i = 0; i < Vn; ++i) {
            double m = mass[i];
            msum += m;
            xm[0] += (double)(x[i].x * mass[i]); xm[1] += (double)(x[i].y * mass[i]); xm[2] += (double)(x[i].z * mass[i]);
            vm[0] += (double)(v[i].x * mass[i]); vm[1] += (double)(v[i].y * mass[i]); vm[2] += (double)(v[i].z * mass[i]);
        }
        V xcm = mk<R>(R(xm[0] / msum), R(xm[1] / msum), R(xm[2] / msum));
        V vcm = mk<R>(R(vm[0] / msum), R(vm[1] / msum), R(vm[2] / msum));
        double L[3] = {0, 0, 0}, i1[3] = {0, 0, 0}, i2[3] = {0, 0, 0};
        for (int i = 0; i < Vn; ++i) {
            V ri = x[i] - xcm;
            V l = cross(ri, v[i] * mass[i]);
            L[0] += (double)l.x; L[1] += (double)l.y; L[2] += (double)l.z;
            V a1 = mk(ri.x * ri.x, ri.y * ri.y, ri.z * ri.z) * mass[i];
            V a2 = -mk(ri.x * ri.y, ri.x * ri.z, ri.y * ri.z) * mass[i];
            i1[0] += (double)a1.x; i1[1] += (double)a1.y; i1[2] += (double)a1.z;
            i2[0] += (double)a2.x; i2[1] += (double)a2.y; i2[2] += (double)a2.z;
        }
        double I[3][3] = {{i1[1] + i1[2], i2[0], i2[1]}, {i2[0], i1[0] + i1[2], i2[2]}, {i2[1], i2[2], i1[0] + i1[1]}};
        double om[3];
        solve3(I, L, om);
        if (recording) {
            rec.M = msum;
            for (int k = 0; k < 3; ++k) {
                rec.xcm[k] = xm[k] / msum; rec.vcm[k] = vm[k] / msum; rec.om[k] = om[k];
                for (int l = 0; l < 3; ++l) rec.I[k][l] = I[k][l];
            }
        }
        V omega = mk<R>(R(om[0]), R(om[1]), R(om[2]));
        R kd = R(prm.kDamp);
        for (int i = 0; i < Vn; ++i) {
            V ri = x[i] - xcm;
            V dv = vcm + cross(omega, ri) - v[i];
            v[i] = v[i] + kd * dv;
        }
        // ExplicitEuler, Physics/CudaPBD.cu:2005-2012
        for (int i = 0; i < Vn; ++i) x[i] = xp[i] + dt * v[i];
    }

    static void solve3(const double I[3][3], const double L[3], double out[3]) {
        double a = I[0][0], b = I[0][1], c = I[0][2], d = I[1][0], e = I[1][1], f = I[1][2], g = I[2][0],
               hh = I[2][1], k = I[2][2];
        double A = e * k - f * hh, Bc = -(d * k - f * g), C = d * hh - e * g;
        double det = a * A + b * Bc + c * C;
        double inv[3][3] = {{A / det, -(b * k - c * hh) / det, (b * f - c * e) / det},
                            {Bc / det, (a * k - c * g) / det, -(a * f - c * d) / det},
                            {C / det, -(a * hh - b * g) / det, (a * e - b * d) / det}};
        for (int r = 0; r < 3; ++r) out[r] = inv[r][0] * L[0] + inv[r][1] * L[1] + inv[r][2] * L[2];
    }

    // ---- 2-5. collision pipeline -------------------------------------------
    // Runs on the current x, xp, v and perm; fills morton/perm/tree/pairs/
    // contacts.  In FP32-mirror mode it is bit-exact with the GPU.
    void collide() {
        int Vn = tp.V, T = tp.T;
        R hh = R(h);
        // Collision/FeatureList.cu:134-148 — particle swept AABBs.
        pmin.resize(Vn); pmax.resize(Vn);
        for (int i = 0; i < Vn; ++i) {
            pmin[i] = subc(vmin(x[i], xp[i]), hh);
            pmax[i] = addc(vmax(x[i], xp[i]), hh);
        }
        // Physics/CudaDeformableUtils.cu:120-151 — per slot (pre-sort order).
        int nodes = 2 * T - 1;
        nmin.assign(std::max(nodes, 1), mk<R>(0, 0, 0));
        nmax.assign(std::max(nodes, 1), mk<R>(0, 0, 0));
        std::vector<u64> keys(T);
        std::vector<V> fn(T);
        perm_before = perm;
        for (int s = 0; s < T; ++s) {
            u32 t = perm[s];
            int a = tp.idx[3 * t], b = tp.idx[3 * t + 1], c = tp.idx[3 * t + 2];
            fn[s] = normalize(cross(x[b] - x[a], x[c] - x[a]));
            V mn = subc(min3(x[a], x[b], x[c]), hh);
            V mx = addc(max3(x[a], x[b], x[c]), hh);
            V pmn = subc(min3(xp[a], xp[b], xp[c]), hh);
            V pmx = addc(max3(xp[a], xp[b], xp[c]), hh);
            V smn = vmin(mn, pmn), smx = vmax(mx, pmx);
            nmin[T - 1 + s] = smn;
            nmax[T - 1 + s] = smx;
            V mid = smn + (smx - smn) / R(2);
            float o0 = prm.mortonOrigin[0], o1 = prm.mortonOrigin[1], o2 = prm.mortonOrigin[2], sc = prm.mortonScale;
            float qx = ((float)mid.x - o0) * sc, qy = ((float)mid.y - o1) * sc, qz = ((float)mid.z - o2) * sc;
            keys[s] = morton3d(qx, qy, qz, prm.mortonMode);
        }
        // Physics/CudaDeformableUtils.cu:190-249 — running vertex normals
        // (only read by the wind term).
        for (int s = 0; s < T; ++s) {
            u32 t = perm[s];
            for (int k = 0; k < 3; ++k) vn[tp.idx[3 * t + k]] = vn[tp.idx[3 * t + k]] + fn[s];
        }
        for (int i = 0; i < Vn; ++i) vn[i] = normalize(vn[i]);
        // Physics/CudaDeformableUtils.cu:346-349 — stable sort of the keys with
        // the triangle payload; the AABBs stay where they are (quirk) unless
        // refLeafAabbQuirk is 0.
        std::vector<u32> order(T);
        std::iota(order.begin(), order.end(), 0u);
        std::stable_sort(order.begin(), order.end(), [&](u32 a, u32 b) { return keys[a] < keys[b]; });
        morton.resize(T);
        std::vector<u32> np(T);
        for (int s = 0; s < T; ++s) { morton[s] = keys[order[s]]; np[s] = perm[order[s]]; }
        if (!prm.refLeafAabbQuirk) {
            std::vector<V> lm(T), lx(T);
            for (int s = 0; s < T; ++s) { lm[s] = nmin[T - 1 + order[s]]; lx[s] = nmax[T - 1 + order[s]]; }
            for (int s = 0; s < T; ++s) { nmin[T - 1 + s] = lm[s]; nmax[T - 1 + s] = lx[s]; }
        }
        perm = np;
        build_tree();
        refit();
        traverse();
        narrowphase();
        collider_contacts();
    }

    // The static collider's contacts of every vertex (the engine's
    // k_collider_query; no counterpart in the reference).  For a face with
    // unit normal n towards the free side and d0 = n . a, the signed heights
    // s0 = n . x_prev - d0, s1 = n . x - d0 (x the prediction) make it a
    // contact when s1 < h + m and s0 > -m (m = kCollMargin h) and the point
    // where the vertex crosses the plane (without a crossing, the
    // prediction) has barycentric coordinates >= -h / perimeter (TestVF's
    // tolerance, Collision/CudaPrimitiveTests.cu:348-406).  The reach lets
    // the constraint act on a vertex the solver iterations drag towards the
    // face after detection, and brings back one that ended a step behind it;
    // the constraint is one-sided, so a contact above its layer is inactive.
    // Only faces whose boxes meet the vertex's swept box inflated by h + m
    // are tested (the engine's BVH culls the same way).  The hits in
    // ascending triangle order, at most kCollSlots (more sets coll_overflow).
    static bool collider_hit(V xp, V x, V a, V b, V c, V n, R d0, R h, R m) {
        const R s0 = dot(n, xp) - d0, s1 = dot(n, x) - d0;
        if (!(s1 < h + m) || !(s0 > -m)) return false;
        const V q = (s0 > R(0) && s1 < R(0)) ? xp + (x - xp) * (s0 / (s0 - s1)) : x;
        const V e1 = b - a, e2 = c - a, e3 = c - b, r = q - a;
        const R d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2), d20 = dot(r, e1), d21 = dot(r, e2);
        const R den = d00 * d11 - d01 * d01;
        if (!(den > R(0))) return false;
        const R wb = (d11 * d20 - d01 * d21) / den, wc = (d00 * d21 - d01 * d20) / den;
        const R wa = R(1) - wb - wc;
        const R del = h / (len(e1) + len(e2) + len(e3));
        return wa >= -del && wb >= -del && wc >= -del;
    }
    void collider_contacts() {
        const int Vn = tp.V, K = kCollSlots, T = (int)(coll_t.size() / 3);
        coll_tri.assign((size_t)Vn * K, -1);
        coll_c.assign((size_t)Vn * K, Contact{});
        coll_overflow = false;
        if (!T) return;
        const R hh = R(h), mm = R(kCollMargin) * hh, hm = hh + mm;
        for (int i = 0; i < Vn; ++i) {
            const V lo = subc(vmin(x[i], xp[i]), hm), hi = addc(vmax(x[i], xp[i]), hm);
            int n = 0;
            for (int t = 0; t < T; ++t) {
                const V a = coll_v[coll_t[3 * t]], b = coll_v[coll_t[3 * t + 1]], c = coll_v[coll_t[3 * t + 2]];
                if (!overlap(lo, hi, min3(a, b, c), max3(a, b, c))) continue;
                V nf = normalize(cross(b - a, c - a));
                if (coll_cw) nf = nf * R(-1);
                const R d0 = dot(nf, a);
                if (!collider_hit(xp[i], x[i], a, b, c, nf, d0, hh, mm)) continue;
                if (n == K) { coll_overflow = true; break; }
                Contact k;
                k.v[0] = i; k.v[1] = k.v[2] = k.v[3] = 0;
                k.w[0] = float(nf.x); k.w[1] = float(nf.y); k.w[2] = float(nf.z); k.w[3] = float(d0);
                coll_tri[(size_t)i * K + n] = t;
                coll_c[(size_t)i * K + n] = k;
                ++n;
            }
        }
    }

    // A vertex projected onto its collider contacts' one-sided constraints
    // n . x >= d0 + h, in slot order (this step's contacts, or the frozen
    // ones); pinned vertices do not move.  Done before the solver (as the
    // reference projects onto its analytic sphere before the iterations,
    // Physics/CudaPBD.cu:1509-1569) and at the end of every iteration, after
    // the Jacobi average: collisions are projected last, so the averaged
    // stretch and bend corrections cannot pull a vertex that crossed a face
    // back through it.
    // pass (recording): 0 before the solver, it + 1 at the end of iteration
    // it; the slots projected go to rec.coll_act for the reverse pass.
    void coll_project_vertex(int i, int pass) {
        if (invm[i] == R(0)) return;
        const int K = kCollSlots;
        const std::vector<int> &ctri = have_frozen_coll ? frozen_coll_tri : coll_tri;
        const std::vector<Contact> &cc = have_frozen_coll ? frozen_coll_c : coll_c;
        if (ctri.size() < (size_t)(i + 1) * K) return;
        const R th = R(h);
        u8 m = 0;
        for (int k = 0; k < K && ctri[(size_t)i * K + k] >= 0; ++k) {
            const Contact &q = cc[(size_t)i * K + k];
            const V n = mk<R>(R(q.w[0]), R(q.w[1]), R(q.w[2]));
            const R c = dot(n, x[i]) - R(q.w[3]) - th;
            if (c < R(0)) {
                x[i] = x[i] + n * (-c);
                m |= (u8)(1u << k);
            }
        }
        if (recording && !rec.coll_act.empty()) rec.coll_act[(size_t)pass * tp.V + i] = m;
    }
    void coll_project() {
        if (recording) { rec.coll_tri.clear(); rec.coll_c.clear(); rec.coll_act.clear(); }
        if (coll_t.empty()) return;
        if (recording) {
            rec.coll_tri = have_frozen_coll ? frozen_coll_tri : coll_tri;
            rec.coll_c = have_frozen_coll ? frozen_coll_c : coll_c;
            rec.coll_act.assign((size_t)(prm.solverIterations + 1) * tp.V, 0);
        }
        for (int i = 0; i < tp.V; ++i) coll_project_vertex(i, 0);
    }
    // The projections of one pass reversed: each projected slot's Jacobian
    // I - n n^T is symmetric, and the slots apply last first.
    void coll_project_reverse(const Record &r, int pass, std::vector<V> &a) const {
        if (r.coll_act.empty()) return;
        const int K = kCollSlots;
        for (int i = 0; i < tp.V; ++i) {
            const u8 m = r.coll_act[(size_t)pass * tp.V + i];
            for (int k = K - 1; k >= 0; --k)
                if ((m >> k) & 1u) {
                    const Contact &q = r.coll_c[(size_t)i * K + k];
                    const V n = mk<R>(R(q.w[0]), R(q.w[1]), R(q.w[2]));
                    a[i] = a[i] - n * dot(n, a[i]);
                }
        }
    }

    // Collision/CudaBVH.cu:163-188.  Two internal nodes may claim the same
    // child when a run of >= 3 equal codes meets FindSplit's midpoint rule;
    // the reference's parents[] write race is resolved here as "largest
    // parent index wins" (the GPU uses atomicMax).
    void build_tree() {
        int T = tp.T, In = T - 1;
        lefts.assign(std::max(In, 0), 0);
        rights.assign(std::max(In, 0), 0);
        parents.assign(std::max(2 * T - 1, 1), -1);
        for (int id = 0; id < In; ++id) {
            int first, last;
            find_range(morton.data(), In, id, first, last);
            int split = find_split(morton.data(), first, last);
            int l = split == first ? In + split : split;
            int r = split + 1 == last ? In + split + 1 : split + 1;
            lefts[id] = l;
            rights[id] = r;
            parents[l] = std::max(parents[l], id);
            parents[r] = std::max(parents[r], id);
        }
    }

    // Collision/CudaBVH.cu:128-149 — bottom-up union; the second arrival at a
    // node proceeds.  rmll/rmlr: rightmost leaf node below each child.  The
    // reference writes a node's box and rightmost leaf without a fence before
    // the atomicExch that lets its parent proceed; run on a GB300 its refit
    // reads stale children at a few nodes per build (boxes with zero
    // components, rightmost leaf 0).  The restatement computes the race-free
    // result, which is what the reference's formulas give whenever the reads
    // see the finished children.
    void refit() {
        int T = tp.T, In = T - 1;
        rmll.assign(std::max(In, 0), 0);
        rmlr.assign(std::max(In, 0), 0);
        if (In <= 0) return;
        std::vector<int> visited(In, 0);
        for (int id = 0; id < T; ++id) {
            int pid = parents[In + id];
            for (int guard = 0; guard <= T && pid >= 0 && pid < In; ++guard) {
                if (visited[pid]++ == 0) break;
                int l = lefts[pid], r = rights[pid];
                nmin[pid] = vmin(nmin[l], nmin[r]);
                nmax[pid] = vmax(nmax[l], nmax[r]);
                rmll[pid] = l >= In ? l : std::max(rmll[l], rmlr[l]);
                rmlr[pid] = r >= In ? r : std::max(rmll[r], rmlr[r]);
                if (pid == 0) break;
                pid = parents[pid];
            }
        }
    }

    // Collision/CudaBVH.cu:23-113 — per-leaf DFS, pairs (i, j>i), at most
    // chunk per leaf, overflow dropped; then the order-preserving compaction
    // of Collision/CudaCollisionDetection.cu:17.
    void traverse() {
        int T = tp.T, In = T - 1;
        pairs.clear();
        dropped = 0;
        stack_overflow = 0;
        if (In <= 0) return;
        int chunk = std::min(prm.BVHChunkSize, T);
        for (int id = 0; id < T; ++id) {
            int me = In + id;
            int stack[64];
            stack[0] = -1;
            int top = 1, node = 0, got = 0;
            V amin = nmin[me], amax = nmax[me];
            do {
                int l = lefts[node], r = rights[node];
                bool ol = false, orr = false;
                if (rmll[node] > me && overlap(amin, amax, nmin[l], nmax[l])) ol = true;
                if (rmlr[node] > me && overlap(amin, amax, nmin[r], nmax[r])) orr = true;
                if (ol && l >= In) {
                    if (got < chunk) { pairs.push_back(id); pairs.push_back(l - In); ++got; }
                    else ++dropped;
                }
                if (orr && r >= In) {
                    if (got < chunk) { pairs.push_back(id); pairs.push_back(r - In); ++got; }
                    else ++dropped;
                }
                bool tl = ol && l < In, tr = orr && r < In;
                if (!tl && !tr) {
                    node = stack[--top];
                } else {
                    node = tl ? l : r;
                    if (tl && tr) {
                        if (top >= 64) { stack_overflow = 1; break; }
                        stack[top++] = r;
                    }
                }
            } while (top != 0);
        }
    }

    // ---- narrowphase --------------------------------------------------------
    // Physics/CudaCubicSolver.cu:126-129
    static R triple(V x21, V x31, V x41, V v21, V v31, V v41, R t) {
        return dot(cross(x21 + t * v21, x31 + t * v31), x41 + t * v41);
    }
    // Physics/CudaCubicSolver.cu:131-153
    static R secant(V x21, V x31, V x41, V v21, V v31, V v41, R a, R b, int maxit) {
        R x0 = a, x1 = b;
        for (int i = 0; i < maxit; ++i) {
            R f0 = triple(x21, x31, x41, v21, v31, v41, x0);
            R f1 = triple(x21, x31, x41, v21, v31, v41, x1);
            R xc = (x0 * f1 - x1 * f0) / (f1 - f0);
            if (std::fabs(xc - x1) < R(kEpsCubic)) return xc;
            x0 = x1;
            x1 = xc;
        }
        return R(-15);
    }
    // Physics/CudaCubicSolver.cu:69-124.  When only the second root lies in
    // [0,1], FindCoplanarityTimes reads critPoint1, which FindCriticalPoints
    // left unset (Physics/CudaCubicSolver.cu:19-33).  The reference's kernels,
    // built and run (tests/golden), behave as if that read returned the first
    // root t1 although it lies outside [0,1]: the interval [0, t1] is then
    // searched, which is how the reference reports contacts at small
    // negative times.  The restatement does the same.
    static int critical_points(V x21, V x31, V x41, V v21, V v31, V v41, R out[2]) {
        V v21v31 = cross(v21, v31), x21v31 = cross(x21, v31), v21x31 = cross(v21, x31), x21x31 = cross(x21, x31);
        R v1v2v3 = dot(v21v31, v41), x1v2v3 = dot(x21v31, v41), v1x2v3 = dot(v21x31, v41),
          v1v2x3 = dot(v21v31, x41), x1x2v3 = dot(x21x31, v41), x1v2x3 = dot(x21v31, x41),
          v1x2x3 = dot(v21x31, x41);
        R a = v1v2v3, b = x1v2v3 + v1x2v3 + v1v2x3, c = x1x2v3 + x1v2x3 + v1x2x3;
        R ad = R(3) * a, bd = R(2) * b;
        R disc = R(4) * (b * b - ad * c);
        R sq = std::sqrt(disc);
        R da = R(2) * ad;
        R t1 = (-bd + sq) / da, t2 = (-bd - sq) / da;
        int n = 0;
        if (disc >= R(kEpsCubic)) {
            const bool in1 = between(t1, R(0), R(1)), in2 = between(t2, R(0), R(1));
            if (in1 || in2) out[n++] = t1;
            if (in1 && in2) out[n++] = t2;
        } else if (std::fabs(disc) < R(kEpsCubic)) {
            if (between(t1, R(0), R(1))) out[n++] = t1;
        }
        return n;
    }
    // Physics/CudaCubicSolver.cu:5-67
    static int coplanarity_times(V x1, V x2, V x3, V x4, V v1, V v2, V v3, V v4, R times[8]) {
        V x21 = x2 - x1, x31 = x3 - x1, x41 = x4 - x1, v21 = v2 - v1, v31 = v3 - v1, v41 = v4 - v1;
        R cp[2];
        int ncp = critical_points(x21, x31, x41, v21, v31, v41, cp);
        R ends[4];
        int ne = 0;
        ends[ne++] = R(0);
        for (int i = 0; i < ncp; ++i) ends[ne++] = cp[i];
        ends[ne++] = R(1);
        int n = 0;
        for (int i = 0; i < ne - 1; ++i) {
            R a = ends[i], b = ends[i + 1];
            R fa = triple(x21, x31, x41, v21, v31, v41, a);
            R fb = triple(x21, x31, x41, v21, v31, v41, b);
            if (std::fabs(fa) < R(kEpsCubic)) times[n++] = a;
            if (fa * fb < R(0)) {
                R t = secant(x21, x31, x41, v21, v31, v41, a, b, 20);
                if (t != R(-15)) times[n++] = t;
            }
        }
        return n;
    }
    // Core/CudaUtils.cu:149-168
    static V project_on_line(V p, V e1, V e2) {
        V ab = e2 - e1, ap = p - e1;
        return e1 + dot(ap, ab) / dot(ab, ab) * ab;
    }
    static V clamp_on_line(V p, V e1, V e2) {
        R d1 = dist(p, e1), d2 = dist(p, e2);
        if (std::fabs(d1 + d2 - dist(e1, e2)) < R(kEpsPbd)) return p;
        return d1 < d2 ? e1 : e2;
    }
    // Collision/CudaPrimitiveTests.cu:348-406
    static bool test_vf(V x4, V x1, V x2, V x3, Contact &c, R th, V *nout = nullptr) {
        V x13 = x1 - x3, x23 = x2 - x3, x43 = x4 - x3;
        V crs = cross(x2 - x1, x3 - x1);
        V n = normalize(crs);
        if (nout) *nout = n;
        if (std::fabs(dot(x43, n)) <= th) {
            R dt = dot(x13, x23);
            R m11 = dot(x13, x13), m12 = dt, m21 = dt, m22 = dot(x23, x23);
            R vr1 = dot(x13, x43), vr2 = dot(x23, x43);
            R w2 = (m11 * vr2 - m21 * vr1) / (m11 * m22 - m21 * m12);
            R w1 = (vr1 - m12 * w2) / m11;
            R w3 = R(1) - w1 - w2;
            R del = th / (len(x13) + len(x23) + len(x1 - x2));
            R lo = R(0), hi = R(1) + del;
            if (between(w1, lo, hi) && between(w2, lo, hi) && between(w3, lo, hi)) {
                c.w[0] = 1.f; c.w[1] = (float)-w1; c.w[2] = (float)-w2; c.w[3] = (float)-w3;
                return true;
            }
        }
        return false;
    }
    // Collision/CudaPrimitiveTests.cu:408-425
    // nout, tout (optional): the contact's normal and, where the reference's
    // test writes it, its time (Physics::PrimitiveContact n and t).
    static bool test_edge_degenerate(V x1, V x3, V x21, V x43, Contact &c, R th, V *nout = nullptr) {
        V m1 = x1 + x21 / R(2), m2 = x3 + x43 / R(2);
        if (dist(m1, m2) <= th) {
            c.w[0] = c.w[1] = c.w[2] = c.w[3] = 0.5f;
            if (nout) *nout = normalize(m1 - m2);
            return true;
        }
        return false;
    }
    // Collision/CudaPrimitiveTests.cu:252-346 (the in-range branch measures
    // cp2 with a, not b, as the reference does).
    static bool test_ee(V x1, V x2, V x3, V x4, Contact &c, R th, V *nout = nullptr, R *tout = nullptr) {
        V x21 = x2 - x1, x31 = x3 - x1, x43 = x4 - x3;
        V crs = cross(x21, x43);
        if (len(crs) < R(kEpsEE)) return test_edge_degenerate(x1, x3, x21, x43, c, th, nout);
        if (is_zero(crs)) return false;
        R dt = dot(-x21, x43);
        R m11 = dot(x21, x21), m12 = dt, m21 = dt, m22 = dot(x43, x43);
        R vr1 = dot(x21, x31), vr2 = dot(-x43, x31);
        R b = (m11 * vr2 - m21 * vr1) / (m11 * m22 - m21 * m12);
        R a = (vr1 - m12 * b) / m11;
        if (between(a, R(0), R(1)) && between(b, R(0), R(1))) {
            V cp1 = x1 + a * x21, cp2 = x3 + a * x43;
            if (dist(cp1, cp2) <= th) {
                c.w[0] = (float)(R(1) - a); c.w[1] = (float)a; c.w[2] = (float)(-(R(1) - b)); c.w[3] = (float)(-b);
                if (nout) {
                    V dir = (x1 + a * x21) - (x3 + b * x43);  // with b here (:305)
                    *nout = normalize(is_zero(dir) ? crs : dir);
                }
                return true;
            }
        } else {
            R ac = clampf(a, R(0), R(1)), bc = clampf(b, R(0), R(1));
            R d1 = std::fabs(a - ac) * len(x21), d2 = std::fabs(b - bc) * len(x43);
            a = ac; b = bc;
            V cp1, cp2;
            if (d1 > d2) {
                cp1 = x1 + a * x21;
                cp2 = clamp_on_line(project_on_line(cp1, x3, x4), x3, x4);
            } else {
                cp2 = x3 + b * x43;
                cp1 = clamp_on_line(project_on_line(cp2, x1, x2), x1, x2);
            }
            if (dist(cp1, cp2) <= th) {
                c.w[0] = (float)(R(1) - a); c.w[1] = (float)a; c.w[2] = (float)(-(R(1) - b)); c.w[3] = (float)(-b);
                if (nout) *nout = normalize(cp1 - cp2);
                if (tout) *tout = R(0);
                return true;
            }
        }
        return false;
    }

    // Collision/CudaCollisionDetection.cu:53-189 (candidate slots),
    // Collision/CudaPrimitiveTests.cu:427-490 (feature AABB cull),
    // :109-238 (CCD on x_prev and v), compactions at
    // Collision/CudaCollisionDetection.cu:264-282.
    void narrowphase() {
        vf.clear();
        ee.clear();
        vf_n.clear();
        R th = R(h), dt = R(prm.timestep);
        size_t P = pairs.size() / 2;
        for (size_t p = 0; p < P; ++p) {
            u32 ta = perm[pairs[2 * p]], tb = perm[pairs[2 * p + 1]];
            int A[3] = {(int)tp.idx[3 * ta], (int)tp.idx[3 * ta + 1], (int)tp.idx[3 * ta + 2]};
            int B[3] = {(int)tp.idx[3 * tb], (int)tp.idx[3 * tb + 1], (int)tp.idx[3 * tb + 2]};
            u8 fa = tp.features[ta], fb = tp.features[tb];
            for (int s = 0; s < 6; ++s) {
                const int *P1 = s < 3 ? A : B, *F1 = s < 3 ? B : A;
                u8 f = s < 3 ? fa : fb;
                if (!((f >> (5 - s % 3)) & 1)) continue;
                Contact c;
                c.v[0] = P1[s % 3]; c.v[1] = F1[0]; c.v[2] = F1[1]; c.v[3] = F1[2];
                c.w[0] = c.w[1] = c.w[2] = c.w[3] = -1.f;
                V nrm = mk<R>(0, 0, 0);
                if (vf_candidate(c, th, dt, &nrm)) { vf.push_back(c); vf_n.push_back(nrm); }
            }
            // EE slot k: edge ea of A x edge eb of B.
            static const int ea_v[3][2] = {{0, 1}, {0, 2}, {1, 2}};
            static const int ea_bit[3] = {2, 0, 1};
            for (int s = 0; s < 9; ++s) {
                int ia = s % 3, ib = s / 3;
                if (!(((fa >> ea_bit[ia]) & 1) & ((fb >> ea_bit[ib]) & 1))) continue;
                Contact c;
                c.v[0] = A[ea_v[ia][0]]; c.v[1] = A[ea_v[ia][1]];
                c.v[2] = B[ea_v[ib][0]]; c.v[3] = B[ea_v[ib][1]];
                c.w[0] = c.w[1] = c.w[2] = c.w[3] = -1.f;
                if (ee_candidate(c, th, dt)) ee.push_back(c);
            }
        }
    }

    bool vf_candidate(Contact &c, R th, R dt, V *nout = nullptr) {
        V tmin = min3(pmin[c.v[1]], pmin[c.v[2]], pmin[c.v[3]]);
        V tmax = max3(pmax[c.v[1]], pmax[c.v[2]], pmax[c.v[3]]);
        if (!overlap(pmin[c.v[0]], pmax[c.v[0]], tmin, tmax)) return false;
        if (c.v[0] == c.v[1] || c.v[0] == c.v[2] || c.v[0] == c.v[3]) return false;
        V x4 = xp[c.v[0]], x1 = xp[c.v[1]], x2 = xp[c.v[2]], x3 = xp[c.v[3]];
        V v4 = v[c.v[0]], v1 = v[c.v[1]], v2 = v[c.v[2]], v3 = v[c.v[3]];
        R times[8];
        int n = coplanarity_times(x1, x2, x3, x4, v1, v2, v3, v4, times);
        for (int i = 0; i < n; ++i) {
            R t = times[i] * dt;
            x4 = x4 + v4 * t; x1 = x1 + v1 * t; x2 = x2 + v2 * t; x3 = x3 + v3 * t;
            if (test_vf(x4, x1, x2, x3, c, th, nout)) return true;
        }
        return false;
    }
    bool ee_candidate(Contact &c, R th, R dt) {
        V e1min = vmin(pmin[c.v[0]], pmin[c.v[1]]), e1max = vmax(pmax[c.v[0]], pmax[c.v[1]]);
        V e2min = vmin(pmin[c.v[2]], pmin[c.v[3]]), e2max = vmax(pmax[c.v[2]], pmax[c.v[3]]);
        if (!overlap(e1min, e1max, e2min, e2max)) return false;
        if (c.v[0] == c.v[2] || c.v[0] == c.v[3] || c.v[1] == c.v[2] || c.v[1] == c.v[3]) return false;
        V x1 = xp[c.v[0]], x2 = xp[c.v[1]], x3 = xp[c.v[2]], x4 = xp[c.v[3]];
        V v1 = v[c.v[0]], v2 = v[c.v[1]], v3 = v[c.v[2]], v4 = v[c.v[3]];
        R times[8];
        int n = coplanarity_times(x1, x2, x3, x4, v1, v2, v3, v4, times);
        for (int i = 0; i < n; ++i) {
            R t = times[i] * dt;
            x1 = x1 + v1 * t; x2 = x2 + v2 * t; x3 = x3 + v3 * t; x4 = x4 + v4 * t;
            if (test_ee(x1, x2, x3, x4, c, th)) return true;
        }
        return false;
    }

    // ---- 6. PBDStepSolver (Physics/CudaPBD.cu:632-660) ----------------------
    void solve(const std::vector<Contact> &cvf, const std::vector<Contact> &cee) {
        int Vn = tp.V, F = (int)tp.fixed.size();
        R th = R(h);
        R gh = R(prm.worldMin[1]);
        // Physics/CudaPBD.cu:1477-1507 — ground constraints.
        std::vector<u8> &gflag = ground_flag;
        gflag.assign(Vn, 0);
        std::vector<V> qc(Vn), nc(Vn);
        if (prm.groundOn) {
            for (int i = 0; i < Vn; ++i) {
                V pos = x[i], prev = xp[i];
                if (forced.on ? forced.ground[i] != 0 : pos.y <= gh + th) {
                    V n = mk<R>(0, 1, 0);
                    V p0 = mk<R>(1, gh + th, 1);
                    V l = pos - prev;
                    R d = dot(p0 - pos, n) / dot(l, n);
                    qc[i] = d * l + pos;
                    nc[i] = n;
                    gflag[i] = 1;
                }
            }
        }
        // Physics/CudaPBD.cu:1571-1592 — LRA flags.
        std::vector<u8> lflag((size_t)Vn * F, 0);
        for (int i = 0; i < Vn; ++i) {
            if (tp.pinned[i]) continue;
            for (int j = 0; j < F; ++j) {
                const size_t k = (size_t)i * F + j;
                if (forced.on) lflag[k] = forced.lra[k];
                else if (dist(x[i], x[tp.fixed[j]]) > R(tp.lra_l0[k])) lflag[k] = 1;
            }
        }
        // Physics/CudaPBD.cu:1509-1569 — the analytic sphere projects x/x_prev
        // directly (its flags are never set, so no iteration term).
        if (prm.sphereOn) sphere_create(th);

        // Dynamic entries grouped by vertex in entry order (the stable sort +
        // RLE of Physics/CudaPBD.cu:711-721).
        size_t nvf = cvf.size(), nee = cee.size();
        std::vector<std::vector<u32>> dyn(Vn);
        for (size_t c = 0; c < nvf + nee; ++c) {
            const Contact &k = c < nvf ? cvf[c] : cee[c - nvf];
            for (int s = 0; s < 4; ++s) dyn[k.v[s]].push_back(u32(c * 4 + s));
        }
        int E = (int)tp.s1.size(), Bn = (int)tp.b1.size();
        std::vector<R> kps(E), kpb(Bn);
        for (int i = 0; i < E; ++i) kps[i] = kp_of(tp.kst[i]);
        for (int i = 0; i < Bn; ++i) kpb[i] = kp_of(tp.kbd[i]);

        std::vector<V> corr_stat(tp.sent.size());
        std::vector<V> corr_dyn((nvf + nee) * 4);
        std::vector<V> acc(Vn);
        std::vector<int> cnt(Vn);
        if (recording) {
            rec.vf = cvf; rec.ee = cee;
            rec.ground = gflag; rec.lra = lflag;
            rec.ground_it.assign(Vn, 0u);
            rec.dyn.assign((size_t)prm.solverIterations * corr_dyn.size(), 0);
            rec.xk.assign(1, x);
        }
        bend_min = bend_min_neg = contact_min = 1e300;
        for (int it = 0; it < prm.solverIterations; ++it) {
            if (track_bend) track_bend_conditioning();
            for (int i = 0; i < Vn; ++i) { acc[i] = mk<R>(0, 0, 0); cnt[i] = 0; }
            // ground, Physics/CudaPBD.cu:1594-1629
            for (int i = 0; i < Vn; ++i)
                if (gflag[i]) {
                    R cv = dot(x[i] - qc[i], nc[i]);
                    bool take = forced.on ? ((forced.ground_it[i] >> it) & 1u) != 0 : cv < R(0);
                    if (take) {
                        acc[i] = acc[i] + (-cv) * nc[i];
                        cnt[i] += 1;
                        if (recording) rec.ground_it[i] |= 1u << it;
                    }
                }
            // LRA, Physics/CudaPBD.cu:1656-1688
            for (int i = 0; i < Vn; ++i) {
                V a = mk<R>(0, 0, 0);
                int c = 0;
                for (int j = 0; j < F; ++j)
                    if (lflag[(size_t)i * F + j]) {
                        V diff = x[i] - x[tp.fixed[j]];
                        R l = len(diff);
                        V n = diff / l;
                        a = a + (-(l - R(tp.lra_l0[(size_t)i * F + j]))) * n;
                        ++c;
                    }
                acc[i] = acc[i] + a;
                cnt[i] += c;
            }
            // static constraints into per-vertex slots, Physics/CudaPBD.cu:942-1147
            for (int i = 0; i < Vn; ++i)
                for (int e = tp.soff[i]; e < tp.soff[i + 1]; ++e) corr_stat[e] = static_corr(tp.sent[e], kps, kpb);
            // Physics/CudaPBD.cu:1417-1446
            for (int i = 0; i < Vn; ++i) {
                V a = mk<R>(0, 0, 0);
                for (int e = tp.soff[i]; e < tp.soff[i + 1]; ++e) a = a + corr_stat[e];
                acc[i] = acc[i] + a;
                cnt[i] += tp.soff[i + 1] - tp.soff[i];
            }
            // dynamic, Physics/CudaPBD.cu:1190-1415 and :1448-1475
            for (size_t c = 0; c < nvf; ++c) vf_corr(cvf[c], th, &corr_dyn[c * 4]);
            for (size_t c = 0; c < nee; ++c) ee_corr(cee[c], th, &corr_dyn[(nvf + c) * 4]);
            if (track_bend) track_contact_conditioning(cvf, cee, th);
            for (int i = 0; i < Vn; ++i) {
                if (dyn[i].empty()) continue;
                V a = mk<R>(0, 0, 0);
                int c = 0;
                for (u32 e : dyn[i]) {
                    bool take = forced.on ? forced.dyn[(size_t)it * corr_dyn.size() + e] != 0 : !is_zero(corr_dyn[e]);
                    if (take) {
                        a = a + corr_dyn[e];
                        ++c;
                        if (recording) rec.dyn[(size_t)it * corr_dyn.size() + e] = 1;
                    }
                }
                acc[i] = acc[i] + a;
                cnt[i] += c;
            }
            // Physics/CudaPBD.cu:1690-1698 (no zero-count guard)
            for (int i = 0; i < Vn; ++i) x[i] = x[i] + acc[i] / R(cnt[i]);
            if (!coll_t.empty())
                for (int i = 0; i < Vn; ++i) coll_project_vertex(i, it + 1);
            if (recording) rec.xk.push_back(x);
        }
    }

    void track_contact_conditioning(const std::vector<Contact> &cvf, const std::vector<Contact> &cee, R th) {
        for (const Contact &k : cvf) {
            const R b0 = clampf(R(-k.w[1]), R(0), R(1)), b1 = clampf(R(-k.w[2]), R(0), R(1)),
                    b2 = clampf(R(-k.w[3]), R(0), R(1));
            const V n = x[k.v[0]] - (x[k.v[1]] * b0 + x[k.v[2]] * b1 + x[k.v[3]] * b2);
            contact_min = std::min(contact_min, double(len(n) / th));
        }
        for (const Contact &k : cee) {
            const V n = (x[k.v[0]] * R(k.w[0]) + x[k.v[1]] * R(k.w[1])) -
                        (x[k.v[2]] * R(-k.w[2]) + x[k.v[3]] * R(-k.w[3]));
            contact_min = std::min(contact_min, double(len(n) / th));
        }
    }

    void track_bend_conditioning() {
        if (tp.tri_bend) return;  // triangle bends have no dihedral angle
        for (size_t k = 0; k < tp.b1.size(); ++k) {
            const V &p2 = x[tp.b2[k]], &p3 = x[tp.b3[k]], &p4 = x[tp.b4[k]];
            const double a[3] = {(double)p2.x, (double)p2.y, (double)p2.z};
            const double b[3] = {(double)p3.x, (double)p3.y, (double)p3.z};
            const double c[3] = {(double)p4.x, (double)p4.y, (double)p4.z};
            const double u[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            const double w[3] = {a[1] * c[2] - a[2] * c[1], a[2] * c[0] - a[0] * c[2], a[0] * c[1] - a[1] * c[0]};
            const double lu = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
            const double lw = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            if (lu <= 0 || lw <= 0) continue;
            const double d = (u[0] * w[0] + u[1] * w[1] + u[2] * w[2]) / (lu * lw);
            bend_min = std::min(bend_min, 1.0 - d);
            bend_min_neg = std::min(bend_min_neg, 1.0 + d);
        }
    }

    V static_corr(int ent, const std::vector<R> &kps, const std::vector<R> &kpb) const {
        int kind = (ent >> 30) & 1, role = (ent >> 28) & 3, c = ent & 0x0FFFFFFF;
        if (kind == ENT_STRETCH) {
            // Physics/CudaPBD.cu:986-1022
            R kp = kps[c];
            int i1 = tp.s1[c], i2 = tp.s2[c];
            R w1 = invm[i1], w2 = invm[i2], ws = w1 + w2;
            if (ws == R(0)) return mk<R>(0, 0, 0);
            V diff = x[i1] - x[i2];
            R l = len(diff);
            if (l <= R(kEpsPbd)) return mk<R>(0, 0, 0);
            V n = diff / l;
            V tt = (l - R(tp.sl0[c])) * n * kp / ws;
            return role == 0 ? (-w1) * tt : w2 * tt;
        }
        if (tp.tri_bend) {
            // Physics/CudaPBD.cu:1149-1187 — triangle bend (b0, b1, v)
            R kp = kpb[c];
            const int i0 = tp.b1[c], i1 = tp.b2[c], iv = tp.b3[c];
            R wb0 = invm[i0], wb1 = invm[i1], wv = invm[iv];
            R W = wb0 + wb1 + R(2) * wv;
            V cc = (x[i0] + x[i1] + x[iv]) / R(3);
            V hv = x[iv] - cc;
            R l = len(hv);
            if (l <= R(kEpsPbd)) return mk<R>(0, 0, 0);
            V term = kp * (hv / W) * (R(1) - R(tp.th0[c]) / l);
            if (role == 0) return (R(2) * wb0) * term;
            if (role == 1) return (R(2) * wb1) * term;
            return (R(-4) * wv) * term;
        }
        // Physics/CudaPBD.cu:1024-1147 (raw positions, phi0 = PI)
        R kp = kpb[c];
        int id[4] = {tp.b1[c], tp.b2[c], tp.b3[c], tp.b4[c]};
        R w[4] = {invm[id[0]], invm[id[1]], invm[id[2]], invm[id[3]]};
        V p2 = x[id[1]], p3 = x[id[2]], p4 = x[id[3]];
        V c23 = cross(p2, p3), c24 = cross(p2, p4);
        R l23 = len(c23), l24 = len(c24);
        if (l23 <= R(kEpsPbd) || l24 <= R(kEpsPbd)) return mk<R>(0, 0, 0);
        V n1 = c23 / l23, n2 = c24 / l24;
        R d = clampf(dot(n1, n2), R(-1), R(1));
        R phi = std::acos(d);
        R phi0 = R(kPi);
        if (d == R(-1)) {
            phi = R(kPi);
            if (phi == phi0) return mk<R>(0, 0, 0);
            if (role == 0) return n1 / R(100);
            if (role == 1) return n2 / R(100);
            return mk<R>(0, 0, 0);
        }
        if (d == R(1)) {
            phi = R(0);
            if (phi == phi0) return mk<R>(0, 0, 0);
        }
        V q3 = (cross(p2, n2) + (cross(n1, p2) * d)) / l23;
        V q4 = (cross(p2, n1) + (cross(n2, p2) * d)) / l24;
        V q2 = -((cross(p3, n2) + (cross(n1, p3) * d)) / l23) - ((cross(p4, n1) + (cross(n2, p4) * d)) / l24);
        V q1 = -q2 - q3 - q4;
        R term = std::sqrt(R(1) - d * d) * (phi - phi0) * kp;
        R s1 = dot(q1, q1), s2 = dot(q2, q2), s3 = dot(q3, q3), s4 = dot(q4, q4);
        R sf = w[0] * s1 + w[1] * s2 + w[2] * s3 + w[3] * s4;
        if (sf <= R(kEpsPbd)) return mk<R>(0, 0, 0);
        R ts = term / sf;
        V q[4] = {q1, q2, q3, q4};
        return (-(w[role] * ts)) * q[role];
    }

    // Physics/CudaPBD.cu:1212-1311
    void vf_corr(const Contact &k, R th, V out[4]) const {
        V p = x[k.v[0]], p0 = x[k.v[1]], p1 = x[k.v[2]], p2 = x[k.v[3]];
        R b0 = clampf(R(-k.w[1]), R(0), R(1)), b1 = clampf(R(-k.w[2]), R(0), R(1)), b2 = clampf(R(-k.w[3]), R(0), R(1));
        R w = invm[k.v[0]], w0 = invm[k.v[1]], w1 = invm[k.v[2]], w2 = invm[k.v[3]];
        V q = p0 * b0 + p1 * b1 + p2 * b2;
        V n = p - q;
        R l = len(n);
        n = n / l;
        R c = l - th;
        V g = n, g0 = -n * b0, g1 = -n * b1, g2 = -n * b2;
        R s = w + w0 * b0 * b0 + w1 * b1 * b1 + w2 * b2 * b2;
        if (s == R(0)) { out[0] = out[1] = out[2] = out[3] = mk<R>(0, 0, 0); return; }
        s = c / s;
        s = c < R(0) ? s : R(0);
        out[0] = (-s * w) * g; out[1] = (-s * w0) * g0; out[2] = (-s * w1) * g1; out[3] = (-s * w2) * g2;
    }
    // Physics/CudaPBD.cu:1313-1415
    void ee_corr(const Contact &k, R th, V out[4]) const {
        V p0 = x[k.v[0]], p1 = x[k.v[1]], p2 = x[k.v[2]], p3 = x[k.v[3]];
        R b0 = R(k.w[0]), b1 = R(k.w[1]), b2 = R(-k.w[2]), b3 = R(-k.w[3]);
        R w0 = invm[k.v[0]], w1 = invm[k.v[1]], w2 = invm[k.v[2]], w3 = invm[k.v[3]];
        V q0 = p0 * b0 + p1 * b1, q1 = p2 * b2 + p3 * b3;
        V n = q0 - q1;
        R l = len(n);
        n = n / l;
        R c = l - th;
        V g0 = n * b0, g1 = n * b1, g2 = -n * b2, g3 = -n * b3;
        R s = w0 * b0 * b0 + w1 * b1 * b1 + w2 * b2 * b2 + w3 * b3 * b3;
        if (s == R(0)) { out[0] = out[1] = out[2] = out[3] = mk<R>(0, 0, 0); return; }
        s = c / s;
        s = c < R(0) ? s : R(0);
        out[0] = (-s * w0) * g0; out[1] = (-s * w1) * g1; out[2] = (-s * w2) * g2; out[3] = (-s * w3) * g3;
    }

    // Physics/CudaPBD.cu:1509-1569 with Collision/CudaCollisionDetection.cu:529-567
    void sphere_create(R th) {
        V sc = mk<R>(prm.spherePos[0], prm.spherePos[1], prm.spherePos[2]);
        R rad = R(prm.sphereRadius) + th;
        if (recording) rec.sphere.assign(tp.V, 0);
        for (int i = 0; i < tp.V; ++i) {
            V pos = x[i], prev = xp[i];
            V q;
            int ret = ray_sphere(prev, pos, sc, rad, q);
            if (forced.on) {
                ret = forced.sphere[i];
                if (ret != 0) {
                    V dir = pos - prev;
                    if (is_zero(dir)) continue;
                    dir = dir / len(dir);
                    V m = prev - sc;
                    R b = dot(m, dir), c = dot(m, m) - rad * rad;
                    R disc = std::fmax(b * b - c, R(0));
                    q = prev + dir * (-b - std::sqrt(disc));
                }
            }
            if (recording) rec.sphere[i] = (int8_t)ret;
            if (ret == -1) {
                V qs = sc + normalize(q - sc) * rad;
                V ns = normalize(qs - sc);
                xp[i] = qs + ns * R(0.0001f);
                x[i] = qs;
            } else if (ret == 1) {
                V ns = normalize(q - sc);
                x[i] = q + ns * R(0.0001f);
            }
        }
    }
    static int ray_sphere(V p1, V p2, V c0, R rad, V &q) {
        V dir = p2 - p1;
        if (is_zero(dir)) return 0;
        R l = len(dir);
        dir = dir / l;
        V m = p1 - c0;
        R b = dot(m, dir);
        R c = dot(m, m) - rad * rad;
        if (c > R(0) && b > R(0)) return 0;
        R disc = b * b - c;
        if (disc < R(0)) return 0;
        R t = -b - std::sqrt(disc);
        if (t < R(0)) { q = p1 + dir * t; return -1; }
        if (t > l) return 0;
        q = p1 + dir * t;
        return 1;
    }

    // ---- 7. PBDStepIntegration + WorldConstraints ---------------------------
    void integrate() {
        R dt = R(prm.timestep);
        for (int i = 0; i < tp.V; ++i) {
            // Physics/CudaPBD.cu:1916-1932
            if (tp.pinned[i]) { v[i] = mk<R>(0, 0, 0); continue; }
            v[i] = (x[i] - xp[i]) / dt;
            xp[i] = x[i];
        }
        // Physics/CudaDeformableUtils.cu:260-269
        for (int i = 0; i < tp.V; ++i) {
            x[i] = mk(std::fmin(std::fmax(x[i].x, R(prm.worldMin[0])), R(prm.worldMax[0])),
                      std::fmin(std::fmax(x[i].y, R(prm.worldMin[1])), R(prm.worldMax[1])),
                      std::fmin(std::fmax(x[i].z, R(prm.worldMin[2])), R(prm.worldMax[2])));
        }
    }

    // ---- adjoint of one step ------------------------------------------------
    // f(d) = (|d| - l0) d/|d| and its (symmetric) Jacobian applied to g: the
    // shape shared by the stretch, LRA and contact corrections.
    static V f_jac(V d, R l, R l0, V g) {
        V n = d / l;
        return g - (l0 / l) * (g - dot(n, g) * n);
    }

    // Reverse of the bend correction (Physics/CudaPBD.cu:1024-1147), written on
    // the algebraically identical stable form: given the incoming gradients
    // ub[j] of the four corrections, returns the gradients of p2, p3, p4 (the
    // correction does not depend on p1) and of kp.
    static void bend_vjp(V p2, V p3, V p4, const R w[4], R kp, R gap, const V ub[4], V &g2, V &g3, V &g4,
                         R &gkp) {
        g2 = g3 = g4 = mk<R>(0, 0, 0);
        gkp = R(0);
        V c23 = cross(p2, p3), c24 = cross(p2, p4);
        R l23 = len(c23), l24 = len(c24);
        if (l23 <= R(kEpsPbd) || l24 <= R(kEpsPbd)) return;
        V n1 = c23 / l23, n2 = c24 / l24;
        V sv = n1 + n2, tv = n1 - n2;
        R ss = dot(sv, sv), tt = dot(tv, tv);
        if (ss == R(0)) return;
        R A = std::sqrt(ss), Bq = std::sqrt(tt);
        R dphi = gap - R(2) * std::atan2(A, Bq);
        R P = ss * tt / R(4), Rt = std::sqrt(P);
        R term = Rt * dphi * kp;
        R opd = ss / R(2);
        V u = sv - n1 * opd, wv = sv - n2 * opd;
        V a3 = cross(p2, u), a4 = cross(p2, wv), b3 = cross(p3, u), b4 = cross(p4, wv);
        V q[4];
        q[2] = a3 / l23;
        q[3] = a4 / l24;
        q[1] = -(b3 / l23 + b4 / l24);
        q[0] = -q[1] - q[2] - q[3];
        R sf = w[0] * dot(q[0], q[0]) + w[1] * dot(q[1], q[1]) + w[2] * dot(q[2], q[2]) + w[3] * dot(q[3], q[3]);
        if (sf <= R(kEpsPbd)) return;
        R sc = term / sf;
        // corr_j = -w_j sc q_j
        R gsc = 0;
        V gq[4];
        for (int j = 0; j < 4; ++j) { gsc += -w[j] * dot(q[j], ub[j]); gq[j] = ub[j] * (-w[j] * sc); }
        R gterm = gsc / sf, gsf = -gsc * sc / sf;
        for (int j = 0; j < 4; ++j) gq[j] = gq[j] + q[j] * (R(2) * w[j] * gsf);
        gq[1] = gq[1] - gq[0]; gq[2] = gq[2] - gq[0]; gq[3] = gq[3] - gq[0];
        V gb3 = -gq[1] / l23, gb4 = -gq[1] / l24;
        R gl23 = dot(gq[1], b3) / (l23 * l23) - dot(gq[2], a3) / (l23 * l23);
        R gl24 = dot(gq[1], b4) / (l24 * l24) - dot(gq[3], a4) / (l24 * l24);
        V ga3 = gq[2] / l23, ga4 = gq[3] / l24;
        V gu = mk<R>(0, 0, 0), gw = mk<R>(0, 0, 0);
        g2 = g2 + cross(u, ga3); gu = gu + cross(ga3, p2);
        g2 = g2 + cross(wv, ga4); gw = gw + cross(ga4, p2);
        g3 = g3 + cross(u, gb3); gu = gu + cross(gb3, p3);
        g4 = g4 + cross(wv, gb4); gw = gw + cross(gb4, p4);
        V gsv = gu + gw, gn1 = -gu * opd, gn2 = -gw * opd;
        R gss = -(dot(gu, n1) + dot(gw, n2)) / R(2), gtt = 0;
        R gRt = gterm * dphi * kp, gdphi = gterm * Rt * kp;
        gkp = gterm * Rt * dphi;
        if (Rt > R(0)) { R gP = gRt / (R(2) * Rt); gss += gP * tt / R(4); gtt += gP * ss / R(4); }
        R den = ss + tt;
        R gA = R(-2) * Bq / den * gdphi, gB = R(2) * A / den * gdphi;
        gss += gA / (R(2) * A);
        if (Bq > R(0)) gtt += gB / (R(2) * Bq);
        gsv = gsv + sv * (R(2) * gss);
        V gtv = tv * (R(2) * gtt);
        gn1 = gn1 + gsv + gtv; gn2 = gn2 + gsv - gtv;
        V gc23 = gn1 / l23 + n1 * (gl23 - dot(gn1, c23) / (l23 * l23));
        V gc24 = gn2 / l24 + n2 * (gl24 - dot(gn2, c24) / (l24 * l24));
        g2 = g2 + cross(p3, gc23) + cross(p4, gc24);
        g3 = g3 + cross(gc23, p2);
        g4 = g4 + cross(gc24, p2);
    }

    // Reverse-mode derivative of step() with the decisions of `r` held fixed
    // (contacts and their weights, ground / LRA activation, counted dynamic
    // terms; the wind term's vertex normals are held fixed too).  gx, gxp, gv
    // hold dL/d(x, x_prev, v) after the step and are overwritten with the
    // gradients before it; dL/dk of every stretch and bend constraint is
    // added to gks, gkb.  The analytic sphere is not differentiated.
    void backward(const Record &r, std::vector<V> &gx, std::vector<V> &gxp, std::vector<V> &gv,
                  std::vector<double> &gks, std::vector<double> &gkb) const {
        const int Vn = tp.V, F = (int)tp.fixed.size(), K = prm.solverIterations;
        const int E = (int)tp.s1.size(), Bn = (int)tp.b1.size();
        const R dt = R(prm.timestep), th = R(h);
        const V zero = mk<R>(0, 0, 0);
        const std::vector<V> &xs = r.xk.back();
        // integration and world clamp (Physics/CudaPBD.cu:1916-1932,
        // Physics/CudaDeformableUtils.cu:260-269)
        auto inside = [&](R v, int k) { return v > R(prm.worldMin[k]) && v < R(prm.worldMax[k]) ? R(1) : R(0); };
        std::vector<V> a(Vn), gxp0(Vn, zero);
        for (int i = 0; i < Vn; ++i) {
            V gc = mk(gx[i].x * inside(xs[i].x, 0), gx[i].y * inside(xs[i].y, 1), gx[i].z * inside(xs[i].z, 2));
            if (tp.pinned[i]) { a[i] = gc; gxp0[i] = gxp[i]; }
            else { a[i] = gxp[i] + gv[i] / dt + gc; gxp0[i] = -gv[i] / dt; }
        }
        // Jacobi iterations in reverse (Physics/CudaPBD.cu:648-659)
        std::vector<R> kps(E), kpb(Bn), dks(E), dkb(Bn);
        auto dkp = [&](double k) { double K1 = (double)K; return (1.0 / K1) * std::pow(1.0 - k, 1.0 / K1 - 1.0); };
        for (int i = 0; i < E; ++i) { kps[i] = kp_of(tp.kst[i]); dks[i] = R(dkp(tp.kst[i])); }
        for (int i = 0; i < Bn; ++i) { kpb[i] = kp_of(tp.kbd[i]); dkb[i] = R(dkp(tp.kbd[i])); }
        const size_t nvf = r.vf.size(), nee = r.ee.size(), ndyn = 4 * (nvf + nee);
        std::vector<int> stat_cnt(Vn), lra_cnt(Vn, 0);
        for (int i = 0; i < Vn; ++i) {
            stat_cnt[i] = tp.soff[i + 1] - tp.soff[i];
            for (int j = 0; j < F; ++j) lra_cnt[i] += r.lra[(size_t)i * F + j] ? 1 : 0;
        }
        const R gap = R(3.14159265358979323846) - R(kPi);
        std::vector<V> u(Vn), g(Vn);
        std::vector<int> cnt(Vn);
        for (int it = K - 1; it >= 0; --it) {
            const std::vector<V> &X = r.xk[it];
            coll_project_reverse(r, it + 1, a);
            for (int i = 0; i < Vn; ++i) cnt[i] = stat_cnt[i] + lra_cnt[i] + (int)((r.ground_it[i] >> it) & 1u);
            for (size_t c = 0; c < nvf + nee; ++c) {
                const Contact &k = c < nvf ? r.vf[c] : r.ee[c - nvf];
                for (int s2 = 0; s2 < 4; ++s2)
                    if (r.dyn[(size_t)it * ndyn + c * 4 + s2]) cnt[k.v[s2]] += 1;
            }
            for (int i = 0; i < Vn; ++i) { u[i] = cnt[i] ? a[i] / R(cnt[i]) : zero; g[i] = a[i]; }
            // ground (Physics/CudaPBD.cu:1594-1629): corr.y = -(x.y - (ground + h))
            for (int i = 0; i < Vn; ++i)
                if ((r.ground_it[i] >> it) & 1u) g[i].y -= u[i].y;
            // LRA (Physics/CudaPBD.cu:1656-1688): corr = -f(x_i - x_fixed)
            for (int i = 0; i < Vn; ++i)
                for (int j = 0; j < F; ++j)
                    if (r.lra[(size_t)i * F + j]) {
                        int fj = tp.fixed[j];
                        V d = X[i] - X[fj];
                        R l = len(d);
                        V dd = f_jac(d, l, R(tp.lra_l0[(size_t)i * F + j]), -u[i]);
                        g[i] = g[i] + dd;
                        g[fj] = g[fj] - dd;
                    }
            // stretch (Physics/CudaPBD.cu:986-1022)
            for (int c = 0; c < E; ++c) {
                int i1 = tp.s1[c], i2 = tp.s2[c];
                R w1 = invm[i1], w2 = invm[i2], ws = w1 + w2;
                if (ws == R(0)) continue;
                V d = X[i1] - X[i2];
                R l = len(d);
                if (l <= R(kEpsPbd)) continue;
                V comb = (u[i2] * w2 - u[i1] * w1) / ws;
                V dd = f_jac(d, l, R(tp.sl0[c]), comb * kps[c]);
                g[i1] = g[i1] + dd;
                g[i2] = g[i2] - dd;
                V fv = d - d * (R(tp.sl0[c]) / l);
                gks[c] += double(dot(fv, comb) * dks[c]);
            }
            // bend (Physics/CudaPBD.cu:1024-1147)
            for (int c = 0; c < Bn; ++c) {
                int id[4] = {tp.b1[c], tp.b2[c], tp.b3[c], tp.b4[c]};
                R w[4] = {invm[id[0]], invm[id[1]], invm[id[2]], invm[id[3]]};
                V ub[4] = {u[id[0]], u[id[1]], u[id[2]], u[id[3]]};
                V g2, g3, g4;
                R gk;
                bend_vjp(X[id[1]], X[id[2]], X[id[3]], w, kpb[c], gap, ub, g2, g3, g4, gk);
                g[id[1]] = g[id[1]] + g2; g[id[2]] = g[id[2]] + g3; g[id[3]] = g[id[3]] + g4;
                gkb[c] += double(gk * dkb[c]);
            }
            // contacts (Physics/CudaPBD.cu:1212-1415), taken entries only
            for (size_t c = 0; c < nvf + nee; ++c) {
                const bool isvf = c < nvf;
                const Contact &k = isvf ? r.vf[c] : r.ee[c - nvf];
                V ub[4];
                bool any = false;
                for (int s2 = 0; s2 < 4; ++s2) {
                    bool t = r.dyn[(size_t)it * ndyn + c * 4 + s2] != 0;
                    ub[s2] = t ? u[k.v[s2]] : zero;
                    any = any || t;
                }
                if (!any) continue;
                R wv[4] = {invm[k.v[0]], invm[k.v[1]], invm[k.v[2]], invm[k.v[3]]};
                R b[4], sgn[4];
                if (isvf) {
                    b[0] = R(1);
                    b[1] = clampf(R(-k.w[1]), R(0), R(1)); b[2] = clampf(R(-k.w[2]), R(0), R(1));
                    b[3] = clampf(R(-k.w[3]), R(0), R(1));
                    sgn[0] = R(1); sgn[1] = sgn[2] = sgn[3] = R(-1);
                } else {
                    b[0] = R(k.w[0]); b[1] = R(k.w[1]); b[2] = R(-k.w[2]); b[3] = R(-k.w[3]);
                    sgn[0] = sgn[1] = R(1); sgn[2] = sgn[3] = R(-1);
                }
                // nvec = sum_s sgn_s b_s x_s ; corr_s = -(w_s sgn_s b_s / den) f(nvec)
                R den = 0;
                for (int s2 = 0; s2 < 4; ++s2) den += wv[s2] * b[s2] * b[s2];
                if (den == R(0)) continue;
                V nv = zero;
                for (int s2 = 0; s2 < 4; ++s2) nv = nv + X[k.v[s2]] * (sgn[s2] * b[s2]);
                R l = len(nv);
                V comb = zero;
                for (int s2 = 0; s2 < 4; ++s2) comb = comb - ub[s2] * (wv[s2] * sgn[s2] * b[s2] / den);
                V dn = f_jac(nv, l, th, comb);
                for (int s2 = 0; s2 < 4; ++s2) g[k.v[s2]] = g[k.v[s2]] + dn * (sgn[s2] * b[s2]);
            }
            a.swap(g);
        }
        coll_project_reverse(r, 0, a);
        // ExplicitEuler (Physics/CudaPBD.cu:2005-2012): x = x_prev + dt v
        std::vector<V> gvc(Vn);
        for (int i = 0; i < Vn; ++i) { gxp0[i] = gxp0[i] + a[i]; gvc[i] = a[i] * dt; }
        // DampVelocities (Physics/CudaPBD.cu:411-458): v_c = v_b + kd (vcm + w x r - v_b)
        const double kd = prm.kDamp, kg = prm.globalVelDamp, M = r.M;
        double S1[3] = {0, 0, 0}, S2[3] = {0, 0, 0};
        auto dv3 = [](double a0, double a1, double a2) { return mk<double>(a0, a1, a2); };
        const V3<double> xcm = dv3(r.xcm[0], r.xcm[1], r.xcm[2]), om = dv3(r.om[0], r.om[1], r.om[2]);
        for (int i = 0; i < Vn; ++i) {
            V3<double> ri = dv3(r.x_in[i].x, r.x_in[i].y, r.x_in[i].z) - xcm;
            V3<double> gi = dv3(gvc[i].x, gvc[i].y, gvc[i].z);
            V3<double> cr = cross(ri, gi);
            S1[0] += gi.x; S1[1] += gi.y; S1[2] += gi.z;
            S2[0] += cr.x; S2[1] += cr.y; S2[2] += cr.z;
        }
        double omb[3] = {kd * S2[0], kd * S2[1], kd * S2[2]}, Lb[3];
        solve3(r.I, omb, Lb);  // I is symmetric: I^-T omb = I^-1 omb
        const V3<double> Lbar = dv3(Lb[0], Lb[1], Lb[2]);
        double Ib[3][3];
        for (int p = 0; p < 3; ++p)
            for (int q2 = 0; q2 < 3; ++q2) Ib[p][q2] = -Lb[p] * r.om[q2];
        const double trI = Ib[0][0] + Ib[1][1] + Ib[2][2];
        const V3<double> vcmbar = dv3(kd * S1[0], kd * S1[1], kd * S1[2]);
        std::vector<V3<double>> rbar(Vn);
        V3<double> rsum = dv3(0, 0, 0);
        for (int i = 0; i < Vn; ++i) {
            const double m = (double)mass[i];
            V3<double> ri = dv3(r.x_in[i].x, r.x_in[i].y, r.x_in[i].z) - xcm;
            V3<double> gi = dv3(gvc[i].x, gvc[i].y, gvc[i].z);
            V3<double> vb = dv3(r.v_b[i].x, r.v_b[i].y, r.v_b[i].z);
            V3<double> gvb = gi * (1.0 - kd) + vcmbar * (m / M) + cross(Lbar, ri) * m;
            V3<double> Isr = dv3((Ib[0][0] + Ib[0][0]) * ri.x + (Ib[0][1] + Ib[1][0]) * ri.y + (Ib[0][2] + Ib[2][0]) * ri.z,
                                 (Ib[1][0] + Ib[0][1]) * ri.x + (Ib[1][1] + Ib[1][1]) * ri.y + (Ib[1][2] + Ib[2][1]) * ri.z,
                                 (Ib[2][0] + Ib[0][2]) * ri.x + (Ib[2][1] + Ib[1][2]) * ri.y + (Ib[2][2] + Ib[2][2]) * ri.z);
            rbar[i] = cross(gi, om) * kd + cross(vb, Lbar) * m + (ri * (2.0 * trI) - Isr) * m;
            rsum = rsum + rbar[i];
            // v_b = (v + dt g_ext) (1 - kg)
            V3<double> gvn = gvb * (1.0 - kg);
            gv[i] = mk<R>(R(gvn.x), R(gvn.y), R(gvn.z));
        }
        for (int i = 0; i < Vn; ++i) {
            V3<double> gxi = rbar[i] - rsum * ((double)mass[i] / M);
            gx[i] = mk<R>(R(gxi.x), R(gxi.y), R(gxi.z));
        }
        gxp.swap(gxp0);
    }

    // ---- friction, CudaPBD::ApplyFriction (Physics/CudaPBD.cu:770-833) -------
    // Runs after the integration when useFriction is set (Physics/
    // CudaDeformableBody.cpp:596-602) and changes velocities only.
    //  * _DampVelRigid (:1879-1912), launched with 255 threads per block over
    //    ceil(V/256) blocks (:777), so only the first 255*ceil(V/256)
    //    vertices are reached: their normal velocity against the ground
    //    plane is scaled by 1 - kFriction and the sum reflected.  (The
    //    sphere flags it also reads are never set.)
    //  * _ApplyFrictionVF (:1745-1794) gives each of a VF contact's four
    //    vertices the contact's face normal; the stable sort + run-length
    //    sums of :813-824 add them per vertex in contact order.
    //    _ApplyFrictionEE (:1796-1845) leaves its entries' vertex ids
    //    unwritten (the lines are commented out), so those entries land on
    //    whatever ids the buffer held; here they are left out, which is what
    //    the reference computes when a step has no EE contacts.
    //  * FinalFrictionStep (:1700-1723): a vertex with a non-zero sum has its
    //    normal velocity along the summed direction scaled by
    //    (1 - kFriction)^count and the sum reflected.
    void friction(const std::vector<Contact> &cvf, const std::vector<V> &nrm) {
        const int Vn = tp.V;
        const R kf = R(prm.kFriction);
        const V up = mk<R>(0, 1, 0);
        auto reflect = [](V a, V n) { return a - R(2) * dot(a, n) * n; };
        const int reach = std::min(Vn, ((Vn + 255) / 256) * 255);
        for (int i = 0; i < reach; ++i) {
            if (!ground_flag[i]) continue;
            V vn = dot(v[i], up) * up;
            V vt = v[i] - vn;
            vn = vn * (R(1) - kf);
            v[i] = reflect(vt + vn, up);
        }
        std::vector<V> acc(Vn, mk<R>(0, 0, 0));
        std::vector<int> cnt(Vn, 0);
        for (size_t c = 0; c < cvf.size() && c < nrm.size(); ++c)
            for (int s = 0; s < 4; ++s) {
                acc[cvf[c].v[s]] = acc[cvf[c].v[s]] + nrm[c];
                cnt[cvf[c].v[s]] += 1;
            }
        for (int i = 0; i < Vn; ++i) {
            if (cnt[i] == 0 || is_zero(acc[i])) continue;
            V fn = normalize(acc[i]);
            V vn = dot(v[i], fn) * fn;
            V vt = v[i] - vn;
            vn = vn * R(std::pow(R(1) - kf, R(cnt[i])));
            v[i] = reflect(vn + vt, fn);
        }
    }

    // One FixedUpdate.  With frozen contacts and skip_collide, the collision
    // stages are not run (a teacher-forced step takes its contacts, and its
    // running normals, from elsewhere).
    bool skip_collide = false;
    void step() {
        external();
        pred_x = x; pred_xp = xp; pred_v = v;
        if (!(have_frozen && skip_collide)) collide();
        coll_project();
        if (have_frozen)
            solve(frozen_vf, frozen_ee);
        else
            solve(vf, ee);
        const bool frozen = have_frozen;
        have_frozen = false;
        have_frozen_coll = false;
        forced.on = false;
        integrate();
        if (prm.useFriction) {
            if (!frozen) friction(vf, vf_n);
            else if (frozen_vf_n.size() == frozen_vf.size()) friction(frozen_vf, frozen_vf_n);
        }
        frozen_vf_n.clear();
    }
};

}  // namespace lco
