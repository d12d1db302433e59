// lc_response.cu — impulse-based collision response:
// CudaDeformableBody::SolveCollisions (Physics/CudaDeformableBody.cpp:523-548),
// i.e. DeformableUtils::CreateImpulses then ApplyImpulses
// (Collision/CudaCollisionResponse.cu:11-300), on caller data.
//
// Every contact gives four impulses (its vertices: weight times the impulse
// along its normal, VF contacts first).  The reference sorts them by vertex
// id with a stable radix sort, run-length encodes the ids and sums each run in
// sorted order; here each vertex gathers its impulse slots through a
// per-vertex list sorted by slot index — the same sequence, so the same sums
// bit for bit — and the reference's launch of AccumulateImpulses over the
// contact count's grid (ceil(C / 256) * 256 threads, one per run) is kept:
// vertices ranked past that many among those with impulses get none.
// Built with -fmad=false: the reference's separate roundings.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "lc_internal.cuh"

namespace lc {
void scan_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap,
              uint32_t *partial, uint32_t *total_out, unsigned long long *total_out64, cudaStream_t st);
void set_last_error(const std::string &msg);

namespace {

__device__ __forceinline__ float3 ldf3(const float *p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// Every contact's vertex ids lie in [0, V).
__global__ void k_imp_check(const lc_primitive_contact *__restrict__ vf, uint64_t nvf,
                            const lc_primitive_contact *__restrict__ ee, uint64_t nee, int V, uint32_t *bad) {
    const uint64_t id = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (id >= nvf + nee) return;
    const lc_primitive_contact &c = id < nvf ? vf[id] : ee[id - nvf];
    for (int k = 0; k < 4; ++k)
        if (c.v[k] < 0 || c.v[k] >= V) atomicOr(bad, 1u);
}

// _CreateImpulses / _CreateImpulseVF / _CreateImpulseEE / _CreateImpulse
// (Collision/CudaCollisionResponse.cu:142-254): the contact's four impulses,
// and the per-vertex impulse counts.
__global__ void k_imp_create(const float *__restrict__ pos, const float *__restrict__ vel,
                             const lc_primitive_contact *__restrict__ vf, uint64_t nvf,
                             const lc_primitive_contact *__restrict__ ee, uint64_t nee, float stiffness, float mass,
                             float dt, float h, float4 *__restrict__ vals, uint32_t *__restrict__ cnt) {
    const uint64_t id = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (id >= nvf + nee) return;
    const bool isvf = id < nvf;
    const lc_primitive_contact c = isvf ? vf[id] : ee[id - nvf];
    float3 vr;
    if (isvf) {
        const float3 cv1 = mul(ldf3(vel, c.v[0]), c.w[0]);
        const float3 cv2 = add(add(mul(ldf3(vel, c.v[1]), c.w[1]), mul(ldf3(vel, c.v[2]), c.w[2])),
                               mul(ldf3(vel, c.v[3]), c.w[3]));
        vr = add(cv1, cv2);
    } else {
        const float3 cv1 = add(mul(ldf3(vel, c.v[0]), c.w[0]), mul(ldf3(vel, c.v[1]), c.w[1]));
        const float3 cv2 = add(mul(ldf3(vel, c.v[2]), c.w[2]), mul(ldf3(vel, c.v[3]), c.w[3]));
        vr = add(cv1, cv2);
    }
    const float3 n = f3(c.n[0], c.n[1], c.n[2]);
    const float3 p = add(add(add(mul(ldf3(pos, c.v[0]), c.w[0]), mul(ldf3(pos, c.v[1]), c.w[1])),
                             mul(ldf3(pos, c.v[2]), c.w[2])),
                         mul(ldf3(pos, c.v[3]), c.w[3]));
    const float d = h - dot(p, n);
    const float vn = dot(vr, n);
    const float dts = (0.1f * d) / dt;
    float i = 0.f;
    if (vn < dts) i = -fminf(dt * stiffness * d, mass * (dts - vn));
    if (vn < 0) i += mass * vn * 0.5f;
    i = fminf(fmaxf(-mass * 0.1f * h, i), mass * 0.1f * h);
    const float ip = (2 * i) / (c.w[0] * c.w[0] + c.w[1] * c.w[1] + c.w[2] * c.w[2] + c.w[3] * c.w[3]);
    const float3 ipv = mul(n, ip);
    for (int k = 0; k < 4; ++k) {
        vals[4 * id + k] = f4(mul(ipv, c.w[k]), 0.f);
        atomicAdd(&cnt[c.v[k]], 1u);
    }
}

// Slots (contact * 4 + k) into their vertex's list, then each list sorted by
// slot: the order the reference's stable sort gives the vertex's run.
__global__ void k_imp_fill(const lc_primitive_contact *__restrict__ vf, uint64_t nvf,
                           const lc_primitive_contact *__restrict__ ee, uint64_t nee, const uint32_t *__restrict__ off,
                           uint32_t *__restrict__ cur, uint32_t *__restrict__ slots) {
    const uint64_t id = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (id >= nvf + nee) return;
    const lc_primitive_contact &c = id < nvf ? vf[id] : ee[id - nvf];
    for (int k = 0; k < 4; ++k) {
        const int v = c.v[k];
        slots[off[v] + atomicAdd(&cur[v], 1u)] = (uint32_t)(4 * id + k);
    }
}

__global__ void k_imp_sort(const uint32_t *__restrict__ off, uint32_t *__restrict__ slots, int V) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const uint32_t a = off[v], b = off[v + 1];
    for (uint32_t i = a + 1; i < b; ++i) {
        const uint32_t key = slots[i];
        uint32_t j = i;
        while (j > a && slots[j - 1] > key) {
            slots[j] = slots[j - 1];
            --j;
        }
        slots[j] = key;
    }
}

__global__ void k_imp_flag(const uint32_t *__restrict__ cnt, uint32_t *__restrict__ flag, int V) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < V) flag[v] = cnt[v] ? 1u : 0u;
}

// AccumulateImpulses (:256-280) for the runs its grid covers, then
// ApplyImpulses (:282-300).
__global__ void k_imp_apply(float *__restrict__ x, const float *__restrict__ xp, float *__restrict__ v,
                            const uint8_t *__restrict__ fixed, int V, const uint32_t *__restrict__ off,
                            const uint32_t *__restrict__ slots, const uint32_t *__restrict__ rank,
                            const float4 *__restrict__ vals, uint64_t threads, float mass, float dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V || fixed[i]) return;
    float3 acc = f3(0.f, 0.f, 0.f);
    const uint32_t a = off[i], b = off[i + 1];
    if (b > a && (uint64_t)rank[i] < threads) {
        float3 s = f3(0.f, 0.f, 0.f);
        for (uint32_t k = a; k < b; ++k) s = add(s, xyz(vals[slots[k]]));
        acc = dvs(s, (float)(int)(b - a));
    }
    const float3 nv = add(ldf3(v, i), dvs(acc, mass));
    const float3 np = add(ldf3(xp, i), mul(nv, dt));
    v[3 * i] = nv.x; v[3 * i + 1] = nv.y; v[3 * i + 2] = nv.z;
    x[3 * i] = np.x; x[3 * i + 1] = np.y; x[3 * i + 2] = np.z;
}

}  // namespace
}  // namespace lc

using namespace lc;

#define LC_R_CUDA(call)                                                                                 \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            lc::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));                     \
            status = LC_ERR_CUDA;                                                                       \
            goto done;                                                                                  \
        }                                                                                               \
    } while (0)

extern "C" lc_status lc_solve_collisions(float *x, const float *x_prev, float *v, const uint8_t *fixed,
                                         int32_t num_vertices, const lc_primitive_contact *vf, uint64_t num_vf,
                                         const lc_primitive_contact *ee, uint64_t num_ee, float stiffness,
                                         float vertex_mass, float timestep, float thickness, void *stream) {
    if (!x || !x_prev || !v || !fixed || num_vertices < 1 || (num_vf && !vf) || (num_ee && !ee) ||
        num_vf + num_ee > 0x3FFFFFFFull || !(vertex_mass > 0.f) || !(timestep > 0.f)) {
        lc::set_last_error("lc_solve_collisions: bad arguments");
        return LC_ERR_INVALID_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int V = num_vertices;
    const uint64_t C = num_vf + num_ee, S = 4 * C;
    const int nb = kThreads;
    const unsigned cblk = (unsigned)std::max<uint64_t>((C + nb - 1) / nb, 1), vblk = (unsigned)((V + nb - 1) / nb);
    lc_status status = LC_OK;
    uint32_t *cnt = nullptr, *off = nullptr, *cur = nullptr, *slots = nullptr, *flag = nullptr, *rank = nullptr,
             *part = nullptr, *bad = nullptr;
    float4 *vals = nullptr;
    uint32_t hbad = 0;
    // scratch in stream order from the device's default pool
    LC_R_CUDA(cudaMallocAsync((void **)&cnt, sizeof(uint32_t) * V, st));
    LC_R_CUDA(cudaMallocAsync((void **)&off, sizeof(uint32_t) * (V + 1), st));
    LC_R_CUDA(cudaMallocAsync((void **)&cur, sizeof(uint32_t) * V, st));
    LC_R_CUDA(cudaMallocAsync((void **)&flag, sizeof(uint32_t) * V, st));
    LC_R_CUDA(cudaMallocAsync((void **)&rank, sizeof(uint32_t) * (V + 1), st));
    LC_R_CUDA(cudaMallocAsync((void **)&part, sizeof(uint32_t) * (kScanBlocks + 1), st));
    LC_R_CUDA(cudaMallocAsync((void **)&bad, sizeof(uint32_t), st));
    LC_R_CUDA(cudaMallocAsync((void **)&slots, sizeof(uint32_t) * std::max<uint64_t>(S, 1), st));
    LC_R_CUDA(cudaMallocAsync((void **)&vals, sizeof(float4) * std::max<uint64_t>(S, 1), st));
    LC_R_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * V, st));
    LC_R_CUDA(cudaMemsetAsync(cur, 0, sizeof(uint32_t) * V, st));
    LC_R_CUDA(cudaMemsetAsync(bad, 0, sizeof(uint32_t), st));
    if (C) {
        k_imp_check<<<cblk, nb, 0, st>>>(vf, num_vf, ee, num_ee, V, bad);
        LC_R_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        LC_R_CUDA(cudaStreamSynchronize(st));
        if (hbad) {
            lc::set_last_error("lc_solve_collisions: a contact vertex id is out of range");
            status = LC_ERR_INVALID_ARG;
            goto done;
        }
        k_imp_create<<<cblk, nb, 0, st>>>(x_prev, v, vf, num_vf, ee, num_ee, stiffness, vertex_mass, timestep,
                                          thickness, vals, cnt);
    }
    scan_u32(cnt, off, nullptr, (uint32_t)V, (uint32_t)V, part, nullptr, nullptr, st);
    if (C) {
        k_imp_fill<<<cblk, nb, 0, st>>>(vf, num_vf, ee, num_ee, off, cur, slots);
        k_imp_sort<<<vblk, nb, 0, st>>>(off, slots, V);
    }
    k_imp_flag<<<vblk, nb, 0, st>>>(cnt, flag, V);
    scan_u32(flag, rank, nullptr, (uint32_t)V, (uint32_t)V, part, nullptr, nullptr, st);
    k_imp_apply<<<vblk, nb, 0, st>>>(x, x_prev, v, fixed, V, off, slots, rank, vals, (C + 255) / 256 * 256,
                                     vertex_mass, timestep);
    LC_R_CUDA(cudaGetLastError());
done:
    for (void *p : {(void *)cnt, (void *)off, (void *)cur, (void *)flag, (void *)rank, (void *)part, (void *)bad,
                    (void *)slots, (void *)vals})
        if (p) cudaFreeAsync(p, st);
    return status;
}
