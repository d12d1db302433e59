// lc_narrow_api.cu — the narrowphase as a callable boundary: the work of
// DeformableUtils::CreateTriangleTests followed by
// DeformableUtils::CCDTriangleTests (Collision/CudaCollisionDetection.cu:6-51,
// 223-283) or by DeformableUtils::DCDTriangleTests (:191-221) on caller data.
// Given the broadphase pairs of a triangle set, its feature-ownership bytes
// and the vertices' predicted positions, previous positions and velocities,
// it produces the VF and EE contacts in the reference's order, as full
// PrimitiveContact records, with the engine's own narrowphase kernels
// (lc_lbvh.cu): candidate masks with the sanity checks (and, for the
// continuous tests, the feature AABB cull), the ordered candidate expansion,
// the warp-queued CCD or the discrete tests, and the emit pass.
//
// A handle owns the work buffers, sized at creation for the largest vertex,
// triangle and pair counts it will see; every call validates the caller's
// indices on the device and reports bad ones instead of reading past an
// array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "lc_internal.cuh"

namespace lc {
void launch_narrow(const DevPtrs &d, const uint32_t *npairs, const uint32_t *ncv, const uint32_t *nce, int grid,
                   int stage, cudaStream_t st);
void scan_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap,
              uint32_t *partial, uint32_t *total_out, unsigned long long *total_out64, cudaStream_t st);
void set_last_error(const std::string &msg);  // lc_api.cu: text for lc_last_error_string()

constexpr uint32_t ERR_NP_INPUT = 1u << 8;  // a caller index was out of range

// Caller state (3 floats per vertex) into the float4 arrays the kernels read
// (x and v may be NULL for the discrete tests, which read x_prev only).
__global__ void k_np_state(const float *__restrict__ x, const float *__restrict__ xp, const float *__restrict__ v,
                           float4 *__restrict__ dx, float4 *__restrict__ dxp, float4 *__restrict__ dv, int V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    if (x) dx[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], 0.f);
    dxp[i] = make_float4(xp[3 * i], xp[3 * i + 1], xp[3 * i + 2], 0.f);
    if (v) dv[i] = make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.f);
}

// Triangle records (v1, v2, v3, ownership bits); a triangle with a vertex id
// out of range is flagged and replaced by (0, 0, 0), which every sanity check
// culls.
__global__ void k_np_tris(const uint32_t *__restrict__ tris, const uint8_t *__restrict__ feats, int T, int V,
                          int4 *__restrict__ out, uint32_t *err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const uint32_t a = tris[3 * t], b = tris[3 * t + 1], c = tris[3 * t + 2];
    const int f = feats ? (int)feats[t] : 0x3F;
    if (a >= (uint32_t)V || b >= (uint32_t)V || c >= (uint32_t)V) {
        atomicOr(err, ERR_NP_INPUT);
        out[t] = make_int4(0, 0, 0, 0);
        return;
    }
    out[t] = make_int4((int)a, (int)b, (int)c, f);
}

// Pairs into the kernels' list; an index out of range is flagged and its
// pair replaced by (0, 0), a triangle against itself, which yields no
// candidate.  Also sets the device pair count.
__global__ void k_np_pairs(const uint32_t *__restrict__ pairs, uint64_t P, int T, uint2 *__restrict__ out,
                           uint32_t *npairs, uint32_t *err) {
    const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p == 0) *npairs = (uint32_t)P;
    if (p >= P) return;
    const uint32_t i = pairs[2 * p], j = pairs[2 * p + 1];
    if (i >= (uint32_t)T || j >= (uint32_t)T) {
        atomicOr(err, ERR_NP_INPUT);
        out[p] = make_uint2(0u, 0u);
        return;
    }
    out[p] = make_uint2(i, j);
}

// Contacts (ids, weights, normal and time) into caller PrimitiveContact
// records, at most cap.
__global__ void k_np_out(const int4 *__restrict__ ids, const float4 *__restrict__ w, const float4 *__restrict__ tn,
                         const uint32_t *__restrict__ n, uint64_t internal_cap, lc_primitive_contact *__restrict__ out,
                         uint64_t cap) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t m = min(min((uint64_t)*n, internal_cap), cap);
    if (k >= m) return;
    const int4 a = ids[k];
    const float4 b = w[k], e = tn[k];
    lc_primitive_contact c;
    c.v[0] = a.x; c.v[1] = a.y; c.v[2] = a.z; c.v[3] = a.w;
    c.w[0] = b.x; c.w[1] = b.y; c.w[2] = b.z; c.w[3] = b.w;
    c.t = e.w;
    c.n[0] = e.x; c.n[1] = e.y; c.n[2] = e.z;
    out[k] = c;
}

}  // namespace lc

using namespace lc;

struct lc_narrowphase {
    DevPtrs d{};
    std::vector<void *> mem;
    int max_V = 0, max_T = 0;
    uint64_t max_P = 0;
    ClothDev *cloth = nullptr;
    uint32_t *npairs = nullptr, *ncand = nullptr, *ncand_e = nullptr, *nvf = nullptr, *nee = nullptr;
    int grid = 0;

    ~lc_narrowphase() {
        for (void *p : mem) cudaFree(p);
    }
    template <class T> bool alloc(T *&out, size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            out = nullptr;
            return false;
        }
        mem.push_back(p);
        out = static_cast<T *>(p);
        return true;
    }
};

static lc_status np_fail(lc_status s, const std::string &msg) {
    lc::set_last_error(msg);
    return s;
}

#define LC_NP_CUDA(call)                                                                          \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return np_fail(LC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

extern "C" {

lc_status lc_narrowphase_create(int32_t max_vertices, int32_t max_triangles, uint64_t max_pairs,
                                uint64_t candidate_capacity, uint64_t contact_capacity, lc_narrowphase **out) {
    if (!out || max_vertices < 3 || max_triangles < 1 || max_pairs < 1 || max_pairs > 0x7FFFFFFFull)
        return np_fail(LC_ERR_INVALID_ARG, "lc_narrowphase_create: bad arguments (pairs at most 2^31 - 1)");
    *out = nullptr;
    lc_narrowphase *h = new (std::nothrow) lc_narrowphase();
    if (!h) return np_fail(LC_ERR_OOM, "lc_narrowphase_create: host allocation failed");
    DevPtrs &d = h->d;
    h->max_V = max_vertices;
    h->max_T = max_triangles;
    h->max_P = max_pairs;
    const uint64_t V = (uint64_t)max_vertices, T = (uint64_t)max_triangles, P = max_pairs;
    d.C = 1;
    d.pair_cap = P;
    d.cand_cap = candidate_capacity ? candidate_capacity : std::min<uint64_t>(15 * P, std::max<uint64_t>(32 * T, 1u << 22));
    d.cand_cap = std::min<uint64_t>(d.cand_cap, 0x7FFFFFF0ull);
    d.vf_cap = d.ee_cap = contact_capacity ? contact_capacity : std::max<uint64_t>(8 * T, 4096);
    const uint64_t GC = P / kPairGroup + 1, HG = d.cand_cap / 32 + 1;
    int *vcl = nullptr, *tcl = nullptr;
    bool ok = h->alloc(h->cloth, 1) && h->alloc(vcl, V) && h->alloc(tcl, T) && h->alloc(d.x, V) &&
              h->alloc(d.xp, V) && h->alloc(d.v, V) && h->alloc(d.tri_slot, T) && h->alloc(d.pairs, P) &&
              h->alloc(d.pair_mask, P) && h->alloc(d.grp_vf_cnt, GC) && h->alloc(d.grp_ee_cnt, GC) &&
              h->alloc(d.grp_vf_off, GC + 1) && h->alloc(d.grp_ee_off, GC + 1) && h->alloc(d.ngroups, 1) &&
              h->alloc(d.cand, d.cand_cap) && h->alloc(d.cand_e, d.cand_cap) && h->alloc(d.hitg_n, 2) &&
              h->alloc(d.vf_v, d.vf_cap) && h->alloc(d.vf_w, d.vf_cap) && h->alloc(d.ee_v, d.ee_cap) &&
              h->alloc(d.ee_w, d.ee_cap) && h->alloc(d.hit_n, 2) && h->alloc(d.scan_tmp, kScanBlocks + 1) &&
              h->alloc(d.err, 1) && h->alloc(d.counters, 4) && h->alloc(h->npairs, 1) && h->alloc(h->ncand, 1) &&
              h->alloc(h->ncand_e, 1) && h->alloc(h->nvf, 1) && h->alloc(h->nee, 1) &&
              h->alloc(d.vf_tn, d.vf_cap) && h->alloc(d.ee_tn, d.ee_cap);
    for (int k = 0; k < 2 && ok; ++k)
        ok = h->alloc(d.hitg_mask[k], HG) && h->alloc(d.hitg_cnt[k], HG) && h->alloc(d.hitg_off[k], HG + 1) &&
             h->alloc(d.hit_q[k], k ? d.ee_cap : d.vf_cap) && h->alloc(d.hit_w[k], k ? d.ee_cap : d.vf_cap) &&
             h->alloc(d.hit_tn[k], k ? d.ee_cap : d.vf_cap);
    if (!ok) {
        delete h;
        return np_fail(LC_ERR_OOM, "lc_narrowphase_create: cudaMalloc failed");
    }
    d.cloth = h->cloth;
    d.vcloth = vcl;
    d.tcloth = tcl;
    cudaError_t e = cudaMemset(vcl, 0, sizeof(int) * V);
    if (e == cudaSuccess) e = cudaMemset(tcl, 0, sizeof(int) * T);
    if (e == cudaSuccess) e = cudaMemset(d.err, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(d.hitg_n, 0, 2 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(d.ngroups, 0, sizeof(uint32_t));
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        delete h;
        return np_fail(LC_ERR_CUDA, std::string("lc_narrowphase_create: ") + cudaGetErrorString(e));
    }
    h->grid = std::max(sms, 1) * 16;
    *out = h;
    return LC_OK;
}

lc_status lc_narrowphase_run(lc_narrowphase *h, int32_t mode, const float *x, const float *x_prev, const float *v,
                             int32_t num_vertices, const uint32_t *triangles, const uint8_t *features,
                             int32_t num_triangles, const uint32_t *pairs, uint64_t num_pairs, float thickness,
                             float timestep, lc_primitive_contact *vf_out, uint64_t vf_cap,
                             lc_primitive_contact *ee_out, uint64_t ee_cap, uint64_t *vf_count, uint64_t *ee_count,
                             void *stream) {
    const bool ccd = mode == LC_NARROW_CCD;
    if (!h || (mode != LC_NARROW_CCD && mode != LC_NARROW_DCD) || (ccd && (!x || !v || !(timestep > 0.f))) ||
        !x_prev || !triangles || !vf_count || !ee_count || (num_pairs && !pairs) || num_vertices < 3 ||
        num_vertices > h->max_V || num_triangles < 1 || num_triangles > h->max_T || num_pairs > h->max_P ||
        (vf_cap && !vf_out) || (ee_cap && !ee_out) || !(thickness >= 0.f))
        return np_fail(LC_ERR_INVALID_ARG, "lc_narrowphase_run: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    DevPtrs &d = h->d;
    d.Vtot = num_vertices;
    d.Ttot = num_triangles;
    ClothDev cd;
    std::memset(&cd, 0, sizeof(cd));
    cd.V = num_vertices;
    cd.T = num_triangles;
    cd.h = thickness;
    cd.dt = timestep;
    LC_NP_CUDA(cudaMemcpyAsync(h->cloth, &cd, sizeof(cd), cudaMemcpyHostToDevice, st));
    LC_NP_CUDA(cudaMemsetAsync(d.err, 0, sizeof(uint32_t), st));
    const int nb = kThreads;
    k_np_state<<<(num_vertices + nb - 1) / nb, nb, 0, st>>>(ccd ? x : nullptr, x_prev, ccd ? v : nullptr, d.x, d.xp,
                                                           d.v, num_vertices);
    k_np_tris<<<(num_triangles + nb - 1) / nb, nb, 0, st>>>(triangles, features, num_triangles, num_vertices,
                                                           d.tri_slot, d.err);
    k_np_pairs<<<(unsigned)std::max<uint64_t>((num_pairs + nb - 1) / nb, 1), nb, 0, st>>>(
        pairs, num_pairs, num_triangles, d.pairs, h->npairs, d.err);
    // Collision/CudaCollisionDetection.cu:53-189, with the cull of
    // Collision/CudaPrimitiveTests.cu:427-490 for the continuous tests, then
    // the ordered expansion
    launch_narrow(d, h->npairs, h->ncand, h->ncand_e, h->grid, ccd ? 0 : 6, st);
    const uint32_t gcap = (uint32_t)(d.pair_cap / kPairGroup + 1);
    scan_u32(d.grp_vf_cnt, d.grp_vf_off, d.ngroups, 0, gcap, d.scan_tmp, h->ncand, nullptr, st);
    scan_u32(d.grp_ee_cnt, d.grp_ee_off, d.ngroups, 0, gcap, d.scan_tmp, h->ncand_e, nullptr, st);
    launch_narrow(d, h->npairs, h->ncand, h->ncand_e, h->grid, 1, st);
    // Collision/CudaPrimitiveTests.cu:96-238: CCD on x_prev and v; or :21-94,
    // the discrete tests at x_prev
    launch_narrow(d, h->npairs, h->ncand, h->ncand_e, h->grid, ccd ? 2 : 7, st);
    launch_narrow(d, h->npairs, h->ncand, h->ncand_e, h->grid, ccd ? 5 : 8, st);
    const uint32_t hcap = (uint32_t)(d.cand_cap / 32 + 1);
    scan_u32(d.hitg_cnt[0], d.hitg_off[0], d.hitg_n, 0, hcap, d.scan_tmp, h->nvf, nullptr, st);
    scan_u32(d.hitg_cnt[1], d.hitg_off[1], d.hitg_n + 1, 0, hcap, d.scan_tmp, h->nee, nullptr, st);
    launch_narrow(d, h->npairs, h->ncand, h->ncand_e, h->grid, 3, st);
    if (vf_cap)
        k_np_out<<<(unsigned)std::max<uint64_t>((std::min(vf_cap, d.vf_cap) + nb - 1) / nb, 1), nb, 0, st>>>(
            d.vf_v, d.vf_w, d.vf_tn, h->nvf, d.vf_cap, vf_out, vf_cap);
    if (ee_cap)
        k_np_out<<<(unsigned)std::max<uint64_t>((std::min(ee_cap, d.ee_cap) + nb - 1) / nb, 1), nb, 0, st>>>(
            d.ee_v, d.ee_w, d.ee_tn, h->nee, d.ee_cap, ee_out, ee_cap);
    LC_NP_CUDA(cudaGetLastError());
    uint32_t counts[2] = {0, 0}, err = 0;
    LC_NP_CUDA(cudaMemcpyAsync(&counts[0], h->nvf, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    LC_NP_CUDA(cudaMemcpyAsync(&counts[1], h->nee, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    LC_NP_CUDA(cudaMemcpyAsync(&err, d.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    LC_NP_CUDA(cudaStreamSynchronize(st));
    *vf_count = counts[0];
    *ee_count = counts[1];
    if (err & ERR_NP_INPUT)
        return np_fail(LC_ERR_INVALID_ARG, "lc_narrowphase_run: a triangle or pair index is out of range");
    if (err & ERR_CAND_OVERFLOW)
        return np_fail(LC_ERR_CAPACITY_OVERFLOW, "lc_narrowphase_run: candidate capacity exceeded");
    if ((err & (ERR_VF_OVERFLOW | ERR_EE_OVERFLOW)) || counts[0] > vf_cap || counts[1] > ee_cap)
        return np_fail(LC_ERR_CAPACITY_OVERFLOW,
                       "lc_narrowphase_run: more contacts than capacity; the counts hold the full numbers");
    return LC_OK;
}

lc_status lc_narrowphase_destroy(lc_narrowphase *h) {
    if (h) {
        cudaDeviceSynchronize();
        delete h;
    }
    return LC_OK;
}

}  // extern "C"
