// lc_api.cu — host side of the engine behind the C ABI of include/lc/lc.h:
// per-cloth construction (the work of the CudaDeformableBody constructor and
// CudaPBD::Init), the packed multi-cloth device layout, the launch sequence
// of one step (CudaDeformableBody::FixedUpdate) with every count kept on the
// device, CUDA-graph capture/replay, state I/O and debug dumps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "lc_internal.cuh"

namespace lc {
// launchers (lc_lbvh.cu, lc_step.cu, lc_scan.cu)
void launch_triangles(const DevPtrs &d, cudaStream_t st);
void launch_collider(const DevPtrs &d, int grid, cudaStream_t st);
void launch_collider_faces(const DevPtrs &d, int ntri, cudaStream_t st);
void launch_leaves_from_boxes(const DevPtrs &d, const float *bmin, const float *bmax, int T, int mode,
                              cudaStream_t st);
void launch_sort(const DevPtrs &d, const int *tile_first, int passes, cudaStream_t st);
void launch_post_sort(const DevPtrs &d, cudaStream_t st);
void launch_karras(const DevPtrs &d, cudaStream_t st);
void launch_refit(const DevPtrs &d, cudaStream_t st);
void launch_traverse(const DevPtrs &d, int block, cudaStream_t st);
void launch_pair_compact(const DevPtrs &d, cudaStream_t st);
void launch_narrow(const DevPtrs &d, const uint32_t *npairs, const uint32_t *ncv, const uint32_t *nce, int grid,
                   int stage, cudaStream_t st);
void launch_wind(const DevPtrs &d, cudaStream_t st);
void launch_external(const DevPtrs &d, cudaStream_t st, float4 *save_x = nullptr, float4 *save_v = nullptr);
void launch_adj_unpack(const AdjPtrs &A, const float *gx, const float *gxp, const float *gv, int n, cudaStream_t st);
void launch_adj_pack(const DevPtrs &d, const AdjPtrs &A, float *gx, float *gxp, float *gv, uint32_t *flag, int n,
                     cudaStream_t st);
void launch_adj_rescale(const DevPtrs &d, float *gx, float *gxp, float *gv, float *gks, float *gkb,
                        const uint32_t *flag, uint32_t *flag_next, int32_t *exponent, int E, int B, cudaStream_t st);
void launch_adjoint(const DevPtrs &d, const AdjPtrs &A, float4 *a, float4 *g, const uint32_t *nvf, const uint32_t *nee,
                    int grid, int nfixed, float *gk_stretch, float *gk_bend, cudaStream_t st);
void launch_vertex_normals(const DevPtrs &d, cudaStream_t st);
void launch_dyn(const DevPtrs &d, const uint32_t *nvf, const uint32_t *nee, int grid, int phase, cudaStream_t st);
void launch_solver_setup(const DevPtrs &d, bool sphere, cudaStream_t st);
void launch_jacobi(const DevPtrs &d, const float4 *xa, float4 *xb, int it, const uint32_t *nvf, int block,
                   cudaStream_t st);
void launch_integrate(const DevPtrs &d, const float4 *xs, cudaStream_t st);
void launch_friction(const DevPtrs &d, const uint32_t *nvf, cudaStream_t st);
void launch_vertex_records(const DevPtrs &d, void *dst, int64_t stride, int pos_off, int nrm_off, cudaStream_t st);
void launch_xyz_unpack(const float *src, float4 *dst, int n, cudaStream_t st);
void launch_xyz_pack(const float4 *src, float *dst, int n, cudaStream_t st);
void scan_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap,
              uint32_t *partial, uint32_t *total_out, unsigned long long *total_out64, cudaStream_t st);
unsigned long long morton3_host(float x, float y, float z, int mode);
struct ClusterArgs {
    const int *cl_cloth;
    const uint32_t *nvf;
    int chunk_cap;
    int contact_gather;      // scatter solver: contacts gathered per owned vertex (no remote atomics)
};
cudaError_t launch_solve_cluster(const DevPtrs &d, const ClusterArgs &a, int cs, bool scatter, int nclusters,
                                 cudaStream_t st);
int cluster_chunk_cap(bool scatter);
int cluster_max_active(int cs, int chunk_cap, bool scatter);
}  // namespace lc

using namespace lc;

static thread_local std::string g_last_error;

static lc_status fail(lc_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

namespace lc {
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace lc

#define LC_CUDA(call)                                                                               \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            return fail(e_ == cudaErrorMemoryAllocation ? LC_ERR_OOM : LC_ERR_CUDA,                 \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                        \
        }                                                                                           \
    } while (0)

// ---------------------------------------------------------------------------
// Host-side construction of one cloth.
// ---------------------------------------------------------------------------
struct HostCloth {
    int V = 0, T = 0;
    lc_cloth_params p{};
    float h = 0, vmass = 0;
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    std::vector<uint8_t> pinned;
    std::vector<int2> s_ids;
    std::vector<double> s_l0;
    std::vector<int4> b_ids;
    std::vector<int> soff;
    std::vector<uint32_t> sent;  // kind<<31 | role<<29 | local constraint
    std::vector<int> fixed;
    std::vector<float> lra_l0;
    std::vector<uint8_t> features;
    std::vector<int> vt_off, vt_idx;
    std::vector<float> vn0;  // initial vertex normals (3V)
};

static inline uint64_t ekey(int a, int b) {
    const uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
    return ((uint64_t)lo << 32) | hi;
}
static inline double pdist(const std::vector<float> &p, int a, int b) {
    const double dx = (double)p[3 * a] - p[3 * b], dy = (double)p[3 * a + 1] - p[3 * b + 1],
                 dz = (double)p[3 * a + 2] - p[3 * b + 2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// Physics/CudaPBD.cu:289-346 — (p1, p2) shared, p3 / p4 opposite.  The
// reference's first scan only breaks its inner loop, so p1 ends up as the
// last vertex of t1 (in t1 order) that t2 shares.
static void shared_edge(const int t1[3], const int t2[3], int &p1, int &p2, int &p3, int &p4) {
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

static lc_status build_host_cloth(const lc_cloth_desc &d, HostCloth &hc) {
    if (d.num_vertices < 2 || d.num_triangles < 1 || !d.positions || !d.indices)
        return fail(LC_ERR_INVALID_ARG, "cloth needs >= 2 vertices, >= 1 triangle, positions and indices");
    if (d.params.solverIterations < 1 || d.params.timestep <= 0.f || d.params.BVHChunkSize < 1)
        return fail(LC_ERR_INVALID_ARG, "solverIterations, timestep and BVHChunkSize must be positive");
    hc.V = d.num_vertices;
    hc.T = d.num_triangles;
    hc.p = d.params;
    hc.pos.assign(d.positions, d.positions + 3 * (size_t)hc.V);
    hc.idx.assign(d.indices, d.indices + 3 * (size_t)hc.T);
    for (uint32_t v : hc.idx)
        if (v >= (uint32_t)hc.V) return fail(LC_ERR_INVALID_ARG, "triangle index out of range");
    hc.pinned.assign(hc.V, 0);
    if (d.pinned)
        for (int i = 0; i < hc.V; ++i) hc.pinned[i] = d.pinned[i] ? 1 : 0;
    // Physics/CudaDeformableBody.cpp:52,86
    hc.vmass = d.params.objectMass / (float)hc.V;
    hc.h = d.params.thicknessFromMesh ? (float)(pdist(hc.pos, 0, 1) / 3.0) : d.params.thickness;

    // Physics/CudaPBD.cu:111-142 — stretch on first sighting of an edge, bend
    // on the second (which forgets the edge).
    std::unordered_map<uint64_t, int> open;
    open.reserve((size_t)hc.T * 2);
    for (int t = 0; t < hc.T; ++t) {
        const int tri[3] = {(int)hc.idx[3 * t], (int)hc.idx[3 * t + 1], (int)hc.idx[3 * t + 2]};
        for (int j = 0; j < 3; ++j) {
            const int a = tri[j], b = tri[(j + 1) % 3];
            const uint64_t k = ekey(a, b);
            auto it = open.find(k);
            if (it != open.end()) {
                const int o = it->second;
                const int t1[3] = {(int)hc.idx[3 * o], (int)hc.idx[3 * o + 1], (int)hc.idx[3 * o + 2]};
                int p1, p2, p3, p4;
                shared_edge(t1, tri, p1, p2, p3, p4);
                hc.b_ids.push_back(make_int4(p1, p2, p3, p4));
                open.erase(it);
            } else {
                open[k] = t;
                hc.s_ids.push_back(make_int2(a, b));
                hc.s_l0.push_back(pdist(hc.pos, a, b));
            }
        }
    }
    for (const int4 &b : hc.b_ids)
        if (b.x < 0 || b.y < 0 || b.z < 0 || b.w < 0)
            return fail(LC_ERR_INVALID_ARG, "degenerate triangle pair (repeated vertex) in the mesh");
    if (d.params.useTriangleBending) {
        // Physics/CudaPBD.cu:474-509 — triangle bends instead of the dihedral
        // ones: every three consecutive vertices of a grid row, then of a grid
        // column, (b0, v, b1), with h0 = |v - centroid|.  w holds h0's bits.
        const int nx = d.params.dims[0], ny = d.params.dims[1];
        if (nx < 1 || ny < 1 || (int64_t)nx * ny != hc.V)
            return fail(LC_ERR_INVALID_ARG, "useTriangleBending needs a grid cloth: dims[0] * dims[1] == vertex count");
        auto lin = [&](int i, int j) { return i * nx + j; };
        auto add_tri = [&](int v1, int v3, int v2) -> bool {
            if (v1 < 0 || v2 < 0 || v3 < 0 || v1 >= hc.V || v2 >= hc.V || v3 >= hc.V) return false;
            double c[3], h2 = 0;
            for (int k = 0; k < 3; ++k) c[k] = ((double)hc.pos[3 * v1 + k] + hc.pos[3 * v2 + k] + hc.pos[3 * v3 + k]) / 3.0;
            for (int k = 0; k < 3; ++k) h2 += ((double)hc.pos[3 * v3 + k] - c[k]) * ((double)hc.pos[3 * v3 + k] - c[k]);
            const float h0 = (float)std::sqrt(h2);
            int bits;
            std::memcpy(&bits, &h0, sizeof(bits));
            hc.b_ids.push_back(make_int4(v1, v2, v3, bits));
            return true;
        };
        hc.b_ids.clear();
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j + 2 < ny; ++j)
                if (!add_tri(lin(i, j), lin(i, j + 1), lin(i, j + 2)))
                    return fail(LC_ERR_INVALID_ARG, "triangle bend outside the grid");
        for (int i = 0; i + 2 < nx; ++i)
            for (int j = 0; j < ny; ++j)
                if (!add_tri(lin(i, j), lin(i + 1, j), lin(i + 2, j)))
                    return fail(LC_ERR_INVALID_ARG, "triangle bend outside the grid");
    }
    const int E = (int)hc.s_ids.size(), B = (int)hc.b_ids.size();
    const int roles = d.params.useTriangleBending ? 3 : 4;
    // Physics/CudaPBD.cu:146-233 — per-vertex slots, stretch first then bend.
    std::vector<int> cnt(hc.V, 0);
    for (const int2 &s : hc.s_ids) { cnt[s.x]++; cnt[s.y]++; }
    for (const int4 &b : hc.b_ids) {
        cnt[b.x]++; cnt[b.y]++; cnt[b.z]++;
        if (roles == 4) cnt[b.w]++;
    }
    hc.soff.assign(hc.V + 1, 0);
    for (int i = 0; i < hc.V; ++i) hc.soff[i + 1] = hc.soff[i] + cnt[i];
    hc.sent.assign(hc.soff[hc.V], 0);
    std::fill(cnt.begin(), cnt.end(), 0);
    auto put = [&](int v, uint32_t kind, uint32_t role, uint32_t c) {
        hc.sent[hc.soff[v] + cnt[v]++] = (kind << 31) | (role << 29) | c;
    };
    for (int i = 0; i < E; ++i) { put(hc.s_ids[i].x, 0, 0, i); put(hc.s_ids[i].y, 0, 1, i); }
    for (int i = 0; i < B; ++i) {
        put(hc.b_ids[i].x, 1, 0, i); put(hc.b_ids[i].y, 1, 1, i);
        put(hc.b_ids[i].z, 1, 2, i);
        if (roles == 4) put(hc.b_ids[i].w, 1, 3, i);
    }
    // Physics/CudaPBD.cu:48-81 — LRA to every pinned vertex.
    for (int i = 0; i < hc.V; ++i)
        if (hc.pinned[i]) hc.fixed.push_back(i);
    const int F = (int)hc.fixed.size();
    hc.lra_l0.assign((size_t)hc.V * F, 0.f);
    for (int i = 0; i < hc.V; ++i)
        for (int j = 0; j < F; ++j)
            if (!hc.pinned[i])
                hc.lra_l0[(size_t)i * F + j] =
                    (float)(pdist(hc.pos, i, hc.fixed[j]) * (1.0 + (double)d.params.strainLimit));
    // Collision/FeatureList.cu:84-132 — ownership: the reference races with
    // atomicExch; here the lowest original triangle index owns a feature.
    hc.features.assign(hc.T, 0);
    std::vector<uint8_t> vt(hc.V, 0);
    std::unordered_set<uint64_t> et;
    et.reserve((size_t)hc.T * 2);
    for (int t = 0; t < hc.T; ++t) {
        const int v1 = hc.idx[3 * t], v2 = hc.idx[3 * t + 1], v3 = hc.idx[3 * t + 2];
        uint8_t f = 0;
        if (!vt[v1]) { vt[v1] = 1; f |= 1 << 5; }
        if (!vt[v2]) { vt[v2] = 1; f |= 1 << 4; }
        if (!vt[v3]) { vt[v3] = 1; f |= 1 << 3; }
        if (et.insert(ekey(v1, v2)).second) f |= 1 << 2;
        if (et.insert(ekey(v2, v3)).second) f |= 1 << 1;
        if (et.insert(ekey(v3, v1)).second) f |= 1 << 0;
        hc.features[t] = f;
    }
    // vertex -> triangles (for the running vertex normals)
    std::vector<int> tc(hc.V, 0);
    for (uint32_t v : hc.idx) tc[v]++;
    hc.vt_off.assign(hc.V + 1, 0);
    for (int i = 0; i < hc.V; ++i) hc.vt_off[i + 1] = hc.vt_off[i] + tc[i];
    hc.vt_idx.assign(hc.vt_off[hc.V], 0);
    std::fill(tc.begin(), tc.end(), 0);
    for (int t = 0; t < hc.T; ++t)
        for (int k = 0; k < 3; ++k) {
            const int v = hc.idx[3 * t + k];
            hc.vt_idx[hc.vt_off[v] + tc[v]++] = t;
        }
    // Initial normals: Physics/CudaDeformableUtils.cu:37-64 (unnormalised face
    // normals) accumulated and normalised (:190-249).
    hc.vn0.assign(3 * (size_t)hc.V, 0.f);
    for (int t = 0; t < hc.T; ++t) {
        const float *a = &hc.pos[3 * hc.idx[3 * t]], *b = &hc.pos[3 * hc.idx[3 * t + 1]],
                    *c = &hc.pos[3 * hc.idx[3 * t + 2]];
        const float3 e1 = f3(b[0] - a[0], b[1] - a[1], b[2] - a[2]);
        const float3 e2 = f3(c[0] - a[0], c[1] - a[1], c[2] - a[2]);
        const float3 n = cross(e1, e2);
        for (int k = 0; k < 3; ++k) {
            float *o = &hc.vn0[3 * hc.idx[3 * t + k]];
            o[0] += n.x; o[1] += n.y; o[2] += n.z;
        }
    }
    for (int i = 0; i < hc.V; ++i) {
        float *o = &hc.vn0[3 * i];
        const float l = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        o[0] /= l; o[1] /= l; o[2] /= l;
    }
    return LC_OK;
}

// ---------------------------------------------------------------------------
// The batch.
// ---------------------------------------------------------------------------
struct DeviceArena {
    std::vector<void *> ptrs;
    ~DeviceArena() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T> lc_status alloc(T *&out, size_t n, const char *what) {
        out = nullptr;
        if (n == 0) n = 1;
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(LC_ERR_OOM, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
        }
        ptrs.push_back(p);
        out = (T *)p;
        return LC_OK;
    }
};

#define LC_TRY(x)                     \
    do {                              \
        lc_status s_ = (x);           \
        if (s_ != LC_OK) return s_;   \
    } while (0)

struct lc_batch {
    int C = 0;
    std::vector<HostCloth> hosts;
    std::vector<ClothDev> cds;
    lc_batch_options opt{};
    DevPtrs d{};
    DeviceArena arena;
    ClothDev *cloth_dev = nullptr;
    int *tile_first = nullptr;
    uint32_t *npairs = nullptr, *nvf = nullptr, *nee = nullptr, *ncand = nullptr, *ncand_e = nullptr;
    int max_iters = 1;
    bool any_wind = false, any_sphere = false;
    int sort_passes = 8;
    int narrow_grid = 0;
    int jacobi_block = 256, traverse_block = 128;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t cap_stream = nullptr;
    cudaStream_t last_stream = nullptr;
    std::vector<int> s_count, b_count;  // per cloth
    std::vector<int> e_off, b_off;
    // cluster-resident solver (lc_cluster.cu)
    bool use_cluster = false;
    int cluster_cs = 8;
    int want_cs = 0;  // 0: pick; 4, 8 or 16: requested through lc_batch_set_tuning
    bool cluster_scatter = false;
    ClusterArgs ca{};
    // adjoint (lc_batch_adjoint_step): the tape of one recorded step
    bool recording = false;
    AdjPtrs adj{};
    float4 *tape_x = nullptr, *tape_xin = nullptr, *tape_vb = nullptr;
    float4 *adj_a = nullptr, *adj_g = nullptr;
    uint32_t *adj_flag = nullptr;  // 2 x C rescale flags, used alternately (lc_batch_adjoint_step_rescaled)
    float *io = nullptr;           // 3 floats per vertex: staging of host <-> device state copies
    int adj_flip = 0;
    int nfixed = 0;
    // debug copies
    float4 *dbg_x = nullptr, *dbg_xp = nullptr, *dbg_v = nullptr;
    uint32_t *dbg_perm_before = nullptr;

    // global indices of the VF / EE contacts of one cloth (contiguous ranges)
    lc_status cloth_contacts(int c, bool vf, std::vector<uint64_t> &gidx, std::vector<int4> &iv,
                             std::vector<float4> &wv);

    // static triangle colliders (lc_batch_set_collider): host copies per
    // cloth, and the device arrays built from all of them
    struct Collider {
        std::vector<float> verts;
        std::vector<uint32_t> tris;
        int tbase = 0;    // first triangle in the flat device arrays
        bool cw = false;  // faces clockwise seen from the free side
    };
    std::vector<Collider> colliders;
    std::vector<void *> coll_mem;  // device arrays of the current colliders (rebuilt on every set)
    int *coll_slots_cnt = nullptr; // per-vertex contact slots (arena), allocated with the first collider
    int *coll_slots_face = nullptr;
    float4 *coll_slots_w = nullptr;

    void free_collider_arrays() {
        for (void *q : coll_mem) cudaFree(q);
        coll_mem.clear();
    }

    ~lc_batch() {
        invalidate_graph();
        if (cap_stream) cudaStreamDestroy(cap_stream);
        free_collider_arrays();
    }

    // graphs of the adjoint step (the recorded step and its reverse pass),
    // one per set of gradient buffers and rescale parity, most recent first
    struct AdjGraph {
        uintptr_t key[7];
        cudaGraph_t g;
        cudaGraphExec_t e;
    };
    std::vector<AdjGraph> adj_graphs;

    void invalidate_graph() {
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        for (AdjGraph &a : adj_graphs) {
            cudaGraphExecDestroy(a.e);
            cudaGraphDestroy(a.g);
        }
        adj_graphs.clear();
    }

    lc_status enqueue_step(cudaStream_t st);
    lc_status setup_cluster();

    // profiling: when non-null, events are recorded at phase boundaries
    cudaEvent_t *prof_ev = nullptr;    // 8 events per step
    cudaEvent_t *kern_ev = nullptr;    // pairs around single kernels: [0,1] jacobi, [2,3] traverse, [4,5] narrow
                                       // filter, [6,7] sort, [8,9] VF CCD, [10,11] EE CCD
    uint32_t launches = 0;
};

static int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

static lc_status enqueue_cluster_solver(lc_batch *b, cudaStream_t st);

#define LC_PHASE(k) do { if (prof_ev) LC_CUDA(cudaEventRecord(prof_ev[k], st)); } while (0)
#define LC_KEV(k) do { if (kern_ev) LC_CUDA(cudaEventRecord(kern_ev[k], st)); } while (0)

lc_status lc_batch::enqueue_step(cudaStream_t st) {
    const bool dbg = opt.debug_capture != 0;
    LC_PHASE(0);
    LC_CUDA(cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long) * 4, st));
    // 1. PBD External
    if (any_wind) launch_wind(d, st);
    launch_external(d, st, recording ? tape_xin : nullptr, recording ? tape_vb : nullptr);
    if (dbg) {
        LC_CUDA(cudaMemcpyAsync(dbg_x, d.x, sizeof(float4) * d.Vtot, cudaMemcpyDeviceToDevice, st));
        LC_CUDA(cudaMemcpyAsync(dbg_xp, d.xp, sizeof(float4) * d.Vtot, cudaMemcpyDeviceToDevice, st));
        LC_CUDA(cudaMemcpyAsync(dbg_v, d.v, sizeof(float4) * d.Vtot, cudaMemcpyDeviceToDevice, st));
        LC_CUDA(cudaMemcpyAsync(dbg_perm_before, d.perm, sizeof(uint32_t) * d.Ttot, cudaMemcpyDeviceToDevice, st));
    }
    LC_PHASE(1);
    // 2. Update Triangles
    launch_triangles(d, st);
    launch_vertex_normals(d, st);
    LC_PHASE(2);
    // 3. Build BVH
    LC_KEV(6);
    launch_sort(d, tile_first, sort_passes, st);
    LC_KEV(7);
    launch_post_sort(d, st);
    LC_CUDA(cudaMemcpyAsync(d.perm, d.perm_alt, sizeof(uint32_t) * d.Ttot, cudaMemcpyDeviceToDevice, st));
    LC_CUDA(cudaMemsetAsync(d.parent, 0xFF, sizeof(int) * (size_t)d.Ntot, st));
    launch_karras(d, st);
    launch_refit(d, st);
    LC_PHASE(3);
    // 4. Create Triangle Tests
    LC_KEV(2);
    launch_traverse(d, traverse_block, st);
    LC_KEV(3);
    scan_u32(d.pair_cnt, d.pair_off, nullptr, (uint32_t)d.Ttot, (uint32_t)d.Ttot, d.scan_tmp, npairs,
             &d.counters[0], st);
    launch_pair_compact(d, st);
    LC_PHASE(4);
    // 5. Perform Triangle Tests
    LC_KEV(4);
    launch_narrow(d, npairs, ncand, ncand_e, narrow_grid, 0, st);  // filter: masks + counts per group of pairs
    LC_KEV(5);
    const uint32_t gcap = (uint32_t)(d.pair_cap / kPairGroup + 1);
    scan_u32(d.grp_vf_cnt, d.grp_vf_off, d.ngroups, 0, gcap, d.scan_tmp, ncand, nullptr, st);
    scan_u32(d.grp_ee_cnt, d.grp_ee_off, d.ngroups, 0, gcap, d.scan_tmp, ncand_e, nullptr, st);
    launch_narrow(d, npairs, ncand, ncand_e, narrow_grid, 1, st);  // expand
    LC_KEV(8);
    launch_narrow(d, npairs, ncand, ncand_e, narrow_grid, 2, st);  // VF CCD
    LC_KEV(9);
    launch_narrow(d, npairs, ncand, ncand_e, narrow_grid, 5, st);  // EE CCD
    LC_KEV(10);
    const uint32_t hcap = (uint32_t)(d.cand_cap / 32 + 1);
    scan_u32(d.hitg_cnt[0], d.hitg_off[0], d.hitg_n, 0, hcap, d.scan_tmp, nvf, &d.counters[1], st);
    scan_u32(d.hitg_cnt[1], d.hitg_off[1], d.hitg_n + 1, 0, hcap, d.scan_tmp, nee, &d.counters[2], st);
    launch_narrow(d, npairs, ncand, ncand_e, narrow_grid, 3, st);  // write contacts
    launch_narrow(d, npairs, ncand, ncand_e, narrow_grid, 4, st);  // per-cloth ranges
    launch_collider(d, narrow_grid, st);                            // static colliders (lc_batch_set_collider)
    LC_PHASE(5);
    // 6. PBD Solver (+ 7. integration fused on the cluster path).  The
    // per-vertex contact CSR feeds the gather solvers; the scatter solver
    // walks the cloth's contact ranges instead.
    // The recorded step of an adjoint batch writes its iterates to the tape
    // and its decisions to the records the reverse pass replays, on either
    // solver; the reverse pass walks the per-vertex contact lists.
    const bool on_chip = use_cluster;
    const bool ordered = !(on_chip && cluster_scatter) || d.friction_any;  // float sums in entry order
    if (ordered || recording || (on_chip && cluster_scatter && ca.contact_gather)) {
        LC_CUDA(cudaMemsetAsync(d.dyn_cnt, 0, sizeof(uint32_t) * (size_t)d.Vtot, st));
        LC_CUDA(cudaMemsetAsync(d.dyn_cur, 0, sizeof(uint32_t) * (size_t)d.Vtot, st));
        launch_dyn(d, nvf, nee, narrow_grid, 0, st);
        scan_u32(d.dyn_cnt, d.dyn_off, nullptr, (uint32_t)d.Vtot, (uint32_t)d.Vtot, d.scan_tmp, nullptr, nullptr, st);
        launch_dyn(d, nvf, nee, narrow_grid, 1, st);
        if (ordered || recording) launch_dyn(d, nvf, nee, narrow_grid, 2, st);
    }
    if (on_chip) {
        LC_KEV(0);
        LC_TRY(enqueue_cluster_solver(this, st));
        LC_KEV(1);
        LC_PHASE(6);
        if (d.friction_any) launch_friction(d, nvf, st);
        LC_PHASE(7);
        LC_CUDA(cudaGetLastError());
        return LC_OK;
    }
    launch_solver_setup(d, any_sphere, st);
    float4 *a = d.x, *b = d.x2;
    if (recording) {  // iterates go to the tape: x^0 = prediction, x^{it+1} after iteration it
        LC_CUDA(cudaMemcpyAsync(tape_x, d.x, sizeof(float4) * (size_t)d.Vtot, cudaMemcpyDeviceToDevice, st));
        a = tape_x;
    }
    for (int it = 0; it < max_iters; ++it) {
        if (recording) b = tape_x + (size_t)(it + 1) * d.Vtot;
        if (it == 0) LC_KEV(0);
        launch_jacobi(d, a, b, it, nvf, jacobi_block, st);
        if (it == 0) LC_KEV(1);
        if (recording) a = b;
        else std::swap(a, b);
    }
    LC_PHASE(6);
    // 7. PBD Integration + WorldConstraints
    launch_integrate(d, a, st);
    if (d.friction_any) launch_friction(d, nvf, st);
    LC_PHASE(7);
    LC_CUDA(cudaGetLastError());
    return LC_OK;
}

// Solver + integration on the cluster-resident path (one launch).
static lc_status enqueue_cluster_solver(lc_batch *b, cudaStream_t st) {
    DevPtrs d = b->d;
    if (b->recording) {
        // the recorded step of an adjoint batch: iterates to the tape
        d.tape_x = b->tape_x;
        d.tape_K = b->max_iters;
    } else if (b->opt.adjoint && !b->opt.debug_capture) {
        // the other steps of an adjoint batch keep no records
        d.dbg_ground_it = nullptr;
        d.dbg_dyn_nz = nullptr;
        d.dbg_sphere = nullptr;
        d.coll_act = nullptr;
    }
    LC_CUDA(launch_solve_cluster(d, b->ca, b->cluster_cs, b->cluster_scatter, b->C, st));
    return LC_OK;
}

template <class T> static lc_status upload(T *dst, const std::vector<T> &src) {
    if (!src.empty()) LC_CUDA(cudaMemcpy(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
    return LC_OK;
}

// Cluster-resident solver: picks the cluster size for the largest cloth and
// the cluster -> cloth schedule (largest cloths first).  Leaves use_cluster
// false when some cloth does not fit on chip.
lc_status lc_batch::setup_cluster() {
    use_cluster = false;
    if (opt.solver_variant == 1) return LC_OK;
    // the scatter form is the default on-chip solver (each constraint
    // evaluated once per iteration); variant 2 selects the gather form
    const bool scatter = opt.solver_variant != 2;
    const int dev_cap = cluster_chunk_cap(scatter);
    int vmax = 0;
    bool ok = true;
    for (int c = 0; c < C; ++c) {
        vmax = std::max(vmax, hosts[c].V);
        if (cds[c].F > 8) ok = false;
    }
    // cluster size: the requested one (lc_tuning.cluster_size) if it fits,
    // else the one that keeps the most CTAs resident (more warps per SM to
    // hide the distributed-shared-memory latency), 8 on a tie
    int cs = 0;
    if (ok) {
        long best = 0;
        for (int cand : {8, 16, 4}) {
            if (want_cs && cand != want_cs) continue;
            const int cap = (vmax + cand - 1) / cand;
            if (cap > dev_cap) continue;
            const long act = (long)cluster_max_active(cand, cap, scatter) * cand;
            if (act > best) { best = act; cs = cand; }
        }
    }
    if (!cs) {
        if (opt.solver_variant >= 2) return fail(LC_ERR_NOT_SUPPORTED, "cluster solver: a cloth does not fit on chip");
        return LC_OK;
    }
    cluster_cs = cs;
    cluster_scatter = scatter;
    std::vector<int> order(C);
    for (int c = 0; c < C; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hosts[x].V > hosts[y].V; });
    int *clc;
    LC_TRY(arena.alloc(clc, C, "cl_cloth"));
    LC_TRY(upload(clc, order));
    ca.cl_cloth = clc;
    ca.nvf = nvf;
    ca.chunk_cap = (vmax + cs - 1) / cs;
    use_cluster = true;
    return LC_OK;
}

static void fill_cloth_dev(const HostCloth &hc, ClothDev &cd) {
    const lc_cloth_params &p = hc.p;
    cd.chunk = std::min(p.BVHChunkSize, hc.T);
    cd.iters = p.solverIterations;
    cd.wind_on = p.windOn ? 1 : 0;
    cd.ground_on = p.groundOn ? 1 : 0;
    cd.sphere_on = p.sphereOn ? 1 : 0;
    cd.tri_bend = p.useTriangleBending ? 1 : 0;
    cd.friction = p.useFriction ? 1 : 0;
    cd.kfriction = p.kFriction;
    cd.morton_mode = p.mortonMode;
    cd.leaf_quirk = p.refLeafAabbQuirk ? 1 : 0;
    cd.dt = p.timestep;
    cd.h = hc.h;
    cd.kdamp = p.kDamp;
    cd.kglobal = p.globalVelDamp;
    for (int k = 0; k < 3; ++k) {
        cd.g[k] = p.gravity[k];
        cd.wmin[k] = p.worldMin[k];
        cd.wmax[k] = p.worldMax[k];
        cd.morton_origin[k] = p.mortonOrigin[k];
        cd.sphere_pos[k] = p.spherePos[k];
        cd.wind_start[k] = p.startWindDir[k];
        cd.wind_min[k] = p.minWindDir[k];
        cd.wind_max[k] = p.maxWindDir[k];
    }
    cd.ground_y = p.worldMin[1];
    cd.morton_scale = p.mortonScale;
    cd.sphere_r = p.sphereRadius;
    cd.wind_var_min = p.windMinVariation;
    cd.wind_var_max = p.windMaxVariation;
}

static lc_status batch_build(lc_batch *b, const lc_cloth_desc *descs, int n, const lc_batch_options &opt_in) {
    lc_batch_options opt = opt_in;
    // adjoint batches: the reverse pass replays the global-memory Jacobi
    // iterations, so the recorded step runs on that solver; the steps that
    // are not recorded (the forward rollout, the segment re-runs) take the
    // on-chip solver when the cloths fit
    b->C = n;
    b->opt = opt;
    b->hosts.resize(n);
    for (int c = 0; c < n; ++c) LC_TRY(build_host_cloth(descs[c], b->hosts[c]));
    // offsets
    b->cds.resize(n);
    int64_t V = 0, T = 0, N = 0, I = 0, F = 0, E = 0, B = 0, S = 0, VT = 0;
    int64_t LRA = 0, PC = 0;
    b->e_off.resize(n);
    b->b_off.resize(n);
    b->s_count.resize(n);
    b->b_count.resize(n);
    std::vector<int> tile_first(n + 1, 0), stile_cloth, stile_start, vblk_cloth, vblk_start, vb_first(n + 1, 0);
    for (int c = 0; c < n; ++c) {
        HostCloth &hc = b->hosts[c];
        ClothDev &cd = b->cds[c];
        std::memset(&cd, 0, sizeof(cd));
        fill_cloth_dev(hc, cd);
        cd.v_off = (int)V; cd.V = hc.V;
        cd.t_off = (int)T; cd.T = hc.T;
        cd.n_off = (int)N;
        cd.i_off = (int)I;
        cd.pc_off = PC;
        cd.f_off = (int)F; cd.F = (int)hc.fixed.size();
        cd.lra_off = LRA;
        cd.s_off = (int)E; cd.s_cnt = (int)hc.s_ids.size();
        cd.b_off = (int)B; cd.b_cnt = (int)hc.b_ids.size();
        cd.coll_root = -1;
        cd.coll_cw = 0;
        b->e_off[c] = (int)E; b->b_off[c] = (int)B;
        b->s_count[c] = (int)hc.s_ids.size();
        b->b_count[c] = (int)hc.b_ids.size();
        tile_first[c] = (int)stile_cloth.size();
        vb_first[c] = (int)vblk_cloth.size();
        for (int s = 0; s < hc.T; s += kSortTile) { stile_cloth.push_back(c); stile_start.push_back((int)T + s); }
        for (int s = 0; s < hc.V; s += kThreads) { vblk_cloth.push_back(c); vblk_start.push_back((int)V + s); }
        V += hc.V; T += hc.T; N += 2 * hc.T - 1; I += hc.T - 1; F += cd.F;
        E += hc.s_ids.size(); B += hc.b_ids.size(); S += hc.sent.size(); VT += hc.vt_idx.size();
        LRA += (int64_t)hc.V * cd.F;
        PC += (int64_t)hc.T * cd.chunk;
        b->max_iters = std::max(b->max_iters, cd.iters);
        b->any_wind |= cd.wind_on != 0;
        b->any_sphere |= cd.sphere_on != 0;
        b->d.friction_any |= cd.friction;
        if (hc.p.mortonMode != b->hosts[0].p.mortonMode)
            return fail(LC_ERR_INVALID_ARG, "all cloths of a batch must use the same Morton mode");
    }
    tile_first[n] = (int)stile_cloth.size();
    vb_first[n] = (int)vblk_cloth.size();
    // pair slots below 2^31: the narrowphase loops stride 32-bit pair indices
    if (V > (1ll << 31) - 2 || T > (1ll << 31) - 2 || E + B >= (1ll << 29) || PC > 0x7FFFFFFFll)
        return fail(LC_ERR_INVALID_ARG, "batch too large for 32-bit indices");
    b->sort_passes = b->hosts[0].p.mortonMode == LC_MORTON_K30 ? 4 : 8;
    for (int c = 0; c < n && opt.adjoint; ++c)
        if (b->cds[c].tri_bend)
            return fail(LC_ERR_NOT_SUPPORTED, "adjoint: triangle bending is not differentiated");
    if (opt.adjoint && b->d.friction_any)
        return fail(LC_ERR_NOT_SUPPORTED, "adjoint: friction is not differentiated; create the batch without useFriction");

    DevPtrs &d = b->d;
    DeviceArena &A = b->arena;
    d.C = n; d.Vtot = (int)V; d.Ttot = (int)T; d.Ntot = (int)N; d.Itot = (int)I;
    d.nstiles = (int)stile_cloth.size();
    d.nvblk = (int)vblk_cloth.size();
    const uint64_t vf_cap = opt.vf_capacity ? opt.vf_capacity : std::max<uint64_t>(8 * (uint64_t)T, 4096);
    const uint64_t ee_cap = opt.ee_capacity ? opt.ee_capacity : std::max<uint64_t>(8 * (uint64_t)T, 4096);
    d.vf_cap = vf_cap; d.ee_cap = ee_cap;
    d.pair_cap = (uint64_t)PC;
    d.dyn_cap = 4 * (vf_cap + ee_cap);

    ClothDev *cdev; ClothState *cst;
    LC_TRY(A.alloc(cdev, n, "cloth table")); d.cloth = cdev; b->cloth_dev = cdev;
    LC_TRY(A.alloc(cst, n, "cloth state")); d.cstate = cst;
    int *vcl, *tcl; LC_TRY(A.alloc(vcl, V, "vcloth")); LC_TRY(A.alloc(tcl, T, "tcloth"));
    d.vcloth = vcl; d.tcloth = tcl;
    LC_TRY(A.alloc(d.x, V, "x")); LC_TRY(A.alloc(d.x2, V, "x2")); LC_TRY(A.alloc(d.xp, V, "xp"));
    LC_TRY(A.alloc(d.v, V, "v")); LC_TRY(A.alloc(d.vn, V, "vn"));
    int4 *tri; LC_TRY(A.alloc(tri, T, "tri")); d.tri = tri;
    LC_TRY(A.alloc(d.perm, T, "perm")); LC_TRY(A.alloc(d.perm_alt, T, "perm_alt"));
    LC_TRY(A.alloc(d.tri_slot, T, "tri_slot"));
    LC_TRY(A.alloc(d.keys, T, "keys")); LC_TRY(A.alloc(d.keys_alt, T, "keys_alt"));
    LC_TRY(A.alloc(d.payload, T, "payload")); LC_TRY(A.alloc(d.payload_alt, T, "payload_alt"));
    LC_TRY(A.alloc(d.fn, T, "fn"));
    int *vto, *vti; LC_TRY(A.alloc(vto, V + 1, "vt_off")); LC_TRY(A.alloc(vti, VT, "vt_idx"));
    d.vt_off = vto; d.vt_idx = vti;
    LC_TRY(A.alloc(d.nmin, N, "nmin")); LC_TRY(A.alloc(d.nmax, N, "nmax"));
    LC_TRY(A.alloc(d.leaf_tmp_min, T, "leaf_tmp_min")); LC_TRY(A.alloc(d.leaf_tmp_max, T, "leaf_tmp_max"));
    LC_TRY(A.alloc(d.parent, N, "parent")); LC_TRY(A.alloc(d.child, I, "child"));
    LC_TRY(A.alloc(d.rml, I, "rml"));
    LC_TRY(A.alloc(d.wnode, 4 * std::max<int64_t>(I, 1), "wnode")); LC_TRY(A.alloc(d.visit, I, "visit"));
    LC_TRY(A.alloc(d.nend, I, "node range ends"));
    LC_TRY(A.alloc(d.rexit, 2 * std::max<int64_t>(I, 1), "refit exits")); LC_TRY(A.alloc(d.nrexit, 1, "refit exit count"));
    LC_TRY(A.alloc(d.pair_cnt, T, "pair_cnt")); LC_TRY(A.alloc(d.pair_off, T + 1, "pair_off"));
    LC_TRY(A.alloc(d.pair_chunk, PC, "pair_chunk")); LC_TRY(A.alloc(d.pairs, PC, "pairs"));
    LC_TRY(A.alloc(d.pair_mask, PC, "pair_mask"));
    LC_TRY(A.alloc(b->io, 3 * std::max<int64_t>(V, 1), "state staging"));
    const int64_t GC = PC / kPairGroup + 1;  // groups of kPairGroup pairs
    LC_TRY(A.alloc(d.grp_vf_cnt, GC, "grp_vf_cnt")); LC_TRY(A.alloc(d.grp_ee_cnt, GC, "grp_ee_cnt"));
    LC_TRY(A.alloc(d.grp_vf_off, GC + 1, "grp_vf_off")); LC_TRY(A.alloc(d.grp_ee_off, GC + 1, "grp_ee_off"));
    LC_TRY(A.alloc(d.ngroups, 1, "ngroups"));
    LC_CUDA(cudaMemset(d.ngroups, 0, sizeof(uint32_t)));
    // at most 15 candidates per pair; by default room for 32 per triangle
    d.cand_cap = opt.cand_capacity ? opt.cand_capacity
                                   : std::min<uint64_t>(15 * (uint64_t)PC, std::max<uint64_t>(32 * (uint64_t)T, 1u << 22));
    d.cand_cap = std::min<uint64_t>(d.cand_cap, 0x7FFFFFF0ull);  // strided 32-bit candidate loops stay below 2^32
    LC_TRY(A.alloc(d.cand, d.cand_cap, "vf candidates")); LC_TRY(A.alloc(d.cand_e, d.cand_cap, "ee candidates"));
    const uint64_t HG = d.cand_cap / 32 + 1;  // groups of 32 candidates
    for (int k = 0; k < 2; ++k) {
        LC_TRY(A.alloc(d.hitg_mask[k], HG, "hit masks")); LC_TRY(A.alloc(d.hitg_cnt[k], HG, "hit counts"));
        LC_TRY(A.alloc(d.hitg_off[k], HG + 1, "hit offsets"));
    }
    LC_TRY(A.alloc(d.hitg_n, 2, "hit groups"));
    LC_CUDA(cudaMemset(d.hitg_n, 0, 2 * sizeof(uint32_t)));
    LC_TRY(A.alloc(d.crange, n, "contact ranges"));
    LC_TRY(A.alloc(d.vf_v, vf_cap, "vf_v")); LC_TRY(A.alloc(d.vf_w, vf_cap, "vf_w"));
    LC_TRY(A.alloc(d.ee_v, ee_cap, "ee_v")); LC_TRY(A.alloc(d.ee_w, ee_cap, "ee_w"));
    LC_TRY(A.alloc(d.hit_q[0], vf_cap, "hit_q_vf")); LC_TRY(A.alloc(d.hit_w[0], vf_cap, "hit_w_vf"));
    LC_TRY(A.alloc(d.hit_q[1], ee_cap, "hit_q_ee")); LC_TRY(A.alloc(d.hit_w[1], ee_cap, "hit_w_ee"));
    LC_TRY(A.alloc(d.hit_n, 2, "hit_n"));
    if (d.friction_any) {
        LC_TRY(A.alloc(d.vf_n, vf_cap, "vf_n"));
        LC_TRY(A.alloc(d.hit_nrm, vf_cap, "hit_nrm_vf"));
    }
    LC_TRY(A.alloc(d.dyn_cnt, V, "dyn_cnt")); LC_TRY(A.alloc(d.dyn_off, V + 1, "dyn_off"));
    LC_TRY(A.alloc(d.dyn_cur, V, "dyn_cur")); LC_TRY(A.alloc(d.dyn_ent, d.dyn_cap, "dyn_ent"));
    int *soff; uint32_t *sent; int2 *sids; float2 *spar; int4 *bids; float *bkp;
    LC_TRY(A.alloc(soff, V + 1, "soff")); LC_TRY(A.alloc(sent, S, "sent"));
    LC_TRY(A.alloc(sids, E, "s_ids")); LC_TRY(A.alloc(spar, E, "s_par"));
    LC_TRY(A.alloc(bids, B, "b_ids")); LC_TRY(A.alloc(bkp, B, "b_kp"));
    d.soff = soff; d.sent = sent; d.s_ids = sids; d.s_par = spar; d.b_ids = bids; d.b_kp = bkp;
    int *fixed; float *lral0; LC_TRY(A.alloc(fixed, F, "fixed")); LC_TRY(A.alloc(lral0, LRA, "lra_l0"));
    d.fixed = fixed; d.lra_l0 = lral0;
    LC_TRY(A.alloc(d.lra_flag, LRA, "lra_flag"));
    LC_TRY(A.alloc(d.ground_qc, V, "ground_qc"));
    LC_TRY(A.alloc(d.damp, 16 * (size_t)n, "damp"));
    LC_TRY(A.alloc(d.counters, 4, "counters"));
    LC_TRY(A.alloc(d.err, 1, "err"));
    LC_TRY(A.alloc(d.scan_tmp, kScanBlocks + 1, "scan_tmp"));
    int *stc, *sts, *tf; LC_TRY(A.alloc(stc, stile_cloth.size(), "stile_cloth"));
    LC_TRY(A.alloc(sts, stile_start.size(), "stile_start")); LC_TRY(A.alloc(tf, n + 1, "tile_first"));
    d.stile_cloth = stc; d.stile_start = sts; b->tile_first = tf;
    LC_TRY(A.alloc(d.shist, (size_t)stile_cloth.size() * kSortBuckets, "shist"));
    LC_TRY(A.alloc(d.sseg, kSortPassesMax + (size_t)n * kSortPassesMax * kSortBuckets, "sort segment totals"));
    LC_TRY(A.alloc(d.sstat, (size_t)kSortPassesMax * stile_cloth.size() * kSortBuckets, "sort look-back status"));
    int *vbc, *vbs, *vbf; LC_TRY(A.alloc(vbc, vblk_cloth.size(), "vblk_cloth")); LC_TRY(A.alloc(vbs, vblk_start.size(), "vblk_start"));
    LC_TRY(A.alloc(vbf, vb_first.size(), "vb_first"));
    d.vblk_cloth = vbc; d.vblk_start = vbs; d.vb_first = vbf;
    LC_TRY(A.alloc(d.damp_part, 16 * vblk_cloth.size(), "damp_part"));
    LC_TRY(A.alloc(d.vbox, 2 * std::max<int64_t>(V, 1), "vertex swept boxes"));
    LC_TRY(A.alloc(b->npairs, 1, "npairs")); LC_TRY(A.alloc(b->nvf, 1, "nvf")); LC_TRY(A.alloc(b->nee, 1, "nee"));
    LC_TRY(A.alloc(b->ncand, 1, "ncand")); LC_TRY(A.alloc(b->ncand_e, 1, "ncand_e"));
    if (opt.debug_capture) {
        LC_TRY(A.alloc(b->dbg_x, V, "dbg_x")); LC_TRY(A.alloc(b->dbg_xp, V, "dbg_xp"));
        LC_TRY(A.alloc(b->dbg_v, V, "dbg_v")); LC_TRY(A.alloc(b->dbg_perm_before, T, "dbg_perm"));
    }
    if (opt.debug_capture || opt.adjoint) {  // the decisions the reverse pass replays
        LC_TRY(A.alloc(d.dbg_ground_it, V, "dbg_ground_it"));
        LC_TRY(A.alloc(d.dbg_dyn_nz, (size_t)b->max_iters * d.dyn_cap, "dbg_dyn_nz"));
        LC_TRY(A.alloc(d.dbg_sphere, V, "dbg_sphere"));
        LC_CUDA(cudaMemset(d.dbg_sphere, 0, (size_t)V));
    }
    d.kpi_gap = (float)(3.14159265358979323846 - (double)kPi);

    // host staging of the flat arrays
    std::vector<int> hv_cloth(V), ht_cloth(T), hvt_off(V + 1, 0), hvt_idx(VT), hsoff(V + 1, 0), hfixed(F);
    std::vector<float4> hx(V), hxp(V), hv(V, make_float4(0, 0, 0, 0)), hvn(V);
    std::vector<int4> htri(T);
    std::vector<uint32_t> hperm(T), hsent(S);
    std::vector<int2> hsids(E);
    std::vector<float2> hspar(E);
    std::vector<int4> hbids(B);
    std::vector<float> hbkp(B), hlra(LRA);
    std::vector<ClothState> hst(n);
    for (int c = 0; c < n; ++c) {
        const HostCloth &hc = b->hosts[c];
        const ClothDev &cd = b->cds[c];
        const int vo = cd.v_off, to = cd.t_off, eo = b->e_off[c], bo = b->b_off[c];
        const double iters = (double)hc.p.solverIterations;
        const float kps = (float)(1.0 - std::pow(1.0 - (double)hc.p.kStretch, 1.0 / iters));
        const float kpb = (float)(1.0 - std::pow(1.0 - (double)hc.p.kBend, 1.0 / iters));
        for (int i = 0; i < hc.V; ++i) {
            const float m = hc.pinned[i] ? 1000.f : hc.vmass;
            const float w = hc.pinned[i] ? 0.f : 1.f / hc.vmass;
            hx[vo + i] = make_float4(hc.pos[3 * i], hc.pos[3 * i + 1], hc.pos[3 * i + 2], w);
            hxp[vo + i] = make_float4(hc.pos[3 * i], hc.pos[3 * i + 1], hc.pos[3 * i + 2], m);
            hvn[vo + i] = make_float4(hc.vn0[3 * i], hc.vn0[3 * i + 1], hc.vn0[3 * i + 2], 0.f);
            hv_cloth[vo + i] = c;
        }
        const int so = (int)hsoff[vo];
        for (int i = 0; i <= hc.V; ++i) hsoff[vo + i] = so + hc.soff[i];
        for (size_t k = 0; k < hc.sent.size(); ++k) {
            const uint32_t e = hc.sent[k];
            const uint32_t kind = e >> 31;
            const uint32_t local = e & 0x1FFFFFFFu;
            hsent[so + k] = (e & 0xE0000000u) | (local + (uint32_t)(kind ? bo : eo));
        }
        for (int t = 0; t < hc.T; ++t) {
            htri[to + t] = make_int4(vo + (int)hc.idx[3 * t], vo + (int)hc.idx[3 * t + 1], vo + (int)hc.idx[3 * t + 2],
                                     hc.features[t]);
            hperm[to + t] = (uint32_t)(to + t);
            ht_cloth[to + t] = c;
        }
        const int vto0 = hvt_off[vo];
        for (int i = 0; i <= hc.V; ++i) hvt_off[vo + i] = vto0 + hc.vt_off[i];
        for (size_t k = 0; k < hc.vt_idx.size(); ++k) hvt_idx[vto0 + k] = to + hc.vt_idx[k];
        for (size_t k = 0; k < hc.s_ids.size(); ++k) {
            hsids[eo + k] = make_int2(vo + hc.s_ids[k].x, vo + hc.s_ids[k].y);
            hspar[eo + k] = make_float2((float)hc.s_l0[k], kps);
        }
        for (size_t k = 0; k < hc.b_ids.size(); ++k) {
            const int4 q = hc.b_ids[k];
            hbids[bo + k] = make_int4(vo + q.x, vo + q.y, vo + q.z, vo + q.w);
            hbkp[bo + k] = kpb;
        }
        for (int j = 0; j < cd.F; ++j) hfixed[cd.f_off + j] = vo + hc.fixed[j];
        for (size_t k = 0; k < hc.lra_l0.size(); ++k) hlra[cd.lra_off + k] = hc.lra_l0[k];
        ClothState s{};
        for (int k = 0; k < 3; ++k) s.wind[k] = hc.p.windOn ? hc.p.startWindDir[k] : 0.f;
        s.rng = hc.p.windSeed ? hc.p.windSeed : 0x9E3779B97F4A7C15ull;
        hst[c] = s;
    }
    LC_TRY(upload(cdev, b->cds));
    LC_TRY(upload(cst, hst));
    LC_TRY(upload(vcl, hv_cloth)); LC_TRY(upload(tcl, ht_cloth));
    LC_TRY(upload(d.x, hx)); LC_TRY(upload(d.xp, hxp)); LC_TRY(upload(d.v, hv)); LC_TRY(upload(d.vn, hvn));
    LC_TRY(upload(tri, htri)); LC_TRY(upload(d.perm, hperm));
    LC_TRY(upload(vto, hvt_off)); LC_TRY(upload(vti, hvt_idx));
    LC_TRY(upload(soff, hsoff)); LC_TRY(upload(sent, hsent));
    LC_TRY(upload(sids, hsids)); LC_TRY(upload(spar, hspar));
    LC_TRY(upload(bids, hbids)); LC_TRY(upload(bkp, hbkp));
    LC_TRY(upload(fixed, hfixed)); LC_TRY(upload(lral0, hlra));
    LC_TRY(upload(stc, stile_cloth)); LC_TRY(upload(sts, stile_start)); LC_TRY(upload(tf, tile_first));
    LC_TRY(upload(vbc, vblk_cloth)); LC_TRY(upload(vbs, vblk_start)); LC_TRY(upload(vbf, vb_first));
    LC_CUDA(cudaMemset(d.err, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(d.counters, 0, sizeof(unsigned long long) * 4));
    LC_CUDA(cudaMemset(d.ground_qc, 0, sizeof(float4) * (size_t)std::max<int64_t>(V, 1)));
    LC_CUDA(cudaMemset(d.dyn_off, 0, sizeof(uint32_t) * (size_t)(V + 1)));
    LC_CUDA(cudaMemset(b->npairs, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(b->nvf, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(b->nee, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(b->ncand, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(b->ncand_e, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(d.crange, 0, sizeof(uint4) * (size_t)n));
    LC_CUDA(cudaMemset(d.nmin, 0, sizeof(float4) * (size_t)N));
    LC_CUDA(cudaMemset(d.nmax, 0, sizeof(float4) * (size_t)N));
    if (opt.adjoint) {
        AdjPtrs &J = b->adj;
        LC_TRY(A.alloc(b->tape_x, (size_t)(b->max_iters + 1) * V, "tape_x"));
        LC_TRY(A.alloc(b->tape_xin, V, "tape_xin")); LC_TRY(A.alloc(b->tape_vb, V, "tape_vb"));
        LC_TRY(A.alloc(b->adj_a, V, "adj_a")); LC_TRY(A.alloc(b->adj_g, V, "adj_g"));
        LC_TRY(A.alloc(J.u, V, "adj_u"));
        LC_TRY(A.alloc(J.gx, V, "adj_gx")); LC_TRY(A.alloc(J.gxp, V, "adj_gxp")); LC_TRY(A.alloc(J.gv, V, "adj_gv"));
        LC_TRY(A.alloc(J.slot, std::max<int64_t>(S, 1), "adj_slot"));
        LC_TRY(A.alloc(J.dyn, std::max<uint64_t>(d.dyn_cap, 1), "adj_dyn"));
        LC_TRY(A.alloc(J.fixed, 3 * std::max<int64_t>(F, 1), "adj_fixed"));
        LC_CUDA(cudaMemset(J.fixed, 0, sizeof(float) * 3 * std::max<int64_t>(F, 1)));
        LC_TRY(A.alloc(J.red, 8 * (vblk_cloth.size() + (size_t)n), "adj_red"));
        LC_TRY(A.alloc(b->adj_flag, 2 * (size_t)n, "adj_flag"));
        LC_CUDA(cudaMemset(b->adj_flag, 0, sizeof(uint32_t) * 2 * (size_t)n));
        // static CSR entry of every (constraint, role): where a constraint's
        // reverse contribution to each of its vertices goes
        std::vector<int> sslot(std::max<int64_t>(2 * E, 1), 0), bslot(std::max<int64_t>(4 * B, 1), 0);
        for (int64_t e = 0; e < S; ++e) {
            const uint32_t ent = hsent[e], k = ent & 0x1FFFFFFFu, role = (ent >> 29) & 3u;
            if (ent >> 31) bslot[4 * (size_t)k + role] = (int)e;
            else sslot[2 * (size_t)k + role] = (int)e;
        }
        int *ds, *db;
        LC_TRY(A.alloc(ds, sslot.size(), "s_slot")); LC_TRY(A.alloc(db, bslot.size(), "b_slot"));
        LC_TRY(upload(ds, sslot)); LC_TRY(upload(db, bslot));
        J.s_slot = ds; J.b_slot = db;
        J.tape_x = b->tape_x; J.tape_xin = b->tape_xin; J.tape_vb = b->tape_vb;
        J.nvblk_red = (int)vblk_cloth.size();
        J.K = b->max_iters;
        J.E = (int)E; J.B = (int)B;
        b->nfixed = (int)F;
    }
    b->narrow_grid = sm_count() * 8;
    b->jacobi_block = opt.block_size > 0 ? opt.block_size : 256;
    LC_TRY(b->setup_cluster());
    LC_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    LC_CUDA(cudaDeviceSynchronize());
    return LC_OK;
}

template <class T>
static lc_status dump(const T *src, uint64_t n, void *dst, uint64_t cap, uint64_t *count) {
    if (count) *count = n;
    if (dst && n && cap) LC_CUDA(cudaMemcpy(dst, src, sizeof(T) * std::min(n, cap), cudaMemcpyDeviceToHost));
    return LC_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void lc_default_params(lc_cloth_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    // Managers/MastersSimulationManager.cpp:33-62
    p->timestep = 1000.f / 60.f / 1000.f;  // Core/Utils.hpp:18-19
    p->kFriction = 0.1f;
    p->kStretch = 0.99f;
    p->kShear = 0.7f;
    p->kBend = 0.1f;
    p->kDamp = 0.05f;
    p->kSpringDamp = 0.2f;
    p->thickness = 0.f;
    p->objectMass = 0.525f;
    p->globalVelDamp = 0.01f;
    p->strainLimit = 0.15f;
    p->gravity[0] = 0.f; p->gravity[1] = -0.0981f; p->gravity[2] = 0.f;
    p->minWindDir[0] = -0.04f; p->minWindDir[1] = -0.1f; p->minWindDir[2] = -0.1f;
    p->startWindDir[0] = 0.02f; p->startWindDir[1] = 0.095f; p->startWindDir[2] = 0.45f;
    p->maxWindDir[0] = 0.04f; p->maxWindDir[1] = 0.135f; p->maxWindDir[2] = 0.4f;
    p->windMinVariation = 0.f;
    p->windMaxVariation = 0.2f;
    p->windOn = 1;
    p->worldMin[0] = p->worldMin[1] = p->worldMin[2] = 0.f;
    p->worldMax[0] = p->worldMax[1] = p->worldMax[2] = 1.f;
    p->dims[0] = p->dims[1] = 60;
    p->solverIterations = 6;
    p->ccdIterations = 5;
    p->BVHChunkSize = 64;
    p->benchmarkSample = 1000;
    p->useTriangleBending = 0;
    p->colorContacts = 0;
    p->useFriction = 0;
    p->thicknessFromMesh = 1;
    p->mortonMode = LC_MORTON_REF63;
    p->refLeafAabbQuirk = 1;
    p->groundOn = 1;
    p->mortonOrigin[0] = p->mortonOrigin[1] = p->mortonOrigin[2] = 0.f;
    p->mortonScale = 1.f;
    p->windSeed = 0;
    p->sphereOn = 0;
    p->sphereRadius = 0.f;
}

void lc_default_options(lc_batch_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->use_graph = 1;
}

const char *lc_last_error_string(void) { return g_last_error.c_str(); }

const char *lc_status_string(lc_status s) {
    switch (s) {
        case LC_OK: return "ok";
        case LC_ERR_INVALID_ARG: return "invalid argument";
        case LC_ERR_OOM: return "out of device memory";
        case LC_ERR_CAPACITY_OVERFLOW: return "contact capacity overflow";
        case LC_ERR_TIMEOUT: return "timeout";
        case LC_ERR_CUDA: return "CUDA error";
        case LC_ERR_NOT_SUPPORTED: return "not supported";
        case LC_ERR_STACK_OVERFLOW: return "BVH traversal stack overflow";
    }
    return "unknown";
}

uint64_t lc_morton3d(float x, float y, float z, int32_t mode) { return morton3_host(x, y, z, mode); }

// Rendering/VisualBodyFactory.cpp:343-391 — grid triangles (alternating
// diagonals); returns the triangle count, fills indices when non-NULL.
int32_t lc_mesh_grid(int32_t rows, int32_t cols, uint32_t *indices) {
    if (rows < 2 || cols < 2) return 0;
    int32_t t = 0;
    for (int i = 0; i < rows - 1; ++i)
        for (int j = 0; j < cols - 1; ++j) {
            uint32_t q[6];
            if ((i + j) % 2 == 0) {
                const uint32_t v[6] = {(uint32_t)(rows * i + j), (uint32_t)(rows * (i + 1) + j), (uint32_t)(rows * i + j + 1),
                                       (uint32_t)(rows * i + j + 1), (uint32_t)(rows * (i + 1) + j),
                                       (uint32_t)(rows * (i + 1) + j + 1)};
                std::memcpy(q, v, sizeof(q));
            } else {
                const uint32_t v[6] = {(uint32_t)(rows * i + j), (uint32_t)(rows * (i + 1) + j),
                                       (uint32_t)(rows * (i + 1) + j + 1), (uint32_t)(rows * (i + 1) + j + 1),
                                       (uint32_t)(rows * i + j + 1), (uint32_t)(rows * i + j)};
                std::memcpy(q, v, sizeof(q));
            }
            if (indices) std::memcpy(indices + 3 * t, q, sizeof(q));
            t += 2;
        }
    return t;
}

// Rendering/VisualBodyFactory.cpp:259-341 — icosphere by midpoint
// subdivision with unwelded vertices (6 per parent triangle per level).
// Returns the triangle count; fills verts (3 per vertex, 18 * T / 4 floats)
// and indices when non-NULL.
int32_t lc_mesh_icosphere(int32_t depth, float *verts, uint32_t *indices) {
    if (depth < 1 || depth > 8) return 0;
    const float X = .525731112119133606f, Z = .850650808352039932f;
    std::vector<float3> v = {f3(-X, 0, Z), f3(X, 0, Z), f3(-X, 0, -Z), f3(X, 0, -Z), f3(0, Z, X), f3(0, Z, -X),
                             f3(0, -Z, X), f3(0, -Z, -X), f3(Z, X, 0), f3(-Z, X, 0), f3(Z, -X, 0), f3(-Z, -X, 0)};
    std::vector<uint32_t> id = {0, 4, 1, 0, 9, 4, 9, 5, 4, 4, 5, 8, 4, 8, 1, 8, 10, 1, 8, 3, 10, 5, 3, 8, 5, 2, 3, 2, 7, 3,
                                7, 10, 3, 7, 6, 10, 7, 11, 6, 11, 0, 6, 0, 1, 6, 6, 1, 10, 9, 0, 11, 9, 11, 2, 9, 2, 5, 7, 2, 11};
    auto nrm = [](float3 a) {
        const float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
        return f3(a.x / l, a.y / l, a.z / l);
    };
    for (int lvl = 0; lvl < depth; ++lvl) {
        std::vector<float3> nv;
        std::vector<uint32_t> ni;
        nv.reserve(id.size() * 2);
        ni.reserve(id.size() * 4);
        for (size_t j = 0; j < id.size(); j += 3) {
            const float3 a = v[id[j]], b = v[id[j + 1]], c = v[id[j + 2]];
            const float3 ab = nrm(add(a, b)), bc = nrm(add(b, c)), ca = nrm(add(c, a));
            const uint32_t base = (uint32_t)nv.size();
            nv.push_back(a); nv.push_back(b); nv.push_back(c);
            nv.push_back(ab); nv.push_back(bc); nv.push_back(ca);
            const uint32_t t[12] = {base, base + 3, base + 5, base + 1, base + 4, base + 3,
                                    base + 2, base + 5, base + 4, base + 3, base + 4, base + 5};
            ni.insert(ni.end(), t, t + 12);
        }
        v.swap(nv);
        id.swap(ni);
    }
    if (verts)
        for (size_t i = 0; i < v.size(); ++i) { verts[3 * i] = v[i].x; verts[3 * i + 1] = v[i].y; verts[3 * i + 2] = v[i].z; }
    if (indices) std::memcpy(indices, id.data(), id.size() * sizeof(uint32_t));
    return (int32_t)(id.size() / 3);
}

lc_status lc_batch_create(const lc_cloth_desc *descs, int32_t num_cloths, const lc_batch_options *opts,
                          lc_batch **out) {
    if (!descs || num_cloths <= 0 || !out) return fail(LC_ERR_INVALID_ARG, "lc_batch_create: bad arguments");
    *out = nullptr;
    lc_batch_options o;
    lc_default_options(&o);
    if (opts) o = *opts;
    std::unique_ptr<lc_batch> b(new lc_batch());
    lc_status s = batch_build(b.get(), descs, num_cloths, o);
    if (s != LC_OK) return s;
    *out = b.release();
    return LC_OK;
}

lc_status lc_batch_destroy(lc_batch *b) {
    if (b) {
        cudaDeviceSynchronize();
        delete b;
    }
    return LC_OK;
}

lc_status lc_batch_step(lc_batch *b, int32_t nsteps, void *stream) {
    if (!b || nsteps < 0) return fail(LC_ERR_INVALID_ARG, "lc_batch_step: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    b->last_stream = st;
    if (!b->opt.use_graph || b->opt.debug_capture) {
        for (int s = 0; s < nsteps; ++s) LC_TRY(b->enqueue_step(st));
        return LC_OK;
    }
    if (!b->gexec) {
        LC_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
        lc_status s = b->enqueue_step(b->cap_stream);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
        if (s != LC_OK) { if (g) cudaGraphDestroy(g); return s; }
        LC_CUDA(e);
        b->graph = g;
        LC_CUDA(cudaGraphInstantiate(&b->gexec, g, 0));
    }
    for (int s = 0; s < nsteps; ++s) LC_CUDA(cudaGraphLaunch(b->gexec, st));
    return LC_OK;
}

// ----- concurrent batches ----------------------------------------------------
struct lc_group {
    std::vector<lc_batch *> b;
    std::vector<cudaStream_t> lane;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
};

lc_status lc_group_destroy(lc_group *g) {
    if (!g) return LC_OK;
    for (size_t i = 0; i < g->lane.size(); ++i) {
        if (g->lane[i]) cudaStreamSynchronize(g->lane[i]);
        for (lc_batch *b : g->b)
            if (b->last_stream == g->lane[i]) b->last_stream = nullptr;
        if (g->lane[i]) cudaStreamDestroy(g->lane[i]);
    }
    for (cudaEvent_t e : g->join)
        if (e) cudaEventDestroy(e);
    if (g->fork) cudaEventDestroy(g->fork);
    delete g;
    return LC_OK;
}

lc_status lc_group_create(lc_batch *const *batches, int32_t count, lc_group **out) {
    if (!batches || count < 1 || !out) return fail(LC_ERR_INVALID_ARG, "lc_group_create: bad arguments");
    *out = nullptr;
    for (int i = 0; i < count; ++i) {
        if (!batches[i]) return fail(LC_ERR_INVALID_ARG, "lc_group_create: null batch");
        for (int j = 0; j < i; ++j)
            if (batches[j] == batches[i]) return fail(LC_ERR_INVALID_ARG, "lc_group_create: a batch appears twice");
    }
    lc_group *g = new lc_group();
    g->b.assign(batches, batches + count);
    g->lane.assign(count, nullptr);
    g->join.assign(count, nullptr);
    cudaError_t e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
    for (int i = 0; i < count && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&g->lane[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        lc_group_destroy(g);
        return fail(LC_ERR_CUDA, std::string("lc_group_create: ") + cudaGetErrorString(e));
    }
    *out = g;
    return LC_OK;
}

lc_status lc_group_step(lc_group *g, int32_t nsteps, void *stream) {
    if (!g || nsteps < 0) return fail(LC_ERR_INVALID_ARG, "lc_group_step: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    LC_CUDA(cudaEventRecord(g->fork, st));
    const size_t n = g->b.size();
    for (size_t i = 0; i < n; ++i) LC_CUDA(cudaStreamWaitEvent(g->lane[i], g->fork, 0));
    lc_status s = LC_OK;
    for (int k = 0; k < nsteps && s == LC_OK; ++k)
        for (size_t i = 0; i < n && s == LC_OK; ++i) s = lc_batch_step(g->b[i], 1, g->lane[i]);
    // join what was enqueued, also after a failure
    for (size_t i = 0; i < n; ++i) {
        LC_CUDA(cudaEventRecord(g->join[i], g->lane[i]));
        LC_CUDA(cudaStreamWaitEvent(st, g->join[i], 0));
        g->b[i]->last_stream = st;
    }
    return s;
}

lc_status lc_group_step_io(lc_group *g, int32_t nsteps, const float *x_in, const float *xp_in, const float *v_in,
                           float *x_out, float *xp_out, float *v_out, int32_t is_host, void *stream) {
    if (!g || nsteps < 0) return fail(LC_ERR_INVALID_ARG, "lc_group_step_io: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    LC_CUDA(cudaEventRecord(g->fork, st));
    const size_t n = g->b.size();
    for (size_t i = 0; i < n; ++i) LC_CUDA(cudaStreamWaitEvent(g->lane[i], g->fork, 0));
    lc_status s = LC_OK;
    for (int k = 0; k < nsteps && s == LC_OK; ++k) {
        size_t off = 0;  // floats before this batch's slice
        for (size_t i = 0; i < n && s == LC_OK; ++i) {
            lc_batch *b = g->b[i];
            cudaStream_t ls = g->lane[i];
            auto in = [&](const float *p) { return p ? p + off : nullptr; };
            auto out = [&](float *p) { return p ? p + off : nullptr; };
            s = lc_batch_write_state(b, in(x_in), in(xp_in), in(v_in), is_host, ls);
            if (s == LC_OK) s = lc_batch_step(b, 1, ls);
            if (s == LC_OK) s = lc_batch_read_state(b, out(x_out), out(xp_out), out(v_out), is_host, ls);
            off += 3 * (size_t)b->d.Vtot;
        }
    }
    // join what was enqueued, also after a failure
    for (size_t i = 0; i < n; ++i) {
        LC_CUDA(cudaEventRecord(g->join[i], g->lane[i]));
        LC_CUDA(cudaStreamWaitEvent(st, g->join[i], 0));
        g->b[i]->last_stream = st;
    }
    return s;
}

lc_status lc_batch_sync(lc_batch *b) {
    if (!b) return fail(LC_ERR_INVALID_ARG, "lc_batch_sync: null batch");
    LC_CUDA(cudaStreamSynchronize(b->last_stream));
    LC_CUDA(cudaDeviceSynchronize());
    uint32_t err = 0;
    LC_CUDA(cudaMemcpy(&err, b->d.err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err & (ERR_VF_OVERFLOW | ERR_EE_OVERFLOW | ERR_DYN_OVERFLOW | ERR_CAND_OVERFLOW | ERR_COLL_OVERFLOW)) {
        cudaMemset(b->d.err, 0, sizeof(uint32_t));
        return fail(LC_ERR_CAPACITY_OVERFLOW,
                    (err & ERR_CAND_OVERFLOW)   ? "narrowphase candidate capacity exceeded; raise lc_batch_options.cand_capacity"
                    : (err & ERR_COLL_OVERFLOW) ? "more static-collider contacts at a vertex than LC_COLLIDER_SLOTS"
                                                : "contact capacity exceeded; raise lc_batch_options.vf/ee_capacity");
    }
    if (err & ERR_STACK) {
        cudaMemset(b->d.err, 0, sizeof(uint32_t));
        return fail(LC_ERR_STACK_OVERFLOW, "BVH traversal stack (64) exceeded");
    }
    if (err & ERR_SORT) {
        cudaMemset(b->d.err, 0, sizeof(uint32_t));
        return fail(LC_ERR_TIMEOUT, "sort look-back wait exceeded its bound");
    }
    return LC_OK;
}

lc_status lc_batch_num_cloths(const lc_batch *b, int32_t *out) {
    if (!b || !out) return fail(LC_ERR_INVALID_ARG, "null argument");
    *out = b->C;
    return LC_OK;
}

lc_status lc_batch_cloth_sizes(const lc_batch *b, int32_t c, int32_t *nv, int32_t *nt) {
    if (!b || c < 0 || c >= b->C) return fail(LC_ERR_INVALID_ARG, "bad cloth index");
    if (nv) *nv = b->hosts[c].V;
    if (nt) *nt = b->hosts[c].T;
    return LC_OK;
}

// Launch shapes (results do not depend on them, except solver_variant which
// picks a different summation of the Jacobi corrections).
lc_status lc_batch_get_tuning(const lc_batch *b, lc_tuning *t) {
    if (!b || !t) return fail(LC_ERR_INVALID_ARG, "lc_batch_get_tuning: bad arguments");
    t->traverse_block = b->traverse_block;
    t->jacobi_block = b->jacobi_block;
    t->narrow_blocks_per_sm = b->narrow_grid / sm_count();
    t->solver_variant = b->use_cluster ? (b->cluster_scatter ? 3 : 2) : 1;
    t->cluster_size = b->use_cluster ? b->cluster_cs : 0;
    t->contact_gather = b->ca.contact_gather;
    return LC_OK;
}

lc_status lc_batch_set_tuning(lc_batch *b, const lc_tuning *t) {
    if (!b || !t) return fail(LC_ERR_INVALID_ARG, "lc_batch_set_tuning: bad arguments");
    auto ok_block = [](int v) { return v >= 32 && v <= 1024 && v % 32 == 0; };
    if (!ok_block(t->traverse_block) || t->traverse_block > kTraverseBlockMax || !ok_block(t->jacobi_block) ||
        t->narrow_blocks_per_sm < 1 ||
        t->narrow_blocks_per_sm > 64 || t->solver_variant < 1 || t->solver_variant > 3 ||
        (t->cluster_size != 0 && t->cluster_size != 4 && t->cluster_size != 8 && t->cluster_size != 16) ||
        t->contact_gather < 0 || t->contact_gather > 1)
        return fail(LC_ERR_INVALID_ARG, "lc_batch_set_tuning: value out of range");
    LC_CUDA(cudaDeviceSynchronize());
    b->traverse_block = t->traverse_block;
    b->jacobi_block = t->jacobi_block;
    if (b->ca.contact_gather != t->contact_gather) b->invalidate_graph();
    b->ca.contact_gather = t->contact_gather;
    b->narrow_grid = sm_count() * t->narrow_blocks_per_sm;
    const int prev = b->opt.solver_variant, prev_cs = b->want_cs;
    b->opt.solver_variant = t->solver_variant;
    b->want_cs = t->cluster_size;
    lc_status s = b->setup_cluster();
    if (s == LC_OK && t->solver_variant >= 2 && t->cluster_size && b->cluster_cs != t->cluster_size)
        s = fail(LC_ERR_NOT_SUPPORTED, "lc_batch_set_tuning: cluster size does not fit");
    if (s != LC_OK) {
        b->opt.solver_variant = prev;
        b->want_cs = prev_cs;
        b->setup_cluster();
        return s;
    }
    b->invalidate_graph();
    return LC_OK;
}

void lc_default_autotune_space(lc_autotune_space *s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    const int32_t tb[] = {64, 128, 256}, jb[] = {128, 256, 512}, nb[] = {4, 8, 16}, sv[] = {1, 2, 3},
                  cs[] = {4, 8, 16}, cg[] = {0, 1};
    std::memcpy(s->traverse_block, tb, sizeof(tb)); s->n_traverse_block = 3;
    std::memcpy(s->jacobi_block, jb, sizeof(jb)); s->n_jacobi_block = 3;
    std::memcpy(s->narrow_blocks_per_sm, nb, sizeof(nb)); s->n_narrow_blocks_per_sm = 3;
    std::memcpy(s->solver_variant, sv, sizeof(sv)); s->n_solver_variant = 3;
    std::memcpy(s->cluster_size, cs, sizeof(cs)); s->n_cluster_size = 3;
    std::memcpy(s->contact_gather, cg, sizeof(cg)); s->n_contact_gather = 2;
}

lc_status lc_batch_autotune(lc_batch *b, const lc_autotune_space *space_in, int32_t steps, int32_t warmup,
                            int32_t allow_variants, void *stream, lc_tuning *best, float *best_ms,
                            lc_autotune_trial *trials, int32_t trials_cap, int32_t *num_trials) {
    if (!b || steps < 1 || warmup < 0 || trials_cap < 0 || (trials_cap && !trials))
        return fail(LC_ERR_INVALID_ARG, "lc_batch_autotune: bad arguments");
    lc_autotune_space sp;
    if (space_in) sp = *space_in; else lc_default_autotune_space(&sp);
    const int32_t counts[6] = {sp.n_traverse_block, sp.n_jacobi_block, sp.n_narrow_blocks_per_sm,
                               sp.n_solver_variant, sp.n_cluster_size, sp.n_contact_gather};
    const int32_t caps[6] = {8, 8, 8, 3, 4, 2};
    for (int k = 0; k < 6; ++k)
        if (counts[k] < 1 || counts[k] > caps[k])
            return fail(LC_ERR_INVALID_ARG, "lc_batch_autotune: every space list needs 1..its capacity values");
    cudaStream_t st = (cudaStream_t)stream;
    lc_tuning original;
    LC_TRY(lc_batch_get_tuning(b, &original));
    if (!allow_variants) { sp.solver_variant[0] = original.solver_variant; sp.n_solver_variant = 1; }
    uint64_t nbytes = 0;
    LC_TRY(lc_batch_state_size(b, &nbytes));
    void *state = nullptr;
    if (cudaMalloc(&state, nbytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(LC_ERR_OOM, "lc_batch_autotune: no room for the saved state");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    struct Guard {
        void *p; cudaEvent_t a, b;
        ~Guard() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); if (p) cudaFree(p); }
    } guard{state, nullptr, nullptr};
    LC_CUDA(cudaEventCreate(&e0)); guard.a = e0;
    LC_CUDA(cudaEventCreate(&e1)); guard.b = e1;
    LC_TRY(lc_batch_sync(b));
    LC_TRY(lc_batch_save_state(b, state, st));
    int32_t n = 0;
    float best_t = 0.f;
    lc_tuning best_cfg = original;
    for (int i0 = 0; i0 < sp.n_traverse_block; ++i0)
    for (int i1 = 0; i1 < sp.n_jacobi_block; ++i1)
    for (int i2 = 0; i2 < sp.n_narrow_blocks_per_sm; ++i2)
    for (int i3 = 0; i3 < sp.n_solver_variant; ++i3)
    for (int i4 = 0; i4 < sp.n_cluster_size; ++i4)
    for (int i5 = 0; i5 < sp.n_contact_gather; ++i5) {
        lc_tuning c;
        c.traverse_block = sp.traverse_block[i0];
        c.jacobi_block = sp.jacobi_block[i1];
        c.narrow_blocks_per_sm = sp.narrow_blocks_per_sm[i2];
        c.solver_variant = sp.solver_variant[i3];
        c.cluster_size = sp.cluster_size[i4];
        c.contact_gather = sp.contact_gather[i5];
        // the Jacobi block matters only to the global-memory solver, the
        // cluster size only to the on-chip ones, the contact mode only to the
        // scatter solver: other combinations would time the same launch twice
        if (c.solver_variant != 1 && i1 != 0) continue;
        if (c.solver_variant == 1 && i4 != 0) continue;
        if (c.solver_variant == 1) c.cluster_size = 0;
        if (c.solver_variant != 3 && i5 != 0) continue;
        if (c.solver_variant != 3) c.contact_gather = 0;
        if (lc_batch_set_tuning(b, &c) != LC_OK) continue;  // a shape the batch cannot take
        LC_TRY(lc_batch_load_state(b, state, st));
        LC_TRY(lc_batch_step(b, warmup, st));
        LC_CUDA(cudaEventRecord(e0, st));
        LC_TRY(lc_batch_step(b, steps, st));
        LC_CUDA(cudaEventRecord(e1, st));
        LC_CUDA(cudaEventSynchronize(e1));
        LC_TRY(lc_batch_sync(b));
        float ms = 0.f;
        LC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= (float)steps;
        if (n < trials_cap) { trials[n].config = c; trials[n].ms_per_step = ms; }
        if (n == 0 || ms < best_t) { best_t = ms; best_cfg = c; }
        ++n;
    }
    LC_TRY(lc_batch_set_tuning(b, &best_cfg));
    LC_TRY(lc_batch_load_state(b, state, st));
    LC_CUDA(cudaStreamSynchronize(st));
    if (best) *best = best_cfg;
    if (best_ms) *best_ms = n ? best_t : -1.f;
    if (num_trials) *num_trials = n;
    if (!n) return fail(LC_ERR_NOT_SUPPORTED, "lc_batch_autotune: the batch took none of the shapes");
    return LC_OK;
}

lc_status lc_batch_constraint_counts(const lc_batch *b, int32_t c, int32_t *ns, int32_t *nb) {
    if (!b || c < 0 || c >= b->C) return fail(LC_ERR_INVALID_ARG, "bad cloth index");
    if (ns) *ns = b->s_count[c];
    if (nb) *nb = b->b_count[c];
    return LC_OK;
}

// Packed xyz (12 B per vertex) from / to n float4 state entries, on stream
// st.  A host transfer is one contiguous copy through the batch's staging
// buffer plus a (un)packing kernel: a strided copy of 12 of every 16 bytes
// moves only a few GB/s through the copy engines.  The staging buffer is the
// batch's own, so copies of one batch are ordered on one stream at a time.
static lc_status take_xyz(lc_batch *b, float *dst, const float4 *src, int n, int is_host, cudaStream_t st) {
    if (!dst) return LC_OK;
    launch_xyz_pack(src, is_host ? b->io : dst, n, st);
    if (is_host) LC_CUDA(cudaMemcpyAsync(dst, b->io, 3 * sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, st));
    return LC_OK;
}
static lc_status put_xyz(lc_batch *b, float4 *dst, const float *src, int n, int is_host, cudaStream_t st) {
    if (!src) return LC_OK;
    if (is_host) LC_CUDA(cudaMemcpyAsync(b->io, src, 3 * sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, st));
    launch_xyz_unpack(is_host ? b->io : src, dst, n, st);
    return LC_OK;
}
static lc_status get3(lc_batch *b, const float4 *src, int n, float *dst, int is_host) {
    LC_TRY(take_xyz(b, dst, src, n, is_host, 0));
    LC_CUDA(cudaStreamSynchronize(0));
    return LC_OK;
}
static lc_status set3(lc_batch *b, float4 *dst, int n, const float *src, int is_host) {
    LC_TRY(put_xyz(b, dst, src, n, is_host, 0));
    LC_CUDA(cudaStreamSynchronize(0));
    return LC_OK;
}

lc_status lc_batch_get_state(lc_batch *b, int32_t c, float *x, float *xp, float *v, float *vn, int32_t is_host) {
    if (!b || c < 0 || c >= b->C) return fail(LC_ERR_INVALID_ARG, "bad cloth index");
    LC_TRY(lc_batch_sync(b));
    const ClothDev &cd = b->cds[c];
    LC_TRY(get3(b, b->d.x + cd.v_off, cd.V, x, is_host));
    LC_TRY(get3(b, b->d.xp + cd.v_off, cd.V, xp, is_host));
    LC_TRY(get3(b, b->d.v + cd.v_off, cd.V, v, is_host));
    LC_TRY(get3(b, b->d.vn + cd.v_off, cd.V, vn, is_host));
    return LC_OK;
}

lc_status lc_batch_set_state(lc_batch *b, int32_t c, const float *x, const float *xp, const float *v, const float *vn,
                             int32_t is_host) {
    if (!b || c < 0 || c >= b->C) return fail(LC_ERR_INVALID_ARG, "bad cloth index");
    LC_CUDA(cudaDeviceSynchronize());
    const ClothDev &cd = b->cds[c];
    LC_TRY(set3(b, b->d.x + cd.v_off, cd.V, x, is_host));
    LC_TRY(set3(b, b->d.xp + cd.v_off, cd.V, xp, is_host));
    LC_TRY(set3(b, b->d.v + cd.v_off, cd.V, v, is_host));
    LC_TRY(set3(b, b->d.vn + cd.v_off, cd.V, vn, is_host));
    return LC_OK;
}

lc_status lc_batch_get_triangle_order(lc_batch *b, int32_t c, uint32_t *perm) {
    if (!b || c < 0 || c >= b->C || !perm) return fail(LC_ERR_INVALID_ARG, "bad arguments");
    LC_TRY(lc_batch_sync(b));
    const ClothDev &cd = b->cds[c];
    std::vector<uint32_t> tmp(cd.T);
    LC_CUDA(cudaMemcpy(tmp.data(), b->d.perm + cd.t_off, sizeof(uint32_t) * cd.T, cudaMemcpyDeviceToHost));
    for (int i = 0; i < cd.T; ++i) perm[i] = tmp[i] - (uint32_t)cd.t_off;
    return LC_OK;
}

lc_status lc_batch_set_triangle_order(lc_batch *b, int32_t c, const uint32_t *perm) {
    if (!b || c < 0 || c >= b->C || !perm) return fail(LC_ERR_INVALID_ARG, "bad arguments");
    const ClothDev &cd = b->cds[c];
    std::vector<uint32_t> tmp(cd.T);
    std::vector<char> seen(cd.T, 0);
    for (int i = 0; i < cd.T; ++i) {
        if (perm[i] >= (uint32_t)cd.T || seen[perm[i]]) return fail(LC_ERR_INVALID_ARG, "not a permutation");
        seen[perm[i]] = 1;
        tmp[i] = perm[i] + (uint32_t)cd.t_off;
    }
    LC_CUDA(cudaDeviceSynchronize());
    LC_CUDA(cudaMemcpy(b->d.perm + cd.t_off, tmp.data(), sizeof(uint32_t) * cd.T, cudaMemcpyHostToDevice));
    return LC_OK;
}

lc_status lc_batch_read_positions(lc_batch *b, float *dst, int32_t is_host, void *stream) {
    if (!b || !dst) return fail(LC_ERR_INVALID_ARG, "bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    LC_TRY(take_xyz(b, dst, b->d.xp, b->d.Vtot, is_host, st));
    LC_CUDA(cudaGetLastError());
    return LC_OK;
}

lc_status lc_batch_write_vertex_records(lc_batch *b, void *dst, int64_t stride, int32_t pos_offset,
                                        int32_t normal_offset, void *stream) {
    if (!b || !dst) return fail(LC_ERR_INVALID_ARG, "lc_batch_write_vertex_records: bad arguments");
    if (stride < 12 || stride % 4 || pos_offset < 0 || normal_offset < 0 || pos_offset % 4 || normal_offset % 4 ||
        pos_offset + 12 > stride || normal_offset + 12 > stride ||
        (pos_offset < normal_offset + 12 && normal_offset < pos_offset + 12) ||
        reinterpret_cast<uintptr_t>(dst) % 4)
        return fail(LC_ERR_INVALID_ARG, "lc_batch_write_vertex_records: stride / offsets / alignment");
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, dst) != cudaSuccess ||
        (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
        cudaGetLastError();
        return fail(LC_ERR_INVALID_ARG, "lc_batch_write_vertex_records: dst must be device memory");
    }
    launch_vertex_records(b->d, dst, stride, pos_offset, normal_offset, (cudaStream_t)stream);
    LC_CUDA(cudaGetLastError());
    return LC_OK;
}

lc_status lc_batch_set_sphere(lc_batch *b, int32_t c, const float pos[3], float radius) {
    if (!b || c < 0 || c >= b->C || !pos) return fail(LC_ERR_INVALID_ARG, "bad arguments");
    ClothDev &cd = b->cds[c];
    for (int k = 0; k < 3; ++k) cd.sphere_pos[k] = pos[k];
    cd.sphere_r = radius;
    const bool newly = !cd.sphere_on;
    cd.sphere_on = 1;
    b->hosts[c].p.sphereOn = 1;
    LC_CUDA(cudaDeviceSynchronize());
    LC_CUDA(cudaMemcpy(b->cloth_dev + c, &cd, sizeof(ClothDev), cudaMemcpyHostToDevice));
    if (newly && !b->any_sphere) {
        b->any_sphere = true;
        b->invalidate_graph();
    }
    return LC_OK;
}

extern "C++" {
// A median-split BVH over one collider's triangles, appended to the flat node
// arrays: leaves hold one triangle each with the triangle's box (the query
// inflates the vertex's box instead), internal nodes the union of their
// children's boxes.  Returns the root's index.
static int build_collider_node(const std::vector<float3> &bmin, const std::vector<float3> &bmax,
                               const std::vector<float3> &cen, std::vector<int> &idx, int b, int e, int tri_base,
                               std::vector<float4> &nmin, std::vector<float4> &nmax, std::vector<int2> &child) {
    const int node = (int)nmin.size();
    nmin.emplace_back();
    nmax.emplace_back();
    child.emplace_back();
    if (e - b == 1) {
        const int t = idx[b];
        nmin[node] = f4(bmin[t], 0.f);
        nmax[node] = f4(bmax[t], 0.f);
        child[node] = make_int2(-(tri_base + t) - 1, -1);
        return node;
    }
    float3 lo = cen[idx[b]], hi = lo;
    for (int k = b + 1; k < e; ++k) { lo = vmin(lo, cen[idx[k]]); hi = vmax(hi, cen[idx[k]]); }
    const float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = hi.z - lo.z;
    const int axis = ex >= ey && ex >= ez ? 0 : (ey >= ez ? 1 : 2);
    const int mid = (b + e) / 2;
    auto key = [&](int t) { return axis == 0 ? cen[t].x : (axis == 1 ? cen[t].y : cen[t].z); };
    std::nth_element(idx.begin() + b, idx.begin() + mid, idx.begin() + e,
                     [&](int p, int q) { return key(p) < key(q) || (key(p) == key(q) && p < q); });
    const int l = build_collider_node(bmin, bmax, cen, idx, b, mid, tri_base, nmin, nmax, child);
    const int r = build_collider_node(bmin, bmax, cen, idx, mid, e, tri_base, nmin, nmax, child);
    nmin[node] = f4(vmin(xyz(nmin[l]), xyz(nmin[r])), 0.f);
    nmax[node] = f4(vmax(xyz(nmax[l]), xyz(nmax[r])), 0.f);
    child[node] = make_int2(l, r);
    return node;
}

// A host vector in a fresh device array whose pointer `owner` keeps.
template <class T>
static lc_status upload_owned(std::vector<void *> &owner, const std::vector<T> &vec, const T *&dst) {
    void *q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(vec.size(), 1)) != cudaSuccess) {
        cudaGetLastError();
        return fail(LC_ERR_OOM, "lc_batch_set_collider: cudaMalloc failed");
    }
    owner.push_back(q);
    if (!vec.empty()) LC_CUDA(cudaMemcpy(q, vec.data(), sizeof(T) * vec.size(), cudaMemcpyHostToDevice));
    dst = static_cast<const T *>(q);
    return LC_OK;
}
}  // extern "C++"

lc_status lc_batch_set_collider(lc_batch *b, int32_t c, const float *vertices, int32_t num_vertices,
                                const uint32_t *indices, int32_t num_triangles, int32_t winding) {
    if (!b || c < 0 || c >= b->C || num_vertices < 0 || num_triangles < 0 ||
        (winding != LC_WINDING_CCW && winding != LC_WINDING_CW) ||
        (num_triangles > 0 && (!vertices || !indices || num_vertices < 3)))
        return fail(LC_ERR_INVALID_ARG, "lc_batch_set_collider: bad arguments");
    for (int64_t k = 0; k < 3 * (int64_t)num_triangles; ++k)
        if (indices[k] >= (uint32_t)num_vertices)
            return fail(LC_ERR_INVALID_ARG, "lc_batch_set_collider: index out of range");
    LC_CUDA(cudaDeviceSynchronize());
    if (b->colliders.empty()) b->colliders.resize(b->C);
    b->colliders[c].verts.assign(vertices, vertices + 3 * (size_t)(num_triangles ? num_vertices : 0));
    b->colliders[c].tris.assign(indices, indices + 3 * (size_t)num_triangles);
    b->colliders[c].cw = winding == LC_WINDING_CW;
    // every cloth's collider into flat arrays, one BVH per cloth
    std::vector<float4> cv, nmin, nmax;
    std::vector<int4> ct;
    std::vector<int2> child;
    bool any = false;
    for (int k = 0; k < b->C; ++k) {
        ClothDev &cd = b->cds[k];
        lc_batch::Collider &col = b->colliders[k];
        const int T = (int)(col.tris.size() / 3);
        cd.coll_cw = col.cw ? 1 : 0;
        if (!T) { cd.coll_root = -1; continue; }
        any = true;
        const int vbase = (int)cv.size(), tbase = (int)ct.size();
        col.tbase = tbase;
        const int NV = (int)(col.verts.size() / 3);
        for (int v = 0; v < NV; ++v)
            cv.push_back(make_float4(col.verts[3 * v], col.verts[3 * v + 1], col.verts[3 * v + 2], 0.f));
        std::vector<float3> bmin(T), bmax(T), cen(T);
        for (int t = 0; t < T; ++t) {
            const uint32_t *q = &col.tris[3 * (size_t)t];
            ct.push_back(make_int4(vbase + (int)q[0], vbase + (int)q[1], vbase + (int)q[2], k));
            const float3 p0 = xyz(cv[vbase + q[0]]), p1 = xyz(cv[vbase + q[1]]), p2 = xyz(cv[vbase + q[2]]);
            bmin[t] = min3(p0, p1, p2);
            bmax[t] = max3(p0, p1, p2);
            cen[t] = f3((bmin[t].x + bmax[t].x) * 0.5f, (bmin[t].y + bmax[t].y) * 0.5f, (bmin[t].z + bmax[t].z) * 0.5f);
        }
        std::vector<int> idx(T);
        std::iota(idx.begin(), idx.end(), 0);
        cd.coll_root = build_collider_node(bmin, bmax, cen, idx, 0, T, tbase, nmin, nmax, child);
    }
    b->free_collider_arrays();
    DevPtrs &d = b->d;
    d.cv = nullptr; d.ct = nullptr; d.cnmin = d.cnmax = nullptr; d.cnchild = nullptr; d.cface_geo = nullptr;
    if (any) {
        LC_TRY(upload_owned(b->coll_mem, cv, d.cv));
        LC_TRY(upload_owned(b->coll_mem, ct, d.ct));
        LC_TRY(upload_owned(b->coll_mem, nmin, d.cnmin));
        LC_TRY(upload_owned(b->coll_mem, nmax, d.cnmax));
        LC_TRY(upload_owned(b->coll_mem, child, d.cnchild));
        {
            void *q = nullptr;
            if (cudaMalloc(&q, sizeof(float4) * 5 * ct.size()) != cudaSuccess) {
                cudaGetLastError();
                return fail(LC_ERR_OOM, "lc_batch_set_collider: cudaMalloc failed");
            }
            b->coll_mem.push_back(q);
            d.cface_geo = static_cast<float4 *>(q);
        }
        if (!b->coll_slots_cnt) {
            const size_t V = (size_t)d.Vtot;
            LC_TRY(b->arena.alloc(b->coll_slots_cnt, V, "collider counts"));
            LC_TRY(b->arena.alloc(b->coll_slots_face, V * kColliderSlots, "collider faces"));
            LC_TRY(b->arena.alloc(b->coll_slots_w, V * kColliderSlots, "collider planes"));
            LC_CUDA(cudaMemset(b->coll_slots_cnt, 0, sizeof(int) * V));
            if (b->opt.adjoint) {  // the reverse pass's record of the projections
                LC_TRY(b->arena.alloc(d.coll_act, (size_t)(b->max_iters + 1) * V, "collider projection masks"));
                LC_CUDA(cudaMemset(d.coll_act, 0, (size_t)(b->max_iters + 1) * V));
            }
        }
    }
    d.ccnt = b->coll_slots_cnt;
    d.cface = b->coll_slots_face;
    d.cw = b->coll_slots_w;
    d.any_collider = any ? 1 : 0;
    if (b->coll_slots_cnt && !any) LC_CUDA(cudaMemset(b->coll_slots_cnt, 0, sizeof(int) * (size_t)d.Vtot));
    LC_CUDA(cudaMemcpy(b->cloth_dev, b->cds.data(), sizeof(ClothDev) * b->cds.size(), cudaMemcpyHostToDevice));
    if (any) {  // the faces' planes and barycentric set-up, once (they read the windings just copied)
        launch_collider_faces(d, (int)ct.size(), nullptr);
        LC_CUDA(cudaDeviceSynchronize());
    }
    b->invalidate_graph();
    return LC_OK;
}

lc_status lc_batch_set_stiffness(lc_batch *b, int32_t c, const float *ks, const float *kb) {
    if (!b || c < 0 || c >= b->C) return fail(LC_ERR_INVALID_ARG, "bad cloth index");
    const HostCloth &hc = b->hosts[c];
    const double iters = (double)hc.p.solverIterations;
    LC_CUDA(cudaDeviceSynchronize());
    if (ks) {
        std::vector<float2> par(hc.s_ids.size());
        for (size_t k = 0; k < par.size(); ++k)
            par[k] = make_float2((float)hc.s_l0[k], (float)(1.0 - std::pow(1.0 - (double)ks[k], 1.0 / iters)));
        if (!par.empty())
            LC_CUDA(cudaMemcpy((void *)(b->d.s_par + b->e_off[c]), par.data(), sizeof(float2) * par.size(),
                               cudaMemcpyHostToDevice));
    }
    if (kb) {
        std::vector<float> kp(hc.b_ids.size());
        for (size_t k = 0; k < kp.size(); ++k) kp[k] = (float)(1.0 - std::pow(1.0 - (double)kb[k], 1.0 / iters));
        if (!kp.empty())
            LC_CUDA(cudaMemcpy((void *)(b->d.b_kp + b->b_off[c]), kp.data(), sizeof(float) * kp.size(),
                               cudaMemcpyHostToDevice));
    }
    return LC_OK;
}

// All stretch and bend stiffnesses of the batch in the global constraint
// order (cloth 0's constraints first), as lc_batch_set_stiffness converts them.
lc_status lc_batch_set_constraint_stiffness(lc_batch *b, const float *ks, const float *kb, int32_t is_host) {
    if (!b) return fail(LC_ERR_INVALID_ARG, "lc_batch_set_constraint_stiffness: null batch");
    std::vector<float> hs, hb;
    size_t E = 0, B = 0;
    for (int c = 0; c < b->C; ++c) { E += b->hosts[c].s_ids.size(); B += b->hosts[c].b_ids.size(); }
    LC_CUDA(cudaDeviceSynchronize());
    if (ks) {
        hs.resize(E);
        if (E) LC_CUDA(cudaMemcpy(hs.data(), ks, sizeof(float) * E, is_host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost));
    }
    if (kb) {
        hb.resize(B);
        if (B) LC_CUDA(cudaMemcpy(hb.data(), kb, sizeof(float) * B, is_host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost));
    }
    for (int c = 0; c < b->C; ++c)
        LC_TRY(lc_batch_set_stiffness(b, c, ks ? hs.data() + b->e_off[c] : nullptr, kb ? hb.data() + b->b_off[c] : nullptr));
    return LC_OK;
}

// Dynamic state of the batch (everything a later step reads from an earlier
// one): x, x_prev, v, running normals, the triangle order and the per-cloth
// wind state, packed into one device buffer.
static size_t al256(size_t n) { return (n + 255) & ~size_t(255); }
static void state_layout(const lc_batch *b, size_t off[6]) {
    const size_t V = (size_t)b->d.Vtot, T = (size_t)b->d.Ttot;
    off[0] = 0;
    off[1] = off[0] + al256(sizeof(float4) * V);
    off[2] = off[1] + al256(sizeof(float4) * V);
    off[3] = off[2] + al256(sizeof(float4) * V);
    off[4] = off[3] + al256(sizeof(float4) * V);
    off[5] = off[4] + al256(sizeof(uint32_t) * T);
}
lc_status lc_batch_state_size(const lc_batch *b, uint64_t *bytes) {
    if (!b || !bytes) return fail(LC_ERR_INVALID_ARG, "lc_batch_state_size: bad arguments");
    size_t off[6];
    state_layout(b, off);
    *bytes = off[5] + al256(sizeof(ClothState) * (size_t)b->C);
    return LC_OK;
}
lc_status lc_batch_save_state(lc_batch *b, void *dst, void *stream) {
    if (!b || !dst) return fail(LC_ERR_INVALID_ARG, "lc_batch_save_state: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t V = (size_t)b->d.Vtot, T = (size_t)b->d.Ttot;
    size_t off[6];
    state_layout(b, off);
    char *p = static_cast<char *>(dst);
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    LC_CUDA(cudaMemcpyAsync(p + off[0], b->d.x, sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(p + off[1], b->d.xp, sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(p + off[2], b->d.v, sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(p + off[3], b->d.vn, sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(p + off[4], b->d.perm, sizeof(uint32_t) * T, k, st));
    LC_CUDA(cudaMemcpyAsync(p + off[5], b->d.cstate, sizeof(ClothState) * (size_t)b->C, k, st));
    return LC_OK;
}
lc_status lc_batch_load_state(lc_batch *b, const void *src, void *stream) {
    if (!b || !src) return fail(LC_ERR_INVALID_ARG, "lc_batch_load_state: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t V = (size_t)b->d.Vtot, T = (size_t)b->d.Ttot;
    size_t off[6];
    state_layout(b, off);
    const char *p = static_cast<const char *>(src);
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    LC_CUDA(cudaMemcpyAsync(b->d.x, p + off[0], sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(b->d.xp, p + off[1], sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(b->d.v, p + off[2], sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(b->d.vn, p + off[3], sizeof(float4) * V, k, st));
    LC_CUDA(cudaMemcpyAsync(b->d.perm, p + off[4], sizeof(uint32_t) * T, k, st));
    LC_CUDA(cudaMemcpyAsync(b->d.cstate, p + off[5], sizeof(ClothState) * (size_t)b->C, k, st));
    return LC_OK;
}

// One step forward (recorded) and its reverse pass; exponent (may be null)
// selects the rescaled form.  See lc.h.
static lc_status adjoint_step(lc_batch *b, float *gx, float *gxp, float *gv, float *gk_stretch, float *gk_bend,
                              int32_t *exponent, void *stream, const char *who) {
    if (!b || !gx || !gxp || !gv) return fail(LC_ERR_INVALID_ARG, std::string(who) + ": bad arguments");
    if (!b->opt.adjoint) return fail(LC_ERR_INVALID_ARG, std::string(who) + ": batch created without the adjoint option");
    cudaStream_t st = (cudaStream_t)stream;
    b->last_stream = st;
    const int V = b->d.Vtot;
    // the recorded step, then its reverse pass, on stream s
    auto enqueue = [&](cudaStream_t s) -> lc_status {
        b->recording = true;
        const lc_status r = b->enqueue_step(s);
        b->recording = false;
        if (r != LC_OK) return r;
        uint32_t *flag = exponent ? b->adj_flag + (size_t)b->adj_flip * b->C : nullptr;
        launch_adj_unpack(b->adj, gx, gxp, gv, V, s);
        launch_adjoint(b->d, b->adj, b->adj_a, b->adj_g, b->nvf, b->nee, b->narrow_grid, b->nfixed, gk_stretch,
                       gk_bend, s);
        launch_adj_pack(b->d, b->adj, gx, gxp, gv, flag, V, s);
        if (exponent) {
            uint32_t *next = b->adj_flag + (size_t)(1 - b->adj_flip) * b->C;
            launch_adj_rescale(b->d, gx, gxp, gv, gk_stretch, gk_bend, flag, next, exponent, b->adj.E, b->adj.B, s);
        }
        LC_CUDA(cudaGetLastError());
        return LC_OK;
    };
    if (!b->opt.use_graph || b->opt.debug_capture) {
        LC_TRY(enqueue(st));
    } else {
        // about 130 short launches for a small cloth: replayed as one graph,
        // captured once per set of gradient buffers and rescale parity
        const uintptr_t key[7] = {(uintptr_t)gx, (uintptr_t)gxp, (uintptr_t)gv, (uintptr_t)gk_stretch,
                                  (uintptr_t)gk_bend, (uintptr_t)exponent, (uintptr_t)b->adj_flip};
        size_t k = 0;
        while (k < b->adj_graphs.size() && std::memcmp(b->adj_graphs[k].key, key, sizeof(key)) != 0) ++k;
        if (k == b->adj_graphs.size()) {
            LC_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
            const lc_status s = enqueue(b->cap_stream);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
            if (s != LC_OK) { if (g) cudaGraphDestroy(g); return s; }
            LC_CUDA(e);
            lc_batch::AdjGraph a{};
            std::memcpy(a.key, key, sizeof(key));
            a.g = g;
            if (cudaGraphInstantiate(&a.e, g, 0) != cudaSuccess) {
                cudaGraphDestroy(g);
                return fail(LC_ERR_CUDA, std::string(who) + ": graph instantiation failed");
            }
            if (b->adj_graphs.size() == 4) {
                cudaGraphExecDestroy(b->adj_graphs.back().e);
                cudaGraphDestroy(b->adj_graphs.back().g);
                b->adj_graphs.pop_back();
            }
            b->adj_graphs.insert(b->adj_graphs.begin(), a);
            k = 0;
        } else if (k) {
            std::rotate(b->adj_graphs.begin(), b->adj_graphs.begin() + k, b->adj_graphs.begin() + k + 1);
            k = 0;
        }
        LC_CUDA(cudaGraphLaunch(b->adj_graphs[k].e, st));
    }
    if (exponent) b->adj_flip = 1 - b->adj_flip;
    return LC_OK;
}

lc_status lc_batch_adjoint_step(lc_batch *b, float *gx, float *gxp, float *gv, float *gk_stretch, float *gk_bend,
                                void *stream) {
    return adjoint_step(b, gx, gxp, gv, gk_stretch, gk_bend, nullptr, stream, "lc_batch_adjoint_step");
}

lc_status lc_batch_adjoint_step_rescaled(lc_batch *b, float *gx, float *gxp, float *gv, float *gk_stretch,
                                         float *gk_bend, int32_t *exponent, void *stream) {
    if (!exponent) return fail(LC_ERR_INVALID_ARG, "lc_batch_adjoint_step_rescaled: exponent is null");
    return adjoint_step(b, gx, gxp, gv, gk_stretch, gk_bend, exponent, stream, "lc_batch_adjoint_step_rescaled");
}

lc_status lc_batch_counters(lc_batch *b, uint64_t out[4]) {
    if (!b || !out) return fail(LC_ERR_INVALID_ARG, "bad arguments");
    lc_status s = lc_batch_sync(b);
    unsigned long long t[4];
    LC_CUDA(cudaMemcpy(t, b->d.counters, sizeof(t), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 4; ++k) out[k] = t[k];
    return s;
}

lc_status lc_batch::cloth_contacts(int c, bool vf, std::vector<uint64_t> &gidx, std::vector<int4> &iv,
                                   std::vector<float4> &wv) {
    // a cloth's contacts of each kind are one contiguous range of the batch's
    // list (k_contact_ranges writes it every step)
    const ClothDev &cd = cds[c];
    uint4 cr;
    LC_CUDA(cudaMemcpy(&cr, d.crange + c, sizeof(uint4), cudaMemcpyDeviceToHost));
    const uint64_t a = vf ? cr.x : cr.z, e = vf ? cr.y : cr.w;
    const uint64_t n = e > a ? e - a : 0;
    std::vector<int4> v(n);
    std::vector<float4> w(n);
    if (n) {
        LC_CUDA(cudaMemcpy(v.data(), (vf ? d.vf_v : d.ee_v) + a, sizeof(int4) * n, cudaMemcpyDeviceToHost));
        LC_CUDA(cudaMemcpy(w.data(), (vf ? d.vf_w : d.ee_w) + a, sizeof(float4) * n, cudaMemcpyDeviceToHost));
    }
    gidx.resize(n); iv.resize(n); wv.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
        gidx[i] = a + i;
        iv[i] = make_int4(v[i].x - cd.v_off, v[i].y - cd.v_off, v[i].z - cd.v_off, v[i].w - cd.v_off);
        wv[i] = w[i];
    }
    return LC_OK;
}

lc_status lc_batch_debug_get(lc_batch *b, int32_t c, int32_t what, void *dst, uint64_t cap, uint64_t *count) {
    if (!b || c < 0 || c >= b->C) return fail(LC_ERR_INVALID_ARG, "bad cloth index");
    LC_TRY(lc_batch_sync(b));
    const ClothDev &cd = b->cds[c];
    const DevPtrs &d = b->d;
    const bool need_dbg = what == LC_DBG_PRED_X || what == LC_DBG_PRED_XPREV || what == LC_DBG_PRED_V ||
                          what == LC_DBG_PERM_BEFORE;
    if (need_dbg && !b->opt.debug_capture) return fail(LC_ERR_INVALID_ARG, "batch created without debug_capture");
    switch (what) {
        case LC_DBG_PRED_X: if (count) *count = cd.V; return get3(b, b->dbg_x + cd.v_off, (int)std::min<uint64_t>(cd.V, cap), (float *)dst, 1);
        case LC_DBG_PRED_XPREV: if (count) *count = cd.V; return get3(b, b->dbg_xp + cd.v_off, (int)std::min<uint64_t>(cd.V, cap), (float *)dst, 1);
        case LC_DBG_PRED_V: if (count) *count = cd.V; return get3(b, b->dbg_v + cd.v_off, (int)std::min<uint64_t>(cd.V, cap), (float *)dst, 1);
        case LC_DBG_PERM_BEFORE:
        case LC_DBG_PERM: {
            std::vector<uint32_t> t(cd.T);
            LC_CUDA(cudaMemcpy(t.data(), (what == LC_DBG_PERM ? d.perm : b->dbg_perm_before) + cd.t_off,
                               sizeof(uint32_t) * cd.T, cudaMemcpyDeviceToHost));
            for (auto &v : t) v -= (uint32_t)cd.t_off;
            if (count) *count = cd.T;
            if (dst) std::memcpy(dst, t.data(), sizeof(uint32_t) * std::min<uint64_t>(cd.T, cap));
            return LC_OK;
        }
        case LC_DBG_MORTON: return dump(d.keys + cd.t_off, (uint64_t)cd.T, dst, cap, count);
        case LC_DBG_LEFTS:
        case LC_DBG_RIGHTS: {
            std::vector<int2> t(std::max(cd.T - 1, 0));
            if (!t.empty())
                LC_CUDA(cudaMemcpy(t.data(), d.child + cd.i_off, sizeof(int2) * t.size(), cudaMemcpyDeviceToHost));
            if (count) *count = t.size();
            if (dst)
                for (size_t i = 0; i < std::min<uint64_t>(t.size(), cap); ++i)
                    ((int *)dst)[i] = what == LC_DBG_LEFTS ? t[i].x : t[i].y;
            return LC_OK;
        }
        case LC_DBG_PARENTS: return dump(d.parent + cd.n_off, (uint64_t)(2 * cd.T - 1), dst, cap, count);
        case LC_DBG_RML: return dump(d.rml + cd.i_off, (uint64_t)std::max(cd.T - 1, 0), dst, cap, count);
        case LC_DBG_NODE_AABB: {
            const uint64_t n = 2 * (uint64_t)cd.T - 1;
            std::vector<float4> mn(n), mx(n);
            LC_CUDA(cudaMemcpy(mn.data(), d.nmin + cd.n_off, sizeof(float4) * n, cudaMemcpyDeviceToHost));
            LC_CUDA(cudaMemcpy(mx.data(), d.nmax + cd.n_off, sizeof(float4) * n, cudaMemcpyDeviceToHost));
            if (count) *count = n;
            if (dst)
                for (uint64_t i = 0; i < std::min(n, cap); ++i) {
                    float *o = (float *)dst + 6 * i;
                    o[0] = mn[i].x; o[1] = mn[i].y; o[2] = mn[i].z; o[3] = mx[i].x; o[4] = mx[i].y; o[5] = mx[i].z;
                }
            return LC_OK;
        }
        case LC_DBG_PAIRS: {
            // pairs of this cloth: slots [t_off, t_off+T) own the range
            std::vector<uint32_t> off(cd.T + 1);
            LC_CUDA(cudaMemcpy(off.data(), d.pair_off + cd.t_off, sizeof(uint32_t) * (cd.T + 1), cudaMemcpyDeviceToHost));
            const uint64_t n = off[cd.T] - off[0];
            std::vector<uint2> t(n);
            if (n) LC_CUDA(cudaMemcpy(t.data(), d.pairs + off[0], sizeof(uint2) * n, cudaMemcpyDeviceToHost));
            if (count) *count = n;
            if (dst)
                for (uint64_t i = 0; i < std::min(n, cap); ++i) {
                    ((uint32_t *)dst)[2 * i] = t[i].x - cd.t_off;
                    ((uint32_t *)dst)[2 * i + 1] = t[i].y - cd.t_off;
                }
            return LC_OK;
        }
        case LC_DBG_VF:
        case LC_DBG_EE: {
            std::vector<uint64_t> gi;
            std::vector<int4> iv;
            std::vector<float4> wv;
            LC_TRY(b->cloth_contacts(c, what == LC_DBG_VF, gi, iv, wv));
            std::vector<lc_contact> outv(iv.size());
            for (size_t i = 0; i < iv.size(); ++i) {
                lc_contact &k = outv[i];
                k.v[0] = iv[i].x; k.v[1] = iv[i].y; k.v[2] = iv[i].z; k.v[3] = iv[i].w;
                k.w[0] = wv[i].x; k.w[1] = wv[i].y; k.w[2] = wv[i].z; k.w[3] = wv[i].w;
            }
            if (count) *count = outv.size();
            if (dst && !outv.empty()) std::memcpy(dst, outv.data(), sizeof(lc_contact) * std::min<uint64_t>(outv.size(), cap));
            return LC_OK;
        }
        case LC_DBG_COLLIDER: {
            const size_t K = kColliderSlots, n = (size_t)cd.V * K;
            std::vector<lc_contact> outv(n);
            for (size_t i = 0; i < n; ++i) {
                outv[i] = lc_contact{};
                outv[i].v[0] = (int)(i / K);
                outv[i].v[1] = -1;
            }
            if (d.any_collider && b->coll_slots_cnt) {
                std::vector<int> cnt(cd.V), face(n);
                std::vector<float4> w(n);
                LC_CUDA(cudaMemcpy(cnt.data(), d.ccnt + cd.v_off, sizeof(int) * cd.V, cudaMemcpyDeviceToHost));
                LC_CUDA(cudaMemcpy(face.data(), d.cface + (size_t)cd.v_off * K, sizeof(int) * n, cudaMemcpyDeviceToHost));
                LC_CUDA(cudaMemcpy(w.data(), d.cw + (size_t)cd.v_off * K, sizeof(float4) * n, cudaMemcpyDeviceToHost));
                const int tbase = b->colliders.empty() ? 0 : b->colliders[c].tbase;
                for (int v = 0; v < cd.V; ++v)
                    for (int k = 0; k < cnt[v] && k < (int)K; ++k) {
                        lc_contact &o = outv[(size_t)v * K + k];
                        o.v[1] = face[(size_t)v * K + k] - tbase;
                        const float4 q = w[(size_t)v * K + k];
                        o.w[0] = q.x; o.w[1] = q.y; o.w[2] = q.z; o.w[3] = q.w;
                    }
            }
            if (count) *count = n;
            if (dst) std::memcpy(dst, outv.data(), sizeof(lc_contact) * std::min<uint64_t>(n, cap));
            return LC_OK;
        }
        case LC_DBG_VF_NORMAL: {
            if (!d.vf_n) return fail(LC_ERR_INVALID_ARG, "VF normals are kept only in batches with friction");
            std::vector<uint64_t> gi;
            std::vector<int4> iv;
            std::vector<float4> wv;
            LC_TRY(b->cloth_contacts(c, true, gi, iv, wv));
            std::vector<float4> nr(gi.size());
            if (!nr.empty())
                LC_CUDA(cudaMemcpy(nr.data(), d.vf_n + gi.front(), sizeof(float4) * nr.size(), cudaMemcpyDeviceToHost));
            if (count) *count = gi.size();
            if (dst)
                for (uint64_t i = 0; i < std::min<uint64_t>(gi.size(), cap); ++i) {
                    ((float *)dst)[3 * i] = nr[i].x;
                    ((float *)dst)[3 * i + 1] = nr[i].y;
                    ((float *)dst)[3 * i + 2] = nr[i].z;
                }
            return LC_OK;
        }
        case LC_DBG_GROUND: {
            std::vector<float4> q(cd.V);
            LC_CUDA(cudaMemcpy(q.data(), d.ground_qc + cd.v_off, sizeof(float4) * cd.V, cudaMemcpyDeviceToHost));
            if (count) *count = cd.V;
            if (dst)
                for (uint64_t i = 0; i < std::min<uint64_t>(cd.V, cap); ++i) ((uint8_t *)dst)[i] = q[i].w != 0.f;
            return LC_OK;
        }
        case LC_DBG_GROUND_ACTIVE:
            if (!b->opt.debug_capture) return fail(LC_ERR_INVALID_ARG, "batch created without debug_capture");
            return dump(d.dbg_ground_it + cd.v_off, (uint64_t)cd.V, dst, cap, count);
        case LC_DBG_LRA: return dump(d.lra_flag + cd.lra_off, (uint64_t)cd.V * cd.F, dst, cap, count);
        case LC_DBG_SPHERE:
            if (!b->opt.debug_capture) return fail(LC_ERR_INVALID_ARG, "batch created without debug_capture");
            return dump(d.dbg_sphere + cd.v_off, (uint64_t)cd.V, dst, cap, count);
        case LC_DBG_DYN_ACTIVE: {
            if (!b->opt.debug_capture) return fail(LC_ERR_INVALID_ARG, "batch created without debug_capture");
            std::vector<uint64_t> gvf, gee;
            std::vector<int4> iv;
            std::vector<float4> wv;
            LC_TRY(b->cloth_contacts(c, true, gvf, iv, wv));
            LC_TRY(b->cloth_contacts(c, false, gee, iv, wv));
            uint32_t nvf_tot = 0;
            LC_CUDA(cudaMemcpy(&nvf_tot, b->nvf, sizeof(uint32_t), cudaMemcpyDeviceToHost));
            nvf_tot = (uint32_t)std::min<uint64_t>(nvf_tot, d.vf_cap);
            const int iters = b->cds[c].iters;
            const size_t nv4 = 4 * gvf.size(), ne4 = 4 * gee.size(), per = nv4 + ne4;
            // per iteration: the cloth's VF entries, then its EE entries (both contiguous)
            std::vector<uint8_t> outv((size_t)iters * per);
            for (int it = 0; it < iters && per; ++it) {
                const uint8_t *src = d.dbg_dyn_nz + (size_t)it * d.dyn_cap;
                if (nv4) LC_CUDA(cudaMemcpy(outv.data() + (size_t)it * per, src + 4 * gvf.front(), nv4,
                                            cudaMemcpyDeviceToHost));
                if (ne4) LC_CUDA(cudaMemcpy(outv.data() + (size_t)it * per + nv4, src + 4 * (nvf_tot + gee.front()),
                                            ne4, cudaMemcpyDeviceToHost));
            }
            if (count) *count = outv.size();
            if (dst && !outv.empty()) std::memcpy(dst, outv.data(), std::min<uint64_t>(outv.size(), cap));
            return LC_OK;
        }
        case LC_DBG_FEATURES: {
            const HostCloth &hc = b->hosts[c];
            if (count) *count = hc.features.size();
            if (dst) std::memcpy(dst, hc.features.data(), std::min<uint64_t>(hc.features.size(), cap));
            return LC_OK;
        }
        default: return fail(LC_ERR_INVALID_ARG, "unknown debug selector");
    }
}

lc_status lc_batch_write_state(lc_batch *b, const float *x, const float *xp, const float *v, int32_t is_host,
                               void *stream) {
    if (!b) return fail(LC_ERR_INVALID_ARG, "null batch");
    cudaStream_t st = (cudaStream_t)stream;
    const int n = b->d.Vtot;
    LC_TRY(put_xyz(b, b->d.x, x, n, is_host, st));
    LC_TRY(put_xyz(b, b->d.xp, xp, n, is_host, st));
    LC_TRY(put_xyz(b, b->d.v, v, n, is_host, st));
    LC_CUDA(cudaGetLastError());
    return LC_OK;
}

lc_status lc_batch_read_state(lc_batch *b, float *x, float *xp, float *v, int32_t is_host, void *stream) {
    if (!b) return fail(LC_ERR_INVALID_ARG, "null batch");
    cudaStream_t st = (cudaStream_t)stream;
    const int n = b->d.Vtot;
    LC_TRY(take_xyz(b, x, b->d.x, n, is_host, st));
    LC_TRY(take_xyz(b, xp, b->d.xp, n, is_host, st));
    LC_TRY(take_xyz(b, v, b->d.v, n, is_host, st));
    LC_CUDA(cudaGetLastError());
    return LC_OK;
}

lc_status lc_batch_profile(lc_batch *b, int32_t nsteps, void *stream, lc_profile *out) {
    if (!b || !out || nsteps < 1) return fail(LC_ERR_INVALID_ARG, "lc_batch_profile: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<cudaEvent_t> pev(8 * (size_t)nsteps), kev(12 * (size_t)nsteps);
    for (auto &e : pev) LC_CUDA(cudaEventCreate(&e));
    for (auto &e : kev) LC_CUDA(cudaEventCreate(&e));
    lc_status s = LC_OK;
    for (int k = 0; k < nsteps && s == LC_OK; ++k) {
        b->prof_ev = &pev[8 * (size_t)k];
        b->kern_ev = &kev[12 * (size_t)k];
        s = b->enqueue_step(st);
    }
    b->prof_ev = nullptr;
    b->kern_ev = nullptr;
    if (s == LC_OK) {
        LC_CUDA(cudaStreamSynchronize(st));
        std::memset(out, 0, sizeof(*out));
        for (int k = 0; k < nsteps; ++k) {
            float ms;
            for (int p = 0; p < 7; ++p) {
                cudaEventElapsedTime(&ms, pev[8 * k + p], pev[8 * k + p + 1]);
                out->phase_ms[p] += ms / nsteps;
            }
            const cudaEvent_t *e = &kev[12 * (size_t)k];
            cudaEventElapsedTime(&ms, e[0], e[1]);
            out->solver_ms += ms / nsteps;
            out->jacobi_ms += (b->use_cluster ? ms / b->max_iters : ms) / nsteps;
            cudaEventElapsedTime(&ms, e[2], e[3]); out->traverse_ms += ms / nsteps;
            cudaEventElapsedTime(&ms, e[4], e[5]); out->narrow_ms += ms / nsteps;
            cudaEventElapsedTime(&ms, e[6], e[7]); out->sort_ms += ms / nsteps;
            cudaEventElapsedTime(&ms, e[8], e[9]); out->ccd_vf_ms += ms / nsteps;
            cudaEventElapsedTime(&ms, e[9], e[10]); out->ccd_ee_ms += ms / nsteps;
        }
        for (int p = 0; p < 7; ++p) out->step_ms += out->phase_ms[p];
        out->solver_variant = b->use_cluster ? (b->cluster_scatter ? 3 : 2) : 1;
        out->cluster_size = b->use_cluster ? b->cluster_cs : 0;
        if (!b->use_cluster) out->solver_ms = out->phase_ms[5];
        // kernel launches per step, counted from the captured graph
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            lc_status s2 = b->enqueue_step(b->cap_stream);
            if (cudaStreamEndCapture(b->cap_stream, &g) == cudaSuccess && g && s2 == LC_OK) {
                size_t nn = 0;
                cudaGraphGetNodes(g, nullptr, &nn);
                std::vector<cudaGraphNode_t> nodes(nn);
                cudaGraphGetNodes(g, nodes.data(), &nn);
                uint32_t kn = 0;
                for (auto nd : nodes) {
                    cudaGraphNodeType t;
                    cudaGraphNodeGetType(nd, &t);
                    if (t == cudaGraphNodeTypeKernel) ++kn;
                }
                out->kernels_per_step = kn;
            }
            if (g) cudaGraphDestroy(g);
        }
    }
    for (auto &e : pev) cudaEventDestroy(e);
    for (auto &e : kev) cudaEventDestroy(e);
    return s;
}

// ----- standalone LBVH ------------------------------------------------------
struct lc_lbvh {
    lc_batch b;  // one cloth whose triangles are the caller's boxes
    int max_T = 0;
    int T = 0;
    int chunk_req = 64;
};

lc_status lc_lbvh_create(int32_t max_triangles, int32_t chunk_size, int32_t morton_mode, lc_lbvh **out) {
    if (max_triangles < 1 || chunk_size < 1 || !out) return fail(LC_ERR_INVALID_ARG, "lc_lbvh_create: bad arguments");
    *out = nullptr;
    std::unique_ptr<lc_lbvh> h(new lc_lbvh());
    lc_batch &b = h->b;
    b.C = 1;
    h->max_T = max_triangles;
    h->chunk_req = chunk_size;
    DevPtrs &d = b.d;
    DeviceArena &A = b.arena;
    const int64_t T = max_triangles, N = 2 * T - 1, I = T - 1, PC = T * std::min<int64_t>(chunk_size, T);
    const int64_t tiles = (T + kSortTile - 1) / kSortTile;
    b.cds.resize(1);
    std::memset(&b.cds[0], 0, sizeof(ClothDev));
    b.cds[0].chunk = (int)std::min<int64_t>(chunk_size, T);
    b.cds[0].morton_mode = morton_mode;
    b.cds[0].leaf_quirk = 0;
    b.cds[0].morton_scale = 1.f;
    b.sort_passes = morton_mode == LC_MORTON_K30 ? 4 : 8;
    d.C = 1;
    ClothDev *cdev;
    LC_TRY(A.alloc(cdev, 1, "cloth table")); d.cloth = cdev; b.cloth_dev = cdev;
    int *tcl; LC_TRY(A.alloc(tcl, T, "tcloth")); d.tcloth = tcl;
    LC_CUDA(cudaMemset(tcl, 0, sizeof(int) * T));
    LC_TRY(A.alloc(d.perm, T, "perm")); LC_TRY(A.alloc(d.perm_alt, T, "perm_alt"));
    LC_TRY(A.alloc(d.keys, T, "keys")); LC_TRY(A.alloc(d.keys_alt, T, "keys_alt"));
    LC_TRY(A.alloc(d.payload, T, "payload")); LC_TRY(A.alloc(d.payload_alt, T, "payload_alt"));
    LC_TRY(A.alloc(d.nmin, N, "nmin")); LC_TRY(A.alloc(d.nmax, N, "nmax"));
    LC_TRY(A.alloc(d.leaf_tmp_min, T, "leaf_tmp_min")); LC_TRY(A.alloc(d.leaf_tmp_max, T, "leaf_tmp_max"));
    LC_TRY(A.alloc(d.parent, N, "parent")); LC_TRY(A.alloc(d.child, I, "child"));
    LC_TRY(A.alloc(d.rml, I, "rml")); LC_TRY(A.alloc(d.visit, I, "visit")); LC_TRY(A.alloc(d.nend, I, "node range ends"));
    LC_TRY(A.alloc(d.rexit, 2 * std::max<int64_t>(I, 1), "refit exits")); LC_TRY(A.alloc(d.nrexit, 1, "refit exit count"));
    LC_TRY(A.alloc(d.pair_cnt, T, "pair_cnt")); LC_TRY(A.alloc(d.pair_off, T + 1, "pair_off"));
    LC_TRY(A.alloc(d.pair_chunk, PC, "pair_chunk")); LC_TRY(A.alloc(d.pairs, PC, "pairs"));
    LC_TRY(A.alloc(d.counters, 4, "counters")); LC_TRY(A.alloc(d.err, 1, "err"));
    LC_TRY(A.alloc(d.scan_tmp, kScanBlocks + 1, "scan_tmp"));
    int *stc, *sts, *tf;
    LC_TRY(A.alloc(stc, tiles, "stile_cloth")); LC_TRY(A.alloc(sts, tiles, "stile_start")); LC_TRY(A.alloc(tf, 2, "tile_first"));
    d.stile_cloth = stc; d.stile_start = sts; b.tile_first = tf;
    LC_TRY(A.alloc(d.shist, tiles * kSortBuckets, "shist"));
    LC_TRY(A.alloc(d.sseg, kSortPassesMax + (size_t)kSortPassesMax * kSortBuckets, "sort segment totals"));
    LC_TRY(A.alloc(d.sstat, (size_t)kSortPassesMax * tiles * kSortBuckets, "sort look-back status"));
    LC_TRY(A.alloc(b.npairs, 1, "npairs"));
    d.pair_cap = (uint64_t)PC;
    LC_CUDA(cudaMemset(d.err, 0, sizeof(uint32_t)));
    LC_CUDA(cudaMemset(stc, 0, sizeof(int) * tiles));
    b.traverse_block = 128;
    *out = h.release();
    return LC_OK;
}

lc_status lc_lbvh_build(lc_lbvh *h, const float *tri_min, const float *tri_max, int32_t num_triangles, void *stream) {
    if (!h || !tri_min || !tri_max || num_triangles < 1 || num_triangles > h->max_T)
        return fail(LC_ERR_INVALID_ARG, "lc_lbvh_build: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    lc_batch &b = h->b;
    DevPtrs &d = b.d;
    const int T = num_triangles;
    if (T != h->T) {
        h->T = T;
        ClothDev &cd = b.cds[0];
        cd.T = T;
        cd.chunk = std::min(h->chunk_req, T);
        std::vector<int> starts;
        for (int s = 0; s < T; s += kSortTile) starts.push_back(s);
        const int tf[2] = {0, (int)starts.size()};
        LC_CUDA(cudaStreamSynchronize(st));
        LC_CUDA(cudaMemcpy((void *)d.stile_start, starts.data(), sizeof(int) * starts.size(), cudaMemcpyHostToDevice));
        LC_CUDA(cudaMemcpy(b.tile_first, tf, sizeof(tf), cudaMemcpyHostToDevice));
        LC_CUDA(cudaMemcpy(b.cloth_dev, &cd, sizeof(ClothDev), cudaMemcpyHostToDevice));
        d.nstiles = (int)starts.size();
    }
    d.Ttot = T;
    d.Ntot = 2 * T - 1;
    d.Itot = T - 1;
    LC_CUDA(cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long) * 4, st));
    launch_leaves_from_boxes(d, tri_min, tri_max, T, b.cds[0].morton_mode, st);
    launch_sort(d, b.tile_first, b.sort_passes, st);
    launch_post_sort(d, st);
    LC_CUDA(cudaMemcpyAsync(d.perm, d.perm_alt, sizeof(uint32_t) * T, cudaMemcpyDeviceToDevice, st));
    LC_CUDA(cudaMemsetAsync(d.parent, 0xFF, sizeof(int) * (size_t)d.Ntot, st));
    launch_karras(d, st);
    launch_refit(d, st);
    LC_CUDA(cudaGetLastError());
    return LC_OK;
}

lc_status lc_lbvh_pairs(lc_lbvh *h, uint32_t *out_pairs, uint64_t cap, uint64_t *count, void *stream) {
    if (!h || !count) return fail(LC_ERR_INVALID_ARG, "lc_lbvh_pairs: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    lc_batch &b = h->b;
    DevPtrs &d = b.d;
    launch_traverse(d, b.traverse_block, st);
    scan_u32(d.pair_cnt, d.pair_off, nullptr, (uint32_t)d.Ttot, (uint32_t)d.Ttot, d.scan_tmp, b.npairs,
             &d.counters[0], st);
    launch_pair_compact(d, st);
    LC_CUDA(cudaGetLastError());
    uint32_t n = 0;
    LC_CUDA(cudaMemcpyAsync(&n, b.npairs, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    LC_CUDA(cudaStreamSynchronize(st));
    *count = n;
    if (out_pairs && n)
        LC_CUDA(cudaMemcpyAsync(out_pairs, d.pairs, sizeof(uint2) * std::min<uint64_t>(n, cap), cudaMemcpyDeviceToDevice, st));
    uint32_t err = 0;
    LC_CUDA(cudaMemcpy(&err, d.err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err & ERR_STACK) return fail(LC_ERR_STACK_OVERFLOW, "BVH traversal stack (64) exceeded");
    if (err & ERR_SORT) return fail(LC_ERR_TIMEOUT, "sort look-back wait exceeded its bound");
    return LC_OK;
}

lc_status lc_lbvh_sorted_ids(lc_lbvh *h, uint32_t *out_ids, void *stream) {
    if (!h || !out_ids) return fail(LC_ERR_INVALID_ARG, "lc_lbvh_sorted_ids: bad arguments");
    LC_CUDA(cudaMemcpyAsync(out_ids, h->b.d.perm, sizeof(uint32_t) * h->T, cudaMemcpyDeviceToDevice,
                            (cudaStream_t)stream));
    return LC_OK;
}

lc_status lc_lbvh_debug_get(lc_lbvh *h, int32_t what, void *dst, uint64_t cap, uint64_t *count) {
    if (!h || h->T < 1) return fail(LC_ERR_INVALID_ARG, "lc_lbvh_debug_get: no hierarchy built");
    switch (what) {
        case LC_DBG_MORTON: case LC_DBG_PERM: case LC_DBG_LEFTS: case LC_DBG_RIGHTS: case LC_DBG_PARENTS:
        case LC_DBG_RML: case LC_DBG_NODE_AABB: case LC_DBG_PAIRS:
            break;
        default:
            return fail(LC_ERR_NOT_SUPPORTED, "lc_lbvh_debug_get: selector not held by a standalone LBVH");
    }
    // the build and the query run on the caller's streams
    LC_CUDA(cudaDeviceSynchronize());
    return lc_batch_debug_get(&h->b, 0, what, dst, cap, count);
}

lc_status lc_lbvh_destroy(lc_lbvh *h) {
    if (h) {
        cudaDeviceSynchronize();
        delete h;
    }
    return LC_OK;
}

}  // extern "C"
