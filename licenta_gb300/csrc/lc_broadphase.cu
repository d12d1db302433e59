// lc_broadphase.cu — the object-level broadphase family of the reference's
// Collision::ICollisionMethod (Collision/ICollisionMethod.h:15-87): given
// one axis-aligned box per scene object, Update() builds the method's
// structure and TestCollision() returns the pairs of objects whose boxes
// overlap.  The reference's members are CPU code over SceneObjects (BVH,
// SweepAndPrune, SpatialGrid, SpatialHashing: Collision/BVH.cpp:11-120,
// SweepAndPrune.cpp:31-176, SpatialGrid.cpp:79-153, SpatialHashing.cpp:
// 20-120); here each is a GPU method over a device array of boxes, and every
// method returns the same set: all pairs (a, b), a < b, whose closed boxes
// overlap (Collision/DataStructures/BoundingBox Collides), with no cap per
// object and no pair lost:
//
//   LC_BP_BRUTE  every pair tested (the yardstick);
//   LC_BP_SAP    sort by the boxes' lower x (the engine's radix sort), then
//                each object sweeps forward while the next lower x is within
//                its upper x;
//   LC_BP_GRID   a uniform grid over the world box: each object enters every
//                cell its box covers, entries are sorted by cell, and a pair
//                is reported in the one cell that holds the lower corner of
//                the two boxes' intersection (no duplicates);
//   LC_BP_HASH   the same over an unbounded grid of a given cell size whose
//                cells are hashed into a fixed table (entries of different
//                cells that share a bucket are told apart by their cell);
//   LC_BP_BVH    a linear BVH over the boxes: 30-bit Morton codes of the
//                box centres with the object index appended (unique keys),
//                the engine's radix sort, a Karras hierarchy (Karras 2012)
//                and a bottom-up refit; then a traversal per leaf that
//                counts, then writes, its pairs with the leaves after it.
//                (The cloth path's LBVH keeps the reference's codes, whose
//                duplicates can cost the hierarchy a leaf; this member
//                must not lose a pair.)
//
// Every pair-producing pass runs twice, counting and then writing at offsets
// from a scan, so the output order is fixed and nothing depends on how
// atomics land.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "lc_internal.cuh"

namespace lc {
void launch_sort(const DevPtrs &d, const int *tile_first, int passes, cudaStream_t st);
void scan_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap,
              uint32_t *partial, uint32_t *total_out, unsigned long long *total_out64, cudaStream_t st);
void set_last_error(const std::string &msg);

namespace {

// The hierarchy splits at the highest differing bit of unique 62-bit keys, so
// it is at most 62 levels deep; the traversal stack and the refit's walk to
// the root have room beyond that.
constexpr int kBpStack = 128;
constexpr int kBpDepth = 130;
enum : uint32_t { BP_ERR_STACK = 1u, BP_ERR_ENTRIES = 2u };

lc_status bp_fail(lc_status s, const std::string &msg) {
    set_last_error(msg);
    return s;
}

__device__ __forceinline__ bool box_overlap(const float *__restrict__ lo, const float *__restrict__ hi, int a, int b) {
    return lo[3 * a] <= hi[3 * b] && hi[3 * a] >= lo[3 * b] && lo[3 * a + 1] <= hi[3 * b + 1] &&
           hi[3 * a + 1] >= lo[3 * b + 1] && lo[3 * a + 2] <= hi[3 * b + 2] && hi[3 * a + 2] >= lo[3 * b + 2];
}
__device__ __forceinline__ void put_pair(uint32_t *out, uint32_t k, int a, int b) {
    out[2 * k] = (uint32_t)min(a, b);
    out[2 * k + 1] = (uint32_t)max(a, b);
}
// A float's order as an unsigned integer (negative values reversed).
__device__ __forceinline__ uint32_t float_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ---- brute force ------------------------------------------------------------
// pass 0 counts the pairs (a, b > a) of object a, pass 1 writes them.
__global__ void k_bp_brute(const float *lo, const float *hi, int n, uint32_t *cnt, const uint32_t *off,
                           uint32_t *out, uint64_t cap, unsigned long long *tests) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    uint32_t c = 0, k = off ? off[a] : 0u;
    for (int b = a + 1; b < n; ++b)
        if (box_overlap(lo, hi, a, b)) {
            if (out && k < cap) put_pair(out, k, a, b);
            ++k;
            ++c;
        }
    if (cnt) {
        cnt[a] = c;
        atomicAdd(tests, (unsigned long long)(n - 1 - a));
    }
}

// ---- sweep and prune ----------------------------------------------------------
__global__ void k_bp_sap_keys(const float *lo, int n, unsigned long long *keys, uint32_t *payload) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    keys[a] = float_key(lo[3 * a]);
    payload[a] = (uint32_t)a;
}
// Rank r (object s = order[r]) sweeps the objects after it in the sorted
// order while their lower x is within its upper x.
__global__ void k_bp_sap_sweep(const float *lo, const float *hi, int n, const uint32_t *__restrict__ order,
                               uint32_t *cnt, const uint32_t *off, uint32_t *out, uint64_t cap,
                               unsigned long long *tests) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int a = (int)order[r];
    const float ax = hi[3 * a];
    uint32_t c = 0, k = off ? off[r] : 0u, t = 0;
    for (int q = r + 1; q < n; ++q) {
        const int b = (int)order[q];
        if (lo[3 * b] > ax) break;
        ++t;
        if (box_overlap(lo, hi, a, b)) {
            if (out && k < cap) put_pair(out, k, a, b);
            ++k;
            ++c;
        }
    }
    if (cnt) {
        cnt[r] = c;
        atomicAdd(tests, (unsigned long long)t);
    }
}

// ---- grids (uniform and hashed) --------------------------------------------
struct GridSpec {
    float wmin[3];
    float inv_cell[3];
    int ncell[3];     // uniform grid: cells per axis (coordinates clamped into it); hash: unused
    uint32_t table;   // hash: table size (a power of two); 0 for the uniform grid
};
__device__ __forceinline__ int cell_of(const GridSpec &g, float v, int ax) {
    const float f = floorf((v - g.wmin[ax]) * g.inv_cell[ax]);
    if (g.table) return (int)fmaxf(fminf(f, 1.0e9f), -1.0e9f);
    return min(max((int)fmaxf(fminf(f, 2.0e9f), -2.0e9f), 0), g.ncell[ax] - 1);
}
__device__ __forceinline__ uint32_t bucket_of(const GridSpec &g, int x, int y, int z) {
    if (!g.table) return (uint32_t)((z * g.ncell[1] + y) * g.ncell[0] + x);
    // the three-prime spatial hash (Teschner et al., 2003)
    const uint32_t h = ((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349663u) ^ ((uint32_t)z * 83492791u);
    return h & (g.table - 1u);
}
// pass 0: entries per object (cells its box covers); pass 1: the entries.
__global__ void k_bp_grid_entries(GridSpec g, const float *lo, const float *hi, int n, uint32_t *cnt,
                                  const uint32_t *off, uint64_t cap, unsigned long long *keys, uint32_t *payload,
                                  int4 *ecell, uint32_t *err) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    int c0[3], c1[3];
    for (int ax = 0; ax < 3; ++ax) {
        c0[ax] = cell_of(g, lo[3 * a + ax], ax);
        c1[ax] = cell_of(g, hi[3 * a + ax], ax);
    }
    const uint64_t m = (uint64_t)(c1[0] - c0[0] + 1) * (uint64_t)(c1[1] - c0[1] + 1) * (uint64_t)(c1[2] - c0[2] + 1);
    if (cnt) {
        if (m > 0xFFFFFFFFull / 4u) { atomicOr(err, BP_ERR_ENTRIES); cnt[a] = 0; return; }
        cnt[a] = (uint32_t)m;
        return;
    }
    uint64_t k = off[a];
    for (int z = c0[2]; z <= c1[2]; ++z)
        for (int y = c0[1]; y <= c1[1]; ++y)
            for (int x = c0[0]; x <= c1[0]; ++x, ++k) {
                if (k >= cap) { atomicOr(err, BP_ERR_ENTRIES); return; }
                keys[k] = bucket_of(g, x, y, z);
                payload[k] = (uint32_t)k;
                ecell[k] = make_int4(x, y, z, a);
            }
}
// Entry at sorted rank r against the entries after it in the same bucket: a
// pair is reported where both entries are the same cell and that cell holds
// the lower corner of the two boxes' intersection.
__global__ void k_bp_grid_pairs(GridSpec g, const float *lo, const float *hi, int ne,
                                const unsigned long long *__restrict__ keys, const uint32_t *__restrict__ order,
                                const int4 *__restrict__ ecell, uint32_t *cnt, const uint32_t *off, uint32_t *out,
                                uint64_t cap, unsigned long long *tests) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ne) return;
    const unsigned long long key = keys[r];
    const int4 e = ecell[order[r]];
    const int a = e.w;
    uint32_t c = 0, k = off ? off[r] : 0u, t = 0;
    for (int q = r + 1; q < ne && keys[q] == key; ++q) {
        const int4 f = ecell[order[q]];
        if (f.x != e.x || f.y != e.y || f.z != e.z) continue;  // another cell in the same bucket
        const int b = f.w;
        ++t;
        if (!box_overlap(lo, hi, a, b)) continue;
        if (cell_of(g, fmaxf(lo[3 * a], lo[3 * b]), 0) != e.x || cell_of(g, fmaxf(lo[3 * a + 1], lo[3 * b + 1]), 1) != e.y ||
            cell_of(g, fmaxf(lo[3 * a + 2], lo[3 * b + 2]), 2) != e.z)
            continue;
        if (out && k < cap) put_pair(out, k, a, b);
        ++k;
        ++c;
    }
    if (cnt) {
        cnt[r] = c;
        atomicAdd(tests, (unsigned long long)t);
    }
}

// ---- BVH ------------------------------------------------------------------------
struct BvhPtrs {
    int2 *child;          // internal node: children (internal 0..n-2, leaves n-1 + slot)
    int *parent;          // 2n-1 nodes
    float4 *nmin, *nmax;  // 2n-1 node boxes
    int *rmost;           // 2n-1: rightmost leaf slot under the node
    int *visit;           // n-1 arrival counters of the refit
    unsigned int *bounds; // 6 ordered-float words: scene box of the box centres
};
__device__ __forceinline__ float ordered_to_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
// Scene box of the centres (one block reduces, six atomics per block).
__global__ void k_bp_bounds(const float *lo, const float *hi, int n, unsigned int *bounds) {
    __shared__ unsigned int s[6];
    if (threadIdx.x < 6) s[threadIdx.x] = threadIdx.x < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n)
        for (int ax = 0; ax < 3; ++ax) {
            const uint32_t k = float_key(0.5f * (lo[3 * a + ax] + hi[3 * a + ax]));
            atomicMin(&s[ax], k);
            atomicMax(&s[3 + ax], k);
        }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(&bounds[threadIdx.x], s[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(&bounds[threadIdx.x], s[threadIdx.x]);
}
__global__ void k_bp_bvh_keys(const float *lo, const float *hi, int n, const unsigned int *bounds,
                              unsigned long long *keys, uint32_t *payload) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    uint32_t m = 0;
    for (int ax = 0; ax < 3; ++ax) {
        const float b0 = ordered_to_float(bounds[ax]), b1 = ordered_to_float(bounds[3 + ax]);
        const float c = 0.5f * (lo[3 * a + ax] + hi[3 * a + ax]);
        const float ext = b1 - b0;
        const float t = ext > 0.f ? (c - b0) / ext : 0.f;
        const uint32_t q = (uint32_t)fminf(fmaxf(t * 1024.f, 0.f), 1023.f);
        m |= spread10(q) << (2 - ax);
    }
    keys[a] = ((unsigned long long)m << 32) | (uint32_t)a;
    payload[a] = (uint32_t)a;
}
__device__ __forceinline__ int bp_delta(const unsigned long long *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    return __clzll(k[i] ^ k[j]);  // keys are unique
}
// Karras (2012), Algorithm 3, on unique keys.
__global__ void k_bp_karras(BvhPtrs B, const unsigned long long *__restrict__ k, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int I = n - 1;
    const int dir = bp_delta(k, n, i, i + 1) - bp_delta(k, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = bp_delta(k, n, i, i - dir);
    int lmax = 2;
    while (bp_delta(k, n, i, i + lmax * dir) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (bp_delta(k, n, i, i + (l + t) * dir) > dmin) l += t;
    const int j = i + l * dir;
    const int dnode = bp_delta(k, n, i, j);
    int sp = 0;
    for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
        if (bp_delta(k, n, i, i + (sp + t) * dir) > dnode) sp += t;
        if (t == 1) break;
    }
    const int gamma = i + sp * dir + min(dir, 0);
    const int left = min(i, j) == gamma ? I + gamma : gamma;
    const int right = max(i, j) == gamma + 1 ? I + gamma + 1 : gamma + 1;
    B.child[i] = make_int2(left, right);
    B.parent[left] = i;
    B.parent[right] = i;
    B.visit[i] = 0;
}
// Leaves' boxes, then the second child to arrive at a node writes its union.
__global__ void k_bp_refit(BvhPtrs B, const float *lo, const float *hi, const uint32_t *__restrict__ order, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int I = n - 1;
    const int a = (int)order[s];
    int node = I + s;
    B.nmin[node] = make_float4(lo[3 * a], lo[3 * a + 1], lo[3 * a + 2], 0.f);
    B.nmax[node] = make_float4(hi[3 * a], hi[3 * a + 1], hi[3 * a + 2], 0.f);
    B.rmost[node] = s;
    if (n == 1) return;
    for (int guard = 0; guard < kBpDepth && node != 0; ++guard) {
        const int p = B.parent[node];
        __threadfence();
        if (atomicAdd(&B.visit[p], 1) == 0) return;  // the other child is not done yet
        __threadfence();
        const int2 ch = B.child[p];
        const float4 l0 = __ldcg(&B.nmin[ch.x]), l1 = __ldcg(&B.nmax[ch.x]);
        const float4 r0 = __ldcg(&B.nmin[ch.y]), r1 = __ldcg(&B.nmax[ch.y]);
        B.nmin[p] = f4(vmin(xyz(l0), xyz(r0)), 0.f);
        B.nmax[p] = f4(vmax(xyz(l1), xyz(r1)), 0.f);
        B.rmost[p] = max(__ldcg(&B.rmost[ch.x]), __ldcg(&B.rmost[ch.y]));
        node = p;
    }
}
// Leaf slot s (box order[s]) against the leaves after it: subtrees whose
// rightmost leaf lies at or before s are skipped.
__global__ void k_bp_bvh(BvhPtrs B, const float *lo, const float *hi, const uint32_t *__restrict__ order, int n,
                         uint32_t *cnt, const uint32_t *off, uint32_t *out, uint64_t cap,
                         unsigned long long *tests, uint32_t *err) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int a = (int)order[s];
    uint32_t c = 0, k = off ? off[s] : 0u, t = 0;
    if (n > 1) {
        const float3 alo = f3(lo[3 * a], lo[3 * a + 1], lo[3 * a + 2]), ahi = f3(hi[3 * a], hi[3 * a + 1], hi[3 * a + 2]);
        const int I = n - 1;
        int stack[kBpStack];
        int top = 0;
        stack[top++] = 0;
        while (top > 0) {
            const int node = stack[--top];
            if (__ldg(&B.rmost[node]) <= s) continue;
            if (!overlap(alo, ahi, xyz(__ldg(&B.nmin[node])), xyz(__ldg(&B.nmax[node])))) continue;
            if (node >= I) {
                const int b = (int)order[node - I];
                ++t;
                if (box_overlap(lo, hi, a, b)) {
                    if (out && k < cap) put_pair(out, k, a, b);
                    ++k;
                    ++c;
                }
                continue;
            }
            if (top + 2 > kBpStack) { atomicOr(err, BP_ERR_STACK); break; }
            const int2 ch = __ldg(&B.child[node]);
            stack[top++] = ch.y;
            stack[top++] = ch.x;
        }
    }
    if (cnt) {
        cnt[s] = c;
        atomicAdd(tests, (unsigned long long)t);
    }
}

inline int nblocks(int64_t n) { return (int)((n + kThreads - 1) / kThreads); }

#define LC_TRY_BP(x)                    \
    do {                                \
        const lc_status s_ = (x);       \
        if (s_ != LC_OK) return s_;     \
    } while (0)
#define LC_BP_CUDA(x)                                                                          \
    do {                                                                                       \
        const cudaError_t e_ = (x);                                                            \
        if (e_ != cudaSuccess) {                                                               \
            cudaGetLastError();                                                                \
            return bp_fail(LC_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));      \
        }                                                                                      \
    } while (0)

}  // namespace
}  // namespace lc

using namespace lc;

struct lc_broadphase {
    lc_broadphase_desc desc{};
    int n = 0;                       // objects of the last update
    const float *lo = nullptr, *hi = nullptr;  // the caller's boxes of the last update
    std::vector<void *> mem;
    uint64_t bytes = 0;
    // sort of up to max_keys u64 keys with u32 payload (one segment)
    DevPtrs sd{};
    int *tile_first = nullptr;
    int sort_passes = 4;
    uint64_t max_keys = 0;
    // counts, offsets and the scan's scratch
    uint32_t *cnt = nullptr, *off = nullptr, *scan_tmp = nullptr, *total = nullptr;
    unsigned long long *tests = nullptr;
    uint32_t *err = nullptr;
    int4 *ecell = nullptr;
    int ne = 0;                      // grid / hash entries of the last update
    BvhPtrs bvh{};
    float *hlo = nullptr, *hhi = nullptr;  // device copies of host boxes (lc_broadphase_update_host)
    uint32_t *stage = nullptr;             // pairs on their way to host memory (lc_broadphase_test_host)
    uint64_t stage_cap = 0;
    GridSpec grid{};
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    uint64_t last_tests = 0, last_pairs = 0;

    template <class T> lc_status alloc(T *&p, uint64_t count, const char *what) {
        void *q = nullptr;
        const size_t sz = sizeof(T) * (size_t)std::max<uint64_t>(count, 1);
        if (cudaMalloc(&q, sz) != cudaSuccess) {
            cudaGetLastError();
            return bp_fail(LC_ERR_OOM, std::string("lc_broadphase_create: cudaMalloc failed for ") + what);
        }
        mem.push_back(q);
        bytes += sz;
        p = static_cast<T *>(q);
        return LC_OK;
    }
    ~lc_broadphase() {
        if (stage) cudaFree(stage);
        for (void *q : mem) cudaFree(q);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    // Sort keys[0, count) with payload on stream st (result in sd.keys / sd.payload).
    lc_status sort(uint64_t count, cudaStream_t st) {
        if (count < 2) return LC_OK;
        std::vector<int> starts;
        for (uint64_t s = 0; s < count; s += kSortTile) starts.push_back((int)s);
        ClothDev cd{};
        cd.T = (int)count;
        const int tf[2] = {0, (int)starts.size()};
        LC_BP_CUDA(cudaMemcpyAsync((void *)sd.stile_start, starts.data(), sizeof(int) * starts.size(),
                                   cudaMemcpyHostToDevice, st));
        LC_BP_CUDA(cudaMemcpyAsync(tile_first, tf, sizeof(tf), cudaMemcpyHostToDevice, st));
        LC_BP_CUDA(cudaMemcpyAsync((void *)sd.cloth, &cd, sizeof(ClothDev), cudaMemcpyHostToDevice, st));
        // the host arrays above are read by the copies before the sort starts
        LC_BP_CUDA(cudaStreamSynchronize(st));
        sd.nstiles = (int)starts.size();
        sd.Ttot = (int)std::min<uint64_t>(count, 0x7FFFFFFFull);  // the one-sweep's 30-bit count check
        launch_sort(sd, tile_first, sort_passes, st);
        return LC_OK;
    }
};

extern "C" {

lc_status lc_broadphase_create(const lc_broadphase_desc *desc, lc_broadphase **out) {
    if (!desc || !out) return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_create: bad arguments");
    *out = nullptr;
    const lc_broadphase_desc &q = *desc;
    if (q.method < LC_BP_BRUTE || q.method > LC_BP_BVH || q.max_objects < 1 || q.max_objects > (1 << 28))
        return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_create: bad method or max_objects");
    std::unique_ptr<lc_broadphase> h(new lc_broadphase());
    h->desc = q;
    const uint64_t N = (uint64_t)q.max_objects;
    uint64_t E = 0;
    if (q.method == LC_BP_GRID) {
        if (q.cells_per_axis < 1 || q.cells_per_axis > 1024)
            return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_create: cells_per_axis must be in [1, 1024]");
        for (int ax = 0; ax < 3; ++ax) {
            if (!(q.world_max[ax] > q.world_min[ax]))
                return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_create: empty world box");
            h->grid.wmin[ax] = q.world_min[ax];
            h->grid.inv_cell[ax] = (float)q.cells_per_axis / (q.world_max[ax] - q.world_min[ax]);
            h->grid.ncell[ax] = q.cells_per_axis;
        }
        h->grid.table = 0;
    } else if (q.method == LC_BP_HASH) {
        if (!(q.cell_size > 0.f) || q.table_size < 1 || (q.table_size & (q.table_size - 1)))
            return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_create: cell_size > 0 and a power-of-two table_size");
        for (int ax = 0; ax < 3; ++ax) {
            h->grid.wmin[ax] = 0.f;
            h->grid.inv_cell[ax] = 1.f / q.cell_size;
            h->grid.ncell[ax] = 0;
        }
        h->grid.table = (uint32_t)q.table_size;
    }
    if (q.method == LC_BP_GRID || q.method == LC_BP_HASH) {
        E = q.max_entries ? q.max_entries : 8 * N;
        if (E > 0xFFFFFFF0ull) return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_create: max_entries too large");
    }
    lc_broadphase &b = *h;
    const uint64_t keys = q.method == LC_BP_BRUTE ? 0 : (E ? E : N);
    const uint64_t counts = std::max<uint64_t>(N, E);
    LC_TRY_BP(b.alloc(b.cnt, counts, "counts"));
    LC_TRY_BP(b.alloc(b.off, counts + 1, "offsets"));
    LC_TRY_BP(b.alloc(b.scan_tmp, kScanBlocks + 1, "scan partials"));
    LC_TRY_BP(b.alloc(b.total, 1, "total"));
    LC_TRY_BP(b.alloc(b.tests, 1, "tests"));
    LC_TRY_BP(b.alloc(b.err, 1, "error word"));
    LC_BP_CUDA(cudaMemset(b.err, 0, sizeof(uint32_t)));
    if (keys) {
        b.max_keys = keys;
        const uint64_t tiles = (keys + kSortTile - 1) / kSortTile;
        DevPtrs &d = b.sd;
        d.C = 1;
        ClothDev *cd;
        LC_TRY_BP(b.alloc(cd, 1, "sort segment"));
        d.cloth = cd;
        int *stc, *sts;
        LC_TRY_BP(b.alloc(stc, tiles, "sort tile segments"));
        LC_BP_CUDA(cudaMemset(stc, 0, sizeof(int) * tiles));
        LC_TRY_BP(b.alloc(sts, tiles, "sort tile starts"));
        d.stile_cloth = stc;
        d.stile_start = sts;
        LC_TRY_BP(b.alloc(d.shist, tiles * kSortBuckets, "sort histograms"));
        LC_TRY_BP(b.alloc(d.sseg, kSortPassesMax + (size_t)kSortPassesMax * kSortBuckets, "sort segment totals"));
        LC_TRY_BP(b.alloc(d.sstat, (size_t)kSortPassesMax * tiles * kSortBuckets, "sort look-back status"));
        d.err = b.err;
        LC_TRY_BP(b.alloc(d.keys, keys, "keys"));
        LC_TRY_BP(b.alloc(d.keys_alt, keys, "keys"));
        LC_TRY_BP(b.alloc(d.payload, keys, "payload"));
        LC_TRY_BP(b.alloc(d.payload_alt, keys, "payload"));
        LC_TRY_BP(b.alloc(b.tile_first, 2, "tile table"));
        b.sort_passes = q.method == LC_BP_BVH ? 8 : 4;
    }
    if (E) LC_TRY_BP(b.alloc(b.ecell, E, "cell entries"));
    if (q.method == LC_BP_BVH) {
        BvhPtrs &B = b.bvh;
        LC_TRY_BP(b.alloc(B.child, N, "children"));
        LC_TRY_BP(b.alloc(B.parent, 2 * N, "parents"));
        LC_TRY_BP(b.alloc(B.nmin, 2 * N, "node boxes"));
        LC_TRY_BP(b.alloc(B.nmax, 2 * N, "node boxes"));
        LC_TRY_BP(b.alloc(B.rmost, 2 * N, "rightmost leaves"));
        LC_TRY_BP(b.alloc(B.visit, N, "arrival counters"));
        LC_TRY_BP(b.alloc(B.bounds, 6, "scene box"));
    }
    LC_TRY_BP(b.alloc(b.hlo, 3 * N, "host box copies"));
    LC_TRY_BP(b.alloc(b.hhi, 3 * N, "host box copies"));
    for (cudaEvent_t &e : b.ev) LC_BP_CUDA(cudaEventCreate(&e));
    *out = h.release();
    return LC_OK;
}

lc_status lc_broadphase_update(lc_broadphase *b, const float *box_min, const float *box_max, int32_t n,
                               void *stream) {
    if (!b || n < 0 || n > b->desc.max_objects || (n > 0 && (!box_min || !box_max)))
        return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_update: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    b->n = n;
    b->lo = box_min;
    b->hi = box_max;
    b->ne = 0;
    LC_BP_CUDA(cudaEventRecord(b->ev[0], st));
    const int m = b->desc.method;
    if (n > 0 && m == LC_BP_SAP) {
        k_bp_sap_keys<<<nblocks(n), kThreads, 0, st>>>(box_min, n, b->sd.keys, b->sd.payload);
        LC_TRY_BP(b->sort((uint64_t)n, st));
    } else if (n > 0 && (m == LC_BP_GRID || m == LC_BP_HASH)) {
        k_bp_grid_entries<<<nblocks(n), kThreads, 0, st>>>(b->grid, box_min, box_max, n, b->cnt, nullptr, 0, nullptr,
                                                            nullptr, nullptr, b->err);
        scan_u32(b->cnt, b->off, nullptr, (uint32_t)n, (uint32_t)n, b->scan_tmp, b->total, nullptr, st);
        uint32_t tot = 0, err = 0;
        LC_BP_CUDA(cudaMemcpyAsync(&tot, b->total, sizeof(tot), cudaMemcpyDeviceToHost, st));
        LC_BP_CUDA(cudaMemcpyAsync(&err, b->err, sizeof(err), cudaMemcpyDeviceToHost, st));
        LC_BP_CUDA(cudaStreamSynchronize(st));
        if (err || tot > b->max_keys) {
            LC_BP_CUDA(cudaMemset(b->err, 0, sizeof(uint32_t)));
            return bp_fail(LC_ERR_CAPACITY_OVERFLOW, "lc_broadphase_update: the boxes cover more grid cells than "
                                                     "lc_broadphase_desc.max_entries (" + std::to_string(tot) + ")");
        }
        b->ne = (int)tot;
        k_bp_grid_entries<<<nblocks(n), kThreads, 0, st>>>(b->grid, box_min, box_max, n, nullptr, b->off, tot,
                                                            b->sd.keys, b->sd.payload, b->ecell, b->err);
        LC_TRY_BP(b->sort(tot, st));
    } else if (n > 0 && m == LC_BP_BVH) {
        const unsigned int init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
        LC_BP_CUDA(cudaMemcpyAsync(b->bvh.bounds, init, sizeof(init), cudaMemcpyHostToDevice, st));
        k_bp_bounds<<<nblocks(n), kThreads, 0, st>>>(box_min, box_max, n, b->bvh.bounds);
        k_bp_bvh_keys<<<nblocks(n), kThreads, 0, st>>>(box_min, box_max, n, b->bvh.bounds, b->sd.keys, b->sd.payload);
        LC_TRY_BP(b->sort((uint64_t)n, st));
        if (n > 1) k_bp_karras<<<nblocks(n - 1), kThreads, 0, st>>>(b->bvh, b->sd.keys, n);
        k_bp_refit<<<nblocks(n), kThreads, 0, st>>>(b->bvh, box_min, box_max, b->sd.payload, n);
    }
    LC_BP_CUDA(cudaGetLastError());
    LC_BP_CUDA(cudaEventRecord(b->ev[1], st));
    return LC_OK;
}

lc_status lc_broadphase_update_host(lc_broadphase *b, const float *box_min, const float *box_max, int32_t n,
                                    void *stream) {
    if (!b || n < 0 || n > b->desc.max_objects || (n > 0 && (!box_min || !box_max)))
        return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_update_host: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0) {
        LC_BP_CUDA(cudaMemcpyAsync(b->hlo, box_min, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
        LC_BP_CUDA(cudaMemcpyAsync(b->hhi, box_max, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
    }
    return lc_broadphase_update(b, b->hlo, b->hhi, n, stream);
}

lc_status lc_broadphase_test(lc_broadphase *b, uint32_t *pairs, uint64_t cap, uint64_t *count, void *stream) {
    if (!b || !count || (cap > 0 && !pairs)) return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_test: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const int n = b->n, m = b->desc.method;
    const float *lo = b->lo, *hi = b->hi;
    LC_BP_CUDA(cudaEventRecord(b->ev[2], st));
    LC_BP_CUDA(cudaMemsetAsync(b->tests, 0, sizeof(unsigned long long), st));
    // the units whose pairs are counted and then written: objects, sorted
    // ranks or grid entries
    const int units = (m == LC_BP_GRID || m == LC_BP_HASH) ? b->ne : n;
    auto run = [&](uint32_t *cnt, const uint32_t *off, uint32_t *out) {
        if (!units) return;
        if (m == LC_BP_BRUTE)
            k_bp_brute<<<nblocks(units), kThreads, 0, st>>>(lo, hi, n, cnt, off, out, cap, b->tests);
        else if (m == LC_BP_SAP)
            k_bp_sap_sweep<<<nblocks(units), kThreads, 0, st>>>(lo, hi, n, b->sd.payload, cnt, off, out, cap,
                                                               b->tests);
        else if (m == LC_BP_BVH)
            k_bp_bvh<<<nblocks(units), kThreads, 0, st>>>(b->bvh, lo, hi, b->sd.payload, n, cnt, off, out, cap,
                                                         b->tests, b->err);
        else
            k_bp_grid_pairs<<<nblocks(units), kThreads, 0, st>>>(b->grid, lo, hi, units, b->sd.keys, b->sd.payload,
                                                                b->ecell, cnt, off, out, cap, b->tests);
    };
    run(b->cnt, nullptr, nullptr);
    uint32_t tot = 0;
    if (units) {
        scan_u32(b->cnt, b->off, nullptr, (uint32_t)units, (uint32_t)units, b->scan_tmp, b->total, nullptr, st);
        if (pairs && cap) run(nullptr, b->off, pairs);
        LC_BP_CUDA(cudaMemcpyAsync(&tot, b->total, sizeof(tot), cudaMemcpyDeviceToHost, st));
    }
    unsigned long long tests = 0;
    uint32_t err = 0;
    LC_BP_CUDA(cudaMemcpyAsync(&tests, b->tests, sizeof(tests), cudaMemcpyDeviceToHost, st));
    LC_BP_CUDA(cudaMemcpyAsync(&err, b->err, sizeof(err), cudaMemcpyDeviceToHost, st));
    LC_BP_CUDA(cudaEventRecord(b->ev[3], st));
    LC_BP_CUDA(cudaStreamSynchronize(st));
    LC_BP_CUDA(cudaGetLastError());
    b->last_tests = tests;
    b->last_pairs = tot;
    *count = tot;
    if (err) {
        LC_BP_CUDA(cudaMemset(b->err, 0, sizeof(uint32_t)));
        if (err & ERR_SORT) return bp_fail(LC_ERR_TIMEOUT, "lc_broadphase_update: sort look-back wait exceeded its bound");
        return bp_fail(LC_ERR_STACK_OVERFLOW, "lc_broadphase_test: BVH traversal stack exceeded");
    }
    if (tot > cap && pairs)
        return bp_fail(LC_ERR_CAPACITY_OVERFLOW, "lc_broadphase_test: more pairs than cap (" + std::to_string(tot) + ")");
    return LC_OK;
}

lc_status lc_broadphase_test_host(lc_broadphase *b, uint32_t *pairs, uint64_t cap, uint64_t *count, void *stream) {
    if (!b || !count || (cap > 0 && !pairs))
        return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_test_host: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    uint64_t n = 0;
    LC_TRY_BP(lc_broadphase_test(b, nullptr, 0, &n, stream));
    const uint64_t want = std::min(n, cap);
    if (want == 0) {
        *count = n;
        return n > cap ? bp_fail(LC_ERR_CAPACITY_OVERFLOW, "lc_broadphase_test_host: more pairs than cap") : LC_OK;
    }
    if (n > b->stage_cap) {
        if (b->stage) cudaFree(b->stage);
        b->stage = nullptr;
        b->stage_cap = 0;
        if (cudaMalloc((void **)&b->stage, sizeof(uint32_t) * 2 * n) != cudaSuccess) {
            cudaGetLastError();
            return bp_fail(LC_ERR_OOM, "lc_broadphase_test_host: cudaMalloc failed for the pair staging buffer");
        }
        b->stage_cap = n;
    }
    LC_TRY_BP(lc_broadphase_test(b, b->stage, b->stage_cap, &n, stream));
    LC_BP_CUDA(cudaMemcpyAsync(pairs, b->stage, sizeof(uint32_t) * 2 * want, cudaMemcpyDeviceToHost, st));
    LC_BP_CUDA(cudaStreamSynchronize(st));
    *count = n;
    return n > cap ? bp_fail(LC_ERR_CAPACITY_OVERFLOW, "lc_broadphase_test_host: more pairs than cap") : LC_OK;
}

lc_status lc_broadphase_get_criteria(lc_broadphase *b, lc_broadphase_criteria *out) {
    if (!b || !out) return bp_fail(LC_ERR_INVALID_ARG, "lc_broadphase_get_criteria: bad arguments");
    float ms = 0.f;
    out->structure_ms = cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]) == cudaSuccess ? ms : -1.f;
    out->collision_ms = cudaEventElapsedTime(&ms, b->ev[2], b->ev[3]) == cudaSuccess ? ms : -1.f;
    cudaGetLastError();
    out->intersection_tests = b->last_tests;
    out->pairs = b->last_pairs;
    out->memory_bytes = b->bytes;
    return LC_OK;
}

lc_status lc_broadphase_destroy(lc_broadphase *b) {
    if (b) {
        cudaDeviceSynchronize();
        delete b;
    }
    return LC_OK;
}

}  // extern "C"
