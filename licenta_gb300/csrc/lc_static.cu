// lc_static.cu — lc_lbvh_pairs_static: the standalone LBVH query of
// lc_lbvh_create / lc_lbvh_build / lc_lbvh_pairs for callers that cannot
// allocate device memory.  Some hosts of this library cannot call cudaMalloc:
// code running under a custom allocator or inside a memory pool that must
// not grow, plugins loaded into a process whose device memory is owned by
// someone else, and real-time loops where an allocation (and its implicit
// device synchronisation) is not allowed.  This entry point therefore keeps
// every intermediate buffer in one scratch array compiled into the library.
//
// The scratch array lives in device memory of every GPU that loads the
// library, for the lifetime of the process.  Host code cannot use the symbol
// itself as a device address (it names a host-side stand-in), so the first
// call on each device looks the address up with cudaGetSymbolAddress while
// that device is current and keeps it for the rest of the process; a
// cudaDeviceReset invalidates it, so the entry point must not be called on a
// device after that device was reset.  Every call ends by copying the pair
// count to the host and waiting for its stream, so it cannot be issued on a
// stream that is being captured.  All calls share the one array: calls that
// overlap on the GPU (two streams, two host threads) race and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "lc_internal.cuh"

namespace lc {
void launch_leaves_from_boxes(const DevPtrs &d, const float *bmin, const float *bmax, int T, int mode,
                              cudaStream_t st);
void launch_sort(const DevPtrs &d, const int *tile_first, int passes, cudaStream_t st);
void launch_post_sort(const DevPtrs &d, cudaStream_t st);
void launch_karras(const DevPtrs &d, cudaStream_t st);
void launch_refit(const DevPtrs &d, cudaStream_t st);
void launch_traverse(const DevPtrs &d, int block, cudaStream_t st);
void scan_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap,
              uint32_t *partial, uint32_t *total_out, unsigned long long *total_out64, cudaStream_t st);

namespace {

constexpr int kStaticMaxT = LC_LBVH_STATIC_MAX_TRIANGLES;
constexpr int kStaticMaxChunk = LC_LBVH_STATIC_MAX_CHUNK;
constexpr int kStaticTiles = (kStaticMaxT + kSortTile - 1) / kSortTile;

constexpr size_t al(size_t n) { return (n + 255) & ~size_t(255); }

// Layout of the scratch array (bytes, each piece 256-byte aligned).
struct Layout {
    size_t cloth, tcloth, keys, keys_alt, payload, payload_alt, perm, perm_alt, leaf_min, leaf_max, nmin, nmax,
        parent, child, rml, visit, pair_cnt, pair_off, pair_chunk, shist, stile_cloth, stile_start, tile_first,
        scan_tmp, counters, err, npairs, total;
};

constexpr Layout make_layout() {
    Layout l{};
    size_t o = 0;
    const size_t T = kStaticMaxT, N = 2 * T - 1;
    l.cloth = o; o += al(sizeof(ClothDev));
    l.tcloth = o; o += al(4 * T);
    l.keys = o; o += al(8 * T);
    l.keys_alt = o; o += al(8 * T);
    l.payload = o; o += al(4 * T);
    l.payload_alt = o; o += al(4 * T);
    l.perm = o; o += al(4 * T);
    l.perm_alt = o; o += al(4 * T);
    l.leaf_min = o; o += al(16 * T);
    l.leaf_max = o; o += al(16 * T);
    l.nmin = o; o += al(16 * N);
    l.nmax = o; o += al(16 * N);
    l.parent = o; o += al(4 * N);
    l.child = o; o += al(8 * T);
    l.rml = o; o += al(8 * T);
    l.visit = o; o += al(4 * T);
    l.pair_cnt = o; o += al(4 * T);
    l.pair_off = o; o += al(4 * (T + 1));
    l.pair_chunk = o; o += al(4 * T * kStaticMaxChunk);
    l.shist = o; o += al(4 * kSortBuckets * (size_t)kStaticTiles);
    l.stile_cloth = o; o += al(4 * (size_t)kStaticTiles);
    l.stile_start = o; o += al(4 * (size_t)kStaticTiles);
    l.tile_first = o; o += al(8);
    l.scan_tmp = o; o += al(4 * (kScanBlocks + 1));
    l.counters = o; o += al(8 * 4);
    l.err = o; o += al(4);
    l.npairs = o; o += al(4);
    l.total = o;
    return l;
}

constexpr Layout kLayout = make_layout();

}  // namespace

// The scratch area: about 0.9 MB for 2048 triangles and chunks of 64.
static __device__ __align__(256) unsigned char g_lbvh_scratch[kLayout.total];

// Per-call set-up of the small tables that the LBVH kernels read, and the
// counters that must start at zero (the array keeps the previous call's data).
__global__ void k_static_init(ClothDev *cd, int *tcloth, int *stile_cloth, int *stile_start, int *tile_first,
                              unsigned long long *counters, uint32_t *err, int T, int chunk, int mode) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        ClothDev c;
        memset(&c, 0, sizeof(c));
        c.T = T;
        c.chunk = chunk;
        c.morton_mode = mode;
        c.leaf_quirk = 0;
        c.morton_scale = 1.f;
        *cd = c;
        const int nt = (T + kSortTile - 1) / kSortTile;
        tile_first[0] = 0;
        tile_first[1] = nt;
        for (int k = 0; k < 4; ++k) counters[k] = 0;
        *err = 0;
    }
    if (t < (T + kSortTile - 1) / kSortTile) {
        stile_cloth[t] = 0;
        stile_start[t] = t * kSortTile;
    }
    if (t < T) tcloth[t] = 0;
}

// Pair compaction into the caller's buffer, never past its capacity: one warp
// per leaf, its lanes copying consecutive pairs of the leaf's chunk, so the
// reads of the chunk and the writes of the output are coalesced.
__global__ void k_static_compact(const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ off,
                                 const uint32_t *__restrict__ chunk_area, int T, int chunk, uint2 *__restrict__ out,
                                 uint64_t cap) {
    const int s = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= T) return;
    const uint32_t n = cnt[s], o = off[s];
    for (uint32_t k = lane; k < n; k += 32)
        if ((uint64_t)o + k < cap) out[o + k] = make_uint2((uint32_t)s, chunk_area[(size_t)s * chunk + k]);
}

static std::mutex g_static_mutex;
static unsigned char *g_static_ptr[256];

// Device address of the scratch array on the current device (looked up once
// per device).
static cudaError_t scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
        if (e != cudaSuccess) return e;
        g_static_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_static_ptr[dev];
    return cudaSuccess;
}

}  // namespace lc

using namespace lc;

namespace lc {
void set_last_error(const std::string &msg);  // lc_api.cu: text for lc_last_error_string()
}

#define LC_STATIC_CUDA(call)                                                             \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            lc::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return LC_ERR_CUDA;                                                          \
        }                                                                                \
    } while (0)

extern "C" lc_status lc_lbvh_pairs_static(const float *tri_min, const float *tri_max, int32_t num_triangles,
                                          int32_t chunk_size, int32_t morton_mode, uint32_t *out_pairs, uint64_t cap,
                                          uint64_t *count, uint32_t *out_sorted_ids, void *stream) {
    if (!tri_min || !tri_max || !count || num_triangles < 2 || chunk_size < 1 ||
        (morton_mode != LC_MORTON_REF63 && morton_mode != LC_MORTON_K30)) {
        lc::set_last_error("lc_lbvh_pairs_static: bad arguments");
        return LC_ERR_INVALID_ARG;
    }
    if (num_triangles > kStaticMaxT || chunk_size > kStaticMaxChunk) {
        lc::set_last_error("lc_lbvh_pairs_static: at most LC_LBVH_STATIC_MAX_TRIANGLES (2048) triangles and "
                           "LC_LBVH_STATIC_MAX_CHUNK (64) pairs per leaf fit in the built-in scratch");
        return LC_ERR_INVALID_ARG;
    }
    if (cap && !out_pairs) {
        lc::set_last_error("lc_lbvh_pairs_static: out_pairs is NULL but cap > 0");
        return LC_ERR_INVALID_ARG;
    }
    unsigned char *base = nullptr;
    LC_STATIC_CUDA(scratch_address(&base));
    cudaStream_t st = (cudaStream_t)stream;
    const int T = num_triangles;
    const int chunk = chunk_size < T ? chunk_size : T;
    const Layout &L = kLayout;

    DevPtrs d;
    std::memset(&d, 0, sizeof(d));
    d.C = 1;
    d.Ttot = T;
    d.Ntot = 2 * T - 1;
    d.Itot = T - 1;
    d.cloth = reinterpret_cast<const ClothDev *>(base + L.cloth);
    d.tcloth = reinterpret_cast<const int *>(base + L.tcloth);
    d.keys = reinterpret_cast<unsigned long long *>(base + L.keys);
    d.keys_alt = reinterpret_cast<unsigned long long *>(base + L.keys_alt);
    d.payload = reinterpret_cast<uint32_t *>(base + L.payload);
    d.payload_alt = reinterpret_cast<uint32_t *>(base + L.payload_alt);
    d.perm = reinterpret_cast<uint32_t *>(base + L.perm);
    d.perm_alt = reinterpret_cast<uint32_t *>(base + L.perm_alt);
    d.leaf_tmp_min = reinterpret_cast<float4 *>(base + L.leaf_min);
    d.leaf_tmp_max = reinterpret_cast<float4 *>(base + L.leaf_max);
    d.nmin = reinterpret_cast<float4 *>(base + L.nmin);
    d.nmax = reinterpret_cast<float4 *>(base + L.nmax);
    d.parent = reinterpret_cast<int *>(base + L.parent);
    d.child = reinterpret_cast<int2 *>(base + L.child);
    d.rml = reinterpret_cast<int2 *>(base + L.rml);
    d.visit = reinterpret_cast<int *>(base + L.visit);
    d.pair_cnt = reinterpret_cast<uint32_t *>(base + L.pair_cnt);
    d.pair_off = reinterpret_cast<uint32_t *>(base + L.pair_off);
    d.pair_chunk = reinterpret_cast<uint32_t *>(base + L.pair_chunk);
    d.shist = reinterpret_cast<uint32_t *>(base + L.shist);
    d.stile_cloth = reinterpret_cast<const int *>(base + L.stile_cloth);
    d.stile_start = reinterpret_cast<const int *>(base + L.stile_start);
    d.nstiles = (T + kSortTile - 1) / kSortTile;
    d.scan_tmp = reinterpret_cast<uint32_t *>(base + L.scan_tmp);
    d.counters = reinterpret_cast<unsigned long long *>(base + L.counters);
    d.err = reinterpret_cast<uint32_t *>(base + L.err);
    d.pair_cap = (uint64_t)T * chunk;
    const int *tile_first = reinterpret_cast<const int *>(base + L.tile_first);
    uint32_t *npairs = reinterpret_cast<uint32_t *>(base + L.npairs);

    const int nb = (T + kThreads - 1) / kThreads;
    k_static_init<<<nb, kThreads, 0, st>>>(const_cast<ClothDev *>(d.cloth), const_cast<int *>(d.tcloth),
                                           const_cast<int *>(d.stile_cloth), const_cast<int *>(d.stile_start),
                                           const_cast<int *>(tile_first), d.counters, d.err, T, chunk, morton_mode);
    launch_leaves_from_boxes(d, tri_min, tri_max, T, morton_mode, st);
    launch_sort(d, tile_first, morton_mode == LC_MORTON_K30 ? 4 : 8, st);
    launch_post_sort(d, st);
    LC_STATIC_CUDA(cudaMemcpyAsync(d.perm, d.perm_alt, sizeof(uint32_t) * T, cudaMemcpyDeviceToDevice, st));
    LC_STATIC_CUDA(cudaMemsetAsync(d.parent, 0xFF, sizeof(int) * (size_t)d.Ntot, st));
    launch_karras(d, st);
    launch_refit(d, st);
    launch_traverse(d, 128, st);
    scan_u32(d.pair_cnt, d.pair_off, nullptr, (uint32_t)T, (uint32_t)T, d.scan_tmp, npairs, &d.counters[0], st);
    const int nwb = (T * 32 + kThreads - 1) / kThreads;  // one warp per leaf
    if (cap) k_static_compact<<<nwb, kThreads, 0, st>>>(d.pair_cnt, d.pair_off, d.pair_chunk, T, chunk,
                                                         reinterpret_cast<uint2 *>(out_pairs), cap);
    if (out_sorted_ids)
        LC_STATIC_CUDA(cudaMemcpyAsync(out_sorted_ids, d.perm, sizeof(uint32_t) * T, cudaMemcpyDeviceToDevice, st));
    LC_STATIC_CUDA(cudaGetLastError());
    uint32_t n = 0, err = 0;
    LC_STATIC_CUDA(cudaMemcpyAsync(&n, npairs, sizeof(n), cudaMemcpyDeviceToHost, st));
    LC_STATIC_CUDA(cudaMemcpyAsync(&err, d.err, sizeof(err), cudaMemcpyDeviceToHost, st));
    LC_STATIC_CUDA(cudaStreamSynchronize(st));
    *count = n;
    if (err & ERR_STACK) {
        lc::set_last_error("lc_lbvh_pairs_static: BVH traversal stack (64) exceeded");
        return LC_ERR_STACK_OVERFLOW;
    }
    if (n > cap) {
        lc::set_last_error("lc_lbvh_pairs_static: more pairs than cap; *count holds the full number");
        return LC_ERR_CAPACITY_OVERFLOW;
    }
    return LC_OK;
}
