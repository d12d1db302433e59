// lc_scan.cu — device-wide exclusive scan of u32 counts whose length may live
// in device memory (so a captured step needs no host round trip).  Replaces
// the host-synchronous CubWrap::ExclusiveSumInPlace / SelectFlagged count
// read-backs of Core/CubWrappers.cuh:26-50, 77-89.
//
// Reduce-then-scan over a fixed grid of kScanBlocks blocks: block b owns the
// contiguous range [b*chunk, (b+1)*chunk) of the n inputs, chunk a whole
// number of 2048-element tiles.  A thread's 8 values of a tile are then 32
// contiguous bytes on a 32-byte boundary (when the arrays start on 16-byte
// boundaries, as cudaMalloc's do), read and written as two 16-byte vectors.
// Deterministic.
#include "lc_internal.cuh"

namespace lc {

constexpr int kScanItems = 8;  // per thread per tile
constexpr uint32_t kScanTile = kThreads * kScanItems;

// Elements per block: ceil(n / kScanBlocks) rounded up to whole tiles.
__device__ __forceinline__ uint64_t scan_chunk(uint32_t n) {
    const uint64_t c = ((uint64_t)n + kScanBlocks - 1) / kScanBlocks;
    return (c + kScanTile - 1) / kScanTile * kScanTile;
}

__device__ __forceinline__ uint32_t scan_len(const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap) {
    uint32_t n = n_dev ? *n_dev : n_static;
    return n < n_cap ? n : n_cap;
}

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t &total) {
    __shared__ uint32_t warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < kThreads / 32 ? warp_sums[lane] : 0u;
        uint32_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < kThreads / 32) warp_sums[lane] = si - s;  // exclusive
    }
    __syncthreads();
    uint32_t excl = incl - v + warp_sums[wid];
    // total = inclusive of the last thread
    __shared__ uint32_t tot;
    if (threadIdx.x == kThreads - 1) tot = excl + v;
    __syncthreads();
    total = tot;
    __syncthreads();
    return excl;
}

__global__ void k_scan_reduce(const uint32_t *__restrict__ in, const uint32_t *n_dev, uint32_t n_static,
                              uint32_t n_cap, uint32_t *__restrict__ partial) {
    const uint32_t n = scan_len(n_dev, n_static, n_cap);
    const uint64_t chunk = scan_chunk(n);
    const uint64_t b0 = blockIdx.x * chunk;
    const uint64_t b1 = min((uint64_t)n, b0 + chunk);
    uint32_t s = 0;
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += kThreads) s += in[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ uint32_t ws[kThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kThreads / 32; ++w) t += ws[w];
        partial[blockIdx.x] = t;
    }
}

// One block of 1024 threads scans the kScanBlocks partials in place;
// partial[kScanBlocks] = total.
__global__ void k_scan_top(uint32_t *__restrict__ partial) {
    __shared__ uint32_t s[kScanBlocks];
    const int t = threadIdx.x;
    s[t] = partial[t];
    __syncthreads();
    for (int o = 1; o < kScanBlocks; o <<= 1) {
        uint32_t v = t >= o ? s[t - o] : 0u;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    partial[t] = t ? s[t - 1] : 0u;
    if (t == kScanBlocks - 1) partial[kScanBlocks] = s[t];
}

__global__ void k_scan_down(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, const uint32_t *n_dev,
                            uint32_t n_static, uint32_t n_cap, const uint32_t *__restrict__ partial,
                            uint32_t *total_out, unsigned long long *total_out64) {
    const uint32_t n = scan_len(n_dev, n_static, n_cap);
    const uint64_t chunk = scan_chunk(n);
    const uint64_t b0 = blockIdx.x * chunk;
    const uint64_t b1 = min((uint64_t)n, b0 + chunk);
    const bool vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0;
    uint32_t carry = partial[blockIdx.x];
    for (uint64_t base = b0; base < b1; base += kScanTile) {
        uint32_t vals[kScanItems];
        uint32_t local = 0;
        const uint64_t mine = base + (uint64_t)threadIdx.x * kScanItems;
        const bool full = vec && mine + kScanItems <= b1;
        if (full) {
            const uint4 a0 = *reinterpret_cast<const uint4 *>(in + mine);
            const uint4 a1 = *reinterpret_cast<const uint4 *>(in + mine + 4);
            vals[0] = a0.x; vals[1] = a0.y; vals[2] = a0.z; vals[3] = a0.w;
            vals[4] = a1.x; vals[5] = a1.y; vals[6] = a1.z; vals[7] = a1.w;
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) vals[k] = mine + k < b1 ? in[mine + k] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) local += vals[k];
        uint32_t tot;
        uint32_t ex = block_excl_scan(local, tot) + carry;
        uint32_t o[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            o[k] = ex;
            ex += vals[k];
        }
        if (full) {
            *reinterpret_cast<uint4 *>(out + mine) = make_uint4(o[0], o[1], o[2], o[3]);
            *reinterpret_cast<uint4 *>(out + mine + 4) = make_uint4(o[4], o[5], o[6], o[7]);
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k)
                if (mine + k < b1) out[mine + k] = o[k];
        }
        carry += tot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t total = partial[kScanBlocks];
        out[n] = total;
        if (total_out) *total_out = total;
        if (total_out64) *total_out64 = total;
    }
}

// out must hold n+1 entries; out[n] = total.  partial: kScanBlocks+1 u32.
void scan_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, uint32_t n_static, uint32_t n_cap,
              uint32_t *partial, uint32_t *total_out, unsigned long long *total_out64, cudaStream_t st) {
    k_scan_reduce<<<kScanBlocks, kThreads, 0, st>>>(in, n_dev, n_static, n_cap, partial);
    k_scan_top<<<1, kScanBlocks, 0, st>>>(partial);
    k_scan_down<<<kScanBlocks, kThreads, 0, st>>>(in, out, n_dev, n_static, n_cap, partial, total_out, total_out64);
}

}  // namespace lc
