// lc_lbvh.cu — triangle boxes + Morton codes, segmented stable radix sort,
// Karras hierarchy, bottom-up refit, leaf-vs-tree traversal, pair
// compaction and the VF/EE narrowphase (feature AABB cull + CCD).
//
// Compiled with -fmad=false: every float expression here keeps the separate
// roundings of the reference kernels, so Morton codes, tree topology, pair
// lists and contact lists are bit-exact against the FP32 oracle for the
// same input positions.
#include <cuda/atomic>

#include "lc_internal.cuh"

namespace lc {

// ---------------------------------------------------------------------------
// Morton encoding: Core/CudaUtils.cu:278-325 (REF63) and the commented 30-bit
// variant at :289-308 (K30).  Bit k of an axis goes to bit 3k.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ unsigned long long spread21(unsigned long long v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__host__ __device__ __forceinline__ unsigned long long spread10(unsigned long long v) {
    v &= 0x3ffull;
    v = (v | (v << 16)) & 0x30000ffull;
    v = (v | (v << 8)) & 0x300f00full;
    v = (v | (v << 4)) & 0x30c30c3ull;
    v = (v | (v << 2)) & 0x9249249ull;
    return v;
}
__host__ __device__ __forceinline__ unsigned long long morton3(float x, float y, float z, int mode) {
    if (mode == LC_MORTON_K30) {
        unsigned long long qx = (unsigned long long)fminf(fmaxf(x * 1024.f, 0.0f), 1023.0f);
        unsigned long long qy = (unsigned long long)fminf(fmaxf(y * 1024.f, 0.0f), 1023.0f);
        unsigned long long qz = (unsigned long long)fminf(fmaxf(z * 1024.f, 0.0f), 1023.0f);
        return (spread10(qx) << 2) + (spread10(qy) << 1) + spread10(qz);
    }
    unsigned long long qx = (unsigned long long)fminf(fmaxf(x * 2097152.f, 0.0f), 2097151.0f);
    unsigned long long qy = (unsigned long long)fminf(fmaxf(y * 2097152.f, 0.0f), 2097151.0f);
    unsigned long long qz = (unsigned long long)fminf(fmaxf(z * 2097152.f, 0.0f), 2097151.0f);
    return (spread21(qx) << 2) + (spread21(qy) << 1) + spread21(qz);
}

unsigned long long morton3_host(float x, float y, float z, int mode) { return morton3(x, y, z, mode); }

// ---------------------------------------------------------------------------
// Triangle update: Physics/CudaDeformableUtils.cu:120-151.  One thread per
// slot; the swept, thickness-inflated box goes to leaf (T-1+slot) — the
// pre-sort slot, which is the reference's leaf-AABB quirk — or to a
// temporary that the post-sort gather places under the sorted leaf.
// ---------------------------------------------------------------------------
__global__ void k_triangles(DevPtrs d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.Ttot) return;
    const int c = d.tcloth[s];
    const ClothDev &cd = d.cloth[c];
    const int local = s - cd.t_off;
    const uint32_t orig = d.perm[s];
    const int4 t = d.tri[orig];
    const float3 a = xyz(d.x[t.x]), b = xyz(d.x[t.y]), cc = xyz(d.x[t.z]);
    const float3 pa = xyz(d.xp[t.x]), pb = xyz(d.xp[t.y]), pc = xyz(d.xp[t.z]);
    const float h = cd.h;
    d.fn[orig] = f4(normalize(cross(sub(b, a), sub(cc, a))), 0.f);
    const float3 mn = subc(min3(a, b, cc), h), mx = addc(max3(a, b, cc), h);
    const float3 pmn = subc(min3(pa, pb, pc), h), pmx = addc(max3(pa, pb, pc), h);
    const float3 smn = vmin(mn, pmn), smx = vmax(mx, pmx);
    if (cd.leaf_quirk) {
        const int node = cd.n_off + (cd.T - 1) + local;
        d.nmin[node] = f4(smn, 0.f);
        d.nmax[node] = f4(smx, 0.f);
    } else {
        d.leaf_tmp_min[s] = f4(smn, 0.f);
        d.leaf_tmp_max[s] = f4(smx, 0.f);
    }
    const float3 mid = add(smn, dvs(sub(smx, smn), 2.f));
    const float qx = (mid.x - cd.morton_origin[0]) * cd.morton_scale;
    const float qy = (mid.y - cd.morton_origin[1]) * cd.morton_scale;
    const float qz = (mid.z - cd.morton_origin[2]) * cd.morton_scale;
    d.keys[s] = morton3(qx, qy, qz, cd.morton_mode);
    d.payload[s] = (uint32_t)local;
}

// Standalone LBVH: leaf boxes supplied by the caller (one cloth, T slots).
__global__ void k_leaves_from_boxes(DevPtrs d, const float *__restrict__ bmin, const float *__restrict__ bmax,
                                    int T, int mode) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= T) return;
    const float3 mn = f3(bmin[3 * s], bmin[3 * s + 1], bmin[3 * s + 2]);
    const float3 mx = f3(bmax[3 * s], bmax[3 * s + 1], bmax[3 * s + 2]);
    d.leaf_tmp_min[s] = f4(mn, 0.f);
    d.leaf_tmp_max[s] = f4(mx, 0.f);
    const float3 mid = add(mn, dvs(sub(mx, mn), 2.f));
    d.keys[s] = morton3(mid.x, mid.y, mid.z, mode);
    d.payload[s] = (uint32_t)s;
    d.perm[s] = (uint32_t)s;
}

// ---------------------------------------------------------------------------
// Segmented stable LSD radix sort of (u64 key, u32 payload), 8-bit digits.
// Tiles never straddle cloths, so every pass ranks keys within their own
// cloth: the result equals a stable sort of each cloth's slots by key, the
// order CUB's SortPairs gives at Physics/CudaDeformableUtils.cu:346-349.
// ---------------------------------------------------------------------------
__global__ void k_sort_hist(DevPtrs d, const unsigned long long *__restrict__ keys, int shift) {
    __shared__ uint32_t hist[kSortBuckets];
    const int tile = blockIdx.x;
    for (int i = threadIdx.x; i < kSortBuckets; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const int c = d.stile_cloth[tile];
    const int start = d.stile_start[tile];
    const ClothDev &cd = d.cloth[c];
    const int end = min(start + kSortTile, cd.t_off + cd.T);
    for (int i = start + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t dig = (uint32_t)(keys[i] >> shift) & (kSortBuckets - 1);
        atomicAdd(&hist[dig], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kSortBuckets; i += blockDim.x) d.shist[(size_t)tile * kSortBuckets + i] = hist[i];
}

// One block per cloth: turns the per-tile digit counts into global scatter
// offsets (digit-major, tile-minor within the cloth).  kOffsetsSplit threads
// per digit each take a contiguous quarter of the cloth's tiles, with their
// loads unrolled, so a cloth of hundreds of tiles (one segment of a million
// keys) is not one serial chain of loads per digit.
constexpr int kOffsetsSplit = 4;
__global__ void __launch_bounds__(kSortBuckets * kOffsetsSplit) k_sort_offsets(DevPtrs d,
                                                                               const int *__restrict__ tile_first) {
    const int c = blockIdx.x;
    const int d0 = threadIdx.x % kSortBuckets, q = threadIdx.x / kSortBuckets;
    const int t0 = tile_first[c], t1 = tile_first[c + 1];
    const int per = (t1 - t0 + kOffsetsSplit - 1) / kOffsetsSplit;
    const int a = min(t1, t0 + q * per), e = min(t1, a + per);
    uint32_t part = 0;
#pragma unroll 8
    for (int t = a; t < e; ++t) part += d.shist[(size_t)t * kSortBuckets + d0];
    __shared__ uint32_t qs[kOffsetsSplit][kSortBuckets];
    __shared__ uint32_t s[kSortBuckets];
    qs[q][d0] = part;
    __syncthreads();
    // digit totals, then their exclusive scan (threads of quarter 0)
    uint32_t tot = 0;
    if (q == 0) {
#pragma unroll
        for (int k = 0; k < kOffsetsSplit; ++k) tot += qs[k][d0];
        s[d0] = tot;
    }
    __syncthreads();
    for (int o = 1; o < kSortBuckets; o <<= 1) {
        const uint32_t v = (q == 0 && d0 >= o) ? s[d0 - o] : 0u;
        __syncthreads();
        if (q == 0) s[d0] += v;
        __syncthreads();
    }
    if (q == 0) s[d0] -= tot;  // exclusive
    __syncthreads();
    uint32_t run = (uint32_t)d.cloth[c].t_off + s[d0];
    for (int k = 0; k < q; ++k) run += qs[k][d0];
#pragma unroll 8
    for (int t = a; t < e; ++t) {
        const size_t k = (size_t)t * kSortBuckets + d0;
        const uint32_t n = d.shist[k];
        d.shist[k] = run;
        run += n;
    }
}

// One-sweep offsets (every sort with look-back scratch; the allocation-free
// entry keeps the per-pass histogram above).  k_sort_hist_all reads each
// tile's keys once and adds the digit counts of every pass to its segment's
// totals, so the digits' first positions in the segment are known before
// the first pass; the scatter of a pass then finds a tile's place among its
// segment's earlier tiles by a decoupled look-back over per-tile, per-digit
// status words (flag in the top two bits: aggregate of the tile alone, or
// inclusive prefix from the segment's first tile).  Tiles take their
// position from a ticket counter, so a block only ever waits on blocks that
// started before it.  The offsets are the numbers k_sort_offsets gives.
constexpr uint32_t kStatAgg = 1u << 30, kStatPre = 2u << 30, kStatCount = kStatAgg - 1;
constexpr uint32_t kLookbackSpins = 1u << 22;  // bound on the status waits of one look-back (then ERR_SORT)
constexpr int kLookbackWindow = 8;               // earlier tiles' statuses read per look-back step
__global__ void __launch_bounds__(kThreads) k_sort_hist_all(DevPtrs d, const unsigned long long *__restrict__ keys,
                                                            int passes) {
    static_assert(kThreads == kSortBuckets, "one thread per digit");
    constexpr int R = kSortTile / kThreads;
    __shared__ uint32_t h[kSortPassesMax][kSortBuckets];
    const int tile = blockIdx.x, t = threadIdx.x, lane = t & 31;
    const int c = d.stile_cloth[tile];
    const int start = d.stile_start[tile];
    const ClothDev &cd = d.cloth[c];
    const int n = min(kSortTile, cd.t_off + cd.T - start);
    for (int p = 0; p < passes; ++p) {
        h[p][t] = 0;
        d.sstat[((size_t)p * d.nstiles + tile) * kSortBuckets + t] = 0;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int li = r * kThreads + t;
        const bool valid = li < n;
        const unsigned long long key = valid ? keys[start + li] : 0ull;
        for (int p = 0; p < passes; ++p) {
            // a digit common to the whole warp (the high digits of nearby
            // Morton codes) is one atomic; otherwise one per lane
            const uint32_t dig = valid ? (uint32_t)(key >> (p * kSortBits)) & (kSortBuckets - 1) : kSortBuckets;
            const uint32_t d0 = __shfl_sync(0xffffffffu, dig, 0);
            if (__all_sync(0xffffffffu, dig == d0)) {
                if (lane == 0 && d0 < kSortBuckets) atomicAdd(&h[p][d0], 32u);
            } else if (valid) {
                atomicAdd(&h[p][dig], 1u);
            }
        }
    }
    __syncthreads();
    uint32_t *seg = d.sseg + kSortPassesMax + (size_t)c * kSortPassesMax * kSortBuckets;
    for (int p = 0; p < passes; ++p)
        if (h[p][t]) atomicAdd(&seg[p * kSortBuckets + t], h[p][t]);
}

// One tile per block, ranked without block-wide rounds: warp w takes the
// tile's keys [256 w, 256 w + 256) in 8 steps of 32 and ranks each key among
// the warp's earlier keys of its digit (warp-private counts, no block
// barrier); one scan per digit over the warps then gives every key its slot
// in the tile sorted by digit, stable because index order is (warp, step,
// lane).  The sorted tile is staged in shared memory and written out with
// consecutive threads on consecutive slots of each digit's run.  With
// kLookback the tile's global slots come from the one-sweep look-back
// (tiles in ticket order), otherwise from k_sort_offsets.
template <bool kLookback>
__global__ void __launch_bounds__(kThreads, 4) k_sort_scatter(DevPtrs d, const unsigned long long *__restrict__ kin,
                                                           const uint32_t *__restrict__ pin,
                                                           unsigned long long *__restrict__ kout,
                                                           uint32_t *__restrict__ pout, int shift, int pass,
                                                           const int *__restrict__ tile_first) {
    constexpr int W = kThreads / 32;
    constexpr int R = kSortTile / kThreads;  // keys per lane
    static_assert(kThreads == kSortBuckets && kSortTile == W * 32 * R, "one thread per digit, 32 R keys per warp");
    __shared__ uint32_t wcnt[W][kSortBuckets];  // per warp: keys of each digit (then: first tile slot)
    __shared__ uint32_t lbase[kSortBuckets];    // first tile slot per digit
    __shared__ uint32_t gbase[kSortBuckets];    // first global slot per digit
    __shared__ uint32_t wsum[W], wseg[W];
    __shared__ unsigned long long skey[kSortTile];
    __shared__ uint32_t spay[kSortTile];
    __shared__ int s_tile, s_bad;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    if (kLookback) {
        if (t == 0) {
            s_tile = (int)atomicAdd(&d.sseg[pass], 1u);
            s_bad = 0;
        }
        __syncthreads();
    }
    const int tile = kLookback ? s_tile : (int)blockIdx.x;
    const int c = d.stile_cloth[tile];
    const int start = d.stile_start[tile];
    const ClothDev &cd = d.cloth[c];
    const int n = min(kSortTile, cd.t_off + cd.T - start);
    if (!kLookback) gbase[t] = d.shist[(size_t)tile * kSortBuckets + t];
#pragma unroll
    for (int w = 0; w < W; ++w) wcnt[w][t] = 0;
    __syncthreads();
    const uint32_t lt_mask = (1u << lane) - 1u;
    unsigned long long kr[R];
    uint32_t pr[R], rk[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int li = wid * 32 * R + r * 32 + lane;
        const bool valid = li < n;
        kr[r] = valid ? kin[start + li] : 0ull;
        pr[r] = valid ? pin[start + li] : 0u;
        const uint32_t dig = valid ? (uint32_t)(kr[r] >> shift) & (kSortBuckets - 1) : kSortBuckets;
        const uint32_t peers = __match_any_sync(0xffffffffu, dig);
        const uint32_t before = valid ? wcnt[wid][dig] : 0u;
        rk[r] = before + __popc(peers & lt_mask);
        __syncwarp();
        if (valid && (peers & lt_mask) == 0) wcnt[wid][dig] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // thread t owns digit t: its tile total, then the exclusive scan of the
    // totals over the digits (first slot of the digit) and over the warps
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) tot += wcnt[w][t];
    // one-sweep: publish the tile's count of digit t, and scan the segment's
    // digit totals (the digits' first positions in the segment)
    uint32_t *stat = nullptr;
    int first = 0;
    uint32_t segtot = 0, segincl = 0;
    if (kLookback) {
        first = tile_first[c];
        stat = d.sstat + (size_t)pass * d.nstiles * kSortBuckets;
        cuda::atomic_ref<uint32_t, cuda::thread_scope_device>(stat[(size_t)tile * kSortBuckets + t])
            .store((tile == first ? kStatPre : kStatAgg) | tot, cuda::memory_order_relaxed);
        segtot = segincl = d.sseg[kSortPassesMax + ((size_t)c * kSortPassesMax + pass) * kSortBuckets + t];
    }
    uint32_t incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
        if (kLookback) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, segincl, o);
            if (lane >= o) segincl += u;
        }
    }
    if (lane == 31) {
        wsum[wid] = incl;
        if (kLookback) wseg[wid] = segincl;
    }
    __syncthreads();
    uint32_t run = incl - tot;
    for (int w = 0; w < wid; ++w) run += wsum[w];
    lbase[t] = run;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const uint32_t v = wcnt[w][t];
        wcnt[w][t] = run;
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int li = wid * 32 * R + r * 32 + lane;
        if (li < n) {
            const uint32_t dig = (uint32_t)(kr[r] >> shift) & (kSortBuckets - 1);
            const uint32_t pos = wcnt[wid][dig] + rk[r];
            skey[pos] = kr[r];
            spay[pos] = pr[r];
        }
    }
    if (kLookback) {
        // the tile's place among the segment's earlier tiles, digit t: sum
        // the aggregates back to the first inclusive prefix
        // A window of kLookbackWindow earlier tiles is read at once (the
        // segment's first tile always holds its inclusive prefix, so the
        // walk never passes it); a window that meets an unpublished tile
        // resumes there.
        uint32_t excl = 0;
        if (tile != first) {
            uint32_t spins = 0;
            for (int j = tile - 1;;) {
                uint32_t sv[kLookbackWindow];
#pragma unroll
                for (int k = 0; k < kLookbackWindow; ++k)
                    sv[k] = j - k >= first ? cuda::atomic_ref<uint32_t, cuda::thread_scope_device>(
                                                 stat[(size_t)(j - k) * kSortBuckets + t])
                                                 .load(cuda::memory_order_relaxed)
                                           : kStatPre;
                bool done = false;
                int k = 0;
                for (; k < kLookbackWindow; ++k) {
                    if (sv[k] == 0) break;  // not published yet
                    excl += sv[k] & kStatCount;
                    if ((sv[k] & ~kStatCount) == kStatPre || j - k == first) {
                        done = true;
                        break;
                    }
                }
                if (done) break;
                j -= k;
                if (k == 0) {
                    if (++spins > kLookbackSpins) {
                        s_bad = 1;
                        atomicOr(d.err, ERR_SORT);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            // published even after a failed wait, so that later tiles end
            cuda::atomic_ref<uint32_t, cuda::thread_scope_device>(stat[(size_t)tile * kSortBuckets + t])
                .store(kStatPre | (excl + tot), cuda::memory_order_relaxed);
        }
        uint32_t dbase = segincl - segtot;
        for (int w = 0; w < wid; ++w) dbase += wseg[w];
        gbase[t] = (uint32_t)cd.t_off + dbase + excl;
    }
    __syncthreads();
    if (kLookback && s_bad) return;
    const uint32_t lo = (uint32_t)cd.t_off, hi = (uint32_t)(cd.t_off + cd.T);
    for (int i = t; i < n; i += kThreads) {
        const unsigned long long key = skey[i];
        const uint32_t dig = (uint32_t)(key >> shift) & (kSortBuckets - 1);
        const uint32_t g = gbase[dig] + (uint32_t)i - lbase[dig];
        if (kLookback && (g < lo || g >= hi)) {  // only after a failed wait elsewhere
            atomicOr(d.err, ERR_SORT);
            continue;
        }
        kout[g] = key;
        pout[g] = spay[i];
    }
}

// After the sort: new triangle order and (fixed mode) leaf boxes gathered by
// the permutation.
__global__ void k_post_sort(DevPtrs d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.Ttot) return;
    const int c = d.tcloth[s];
    const ClothDev &cd = d.cloth[c];
    const int src = cd.t_off + (int)d.payload[s];
    const uint32_t orig = d.perm[src];
    d.perm_alt[s] = orig;
    if (d.tri_slot) d.tri_slot[s] = d.tri[orig];  // one gather per slot instead of two per pair
    if (!cd.leaf_quirk) {
        const int node = cd.n_off + (cd.T - 1) + (s - cd.t_off);
        d.nmin[node] = d.leaf_tmp_min[src];
        d.nmax[node] = d.leaf_tmp_max[src];
    }
}

// ---------------------------------------------------------------------------
// Karras hierarchy: Collision/CudaBVH.cu:163-242, Core/CudaUtils.cu:338-362.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int delta(const unsigned long long *__restrict__ m, int i, int j, int maxi) {
    if (j < 0 || j > maxi) return -1;
    const unsigned long long x = m[i] ^ m[j];
    return x ? __clzll((long long)x) : __clzll((long long)((unsigned long long)i ^ (unsigned long long)j)) + 64;
}
__device__ __forceinline__ int sgn_ref(int a) { return signbit((float)a) ? -1 : 1; }

__global__ void k_karras(DevPtrs d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0 && d.nrexit) *d.nrexit = 0;  // k_refit_local appends to it
    if (s >= d.Ttot) return;
    const int c = d.tcloth[s];
    const ClothDev &cd = d.cloth[c];
    const int id = s - cd.t_off;
    const int In = cd.T - 1;
    if (id >= In) return;
    const unsigned long long *m = d.keys + cd.t_off;
    // FindRange
    const int dd = sgn_ref(delta(m, id, id + 1, In) - delta(m, id, id - 1, In));
    const int delmin = delta(m, id, id - dd, In);
    int lmax = 2;
    while (delta(m, id, id + lmax * dd, In) > delmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(m, id, id + (l + t) * dd, In) > delmin) l += t;
    const int j = id + l * dd;
    const int first = min(id, j), last = max(id, j);
    // FindSplit (code-only prefix)
    int split;
    const unsigned long long fc = m[first], lc = m[last];
    if (fc == lc) {
        split = (first + last) >> 1;
    } else {
        const int com = __clzll((long long)(fc ^ lc));
        split = first;
        int step = last - first;
        do {
            step = (step + 1) >> 1;
            const int ns = split + step;
            if (ns < last) {
                if (__clzll((long long)(fc ^ m[ns])) > com) split = ns;
            }
        } while (step > 1);
    }
    const int left = split == first ? In + split : split;
    const int right = split + 1 == last ? In + split + 1 : split + 1;
    d.child[cd.i_off + id] = make_int2(left, right);
    if (d.nend) d.nend[cd.i_off + id] = j;
    // An internal node that the refit never reaches (possible only when a run
    // of >= 3 equal codes makes two nodes claim one child) keeps stale data in
    // the reference; here it keeps zeros, deterministically.
    d.nmin[cd.n_off + id] = make_float4(0.f, 0.f, 0.f, 0.f);
    d.nmax[cd.n_off + id] = make_float4(0.f, 0.f, 0.f, 0.f);
    d.rml[cd.i_off + id] = make_int2(0, 0);
    // The reference's parents[] write race resolved as "largest parent wins".
    atomicMax(&d.parent[cd.n_off + left], id);
    atomicMax(&d.parent[cd.n_off + right], id);
    d.visit[cd.i_off + id] = 0;
}

// Bottom-up refit: Collision/CudaBVH.cu:128-149.  The second arrival at a
// node unions its children; the arrival counter is an acq_rel atomic, which
// orders the child writes before it, and the children are re-read from L2.
// refit_climb starts at node pid, arriving from a child whose box is written.
__device__ __forceinline__ void refit_climb(const DevPtrs &d, const ClothDev &cd, int pid) {
    const int In = cd.T - 1;
    for (int guard = 0; guard <= cd.T; ++guard) {
        if (pid < 0 || pid >= In) {
            if (pid != 0) atomicOr(d.err, ERR_TREE);
            return;
        }
        // child ids and parent links come from k_karras (an earlier launch):
        // they are read ahead of the counter, so their round trip overlaps
        // the release below instead of following the acquire
        const int2 ch = __ldg(&d.child[cd.i_off + pid]);
        const int up = pid ? __ldg(&d.parent[cd.n_off + pid]) : 0;
        // acq_rel at device scope: releases this thread's writes of the child
        // it came from, and the second arrival acquires the first one's
        // (the reference's arrival counter has no ordering at all)
        cuda::atomic_ref<int, cuda::thread_scope_device> visit(d.visit[cd.i_off + pid]);
        if (visit.fetch_add(1, cuda::memory_order_acq_rel) == 0) return;
        const float4 lmn = __ldcg(&d.nmin[cd.n_off + ch.x]), lmx = __ldcg(&d.nmax[cd.n_off + ch.x]);
        const float4 rmn = __ldcg(&d.nmin[cd.n_off + ch.y]), rmx = __ldcg(&d.nmax[cd.n_off + ch.y]);
        d.nmin[cd.n_off + pid] = f4(vmin(xyz(lmn), xyz(rmn)), 0.f);
        d.nmax[cd.n_off + pid] = f4(vmax(xyz(lmx), xyz(rmx)), 0.f);
        int rl, rr;
        if (ch.x >= In) rl = ch.x;
        else { const int2 q = __ldcg(&d.rml[cd.i_off + ch.x]); rl = max(q.x, q.y); }
        if (ch.y >= In) rr = ch.y;
        else { const int2 q = __ldcg(&d.rml[cd.i_off + ch.y]); rr = max(q.x, q.y); }
        d.rml[cd.i_off + pid] = make_int2(rl, rr);
        if (pid == 0) return;
        pid = up;
    }
    atomicOr(d.err, ERR_TREE);
}

// One thread per leaf, the whole climb in L2 (the allocation-free entry).
__global__ void k_refit(DevPtrs d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.Ttot) return;
    const ClothDev &cd = d.cloth[d.tcloth[s]];
    const int id = s - cd.t_off;
    const int In = cd.T - 1;
    if (In <= 0) return;
    refit_climb(d, cd, d.parent[cd.n_off + In + id]);
}

// The same refit in two launches.  k_refit_local: block b owns the slots
// [256 b, 256 b + 256); an internal node whose leaf range [min(i, j),
// max(i, j)] lies inside one block (node i sits at one end of its range, so
// its slot is inside too) is "local": its arrival counter, box and rightmost
// leaves live in that block's shared memory (block-scope acq_rel counter),
// and its box is also written out.  A thread that reaches a node whose
// range crosses a block boundary stops there and leaves the arrival to
// k_refit_upper (each thread leaves at most one); the block writes its
// arrivals out densely, one global atomic per block.  k_refit_upper then
// climbs from the few left arrivals in L2 as k_refit does, so no block of
// the launch over all leaves waits on a climb to the root.
// Every arrival at a local node comes from inside its block: the ranges
// come from the index-tiebroken prefix (unique keys), so any two ranges are
// nested or disjoint, and an internal child is strictly inside its
// parent's range (a child at the range's end is a leaf), so its own range
// lies inside too -- also where equal codes make two nodes claim one child.
// Shared boxes start at zero, like the global ones k_karras clears.
__global__ void __launch_bounds__(kThreads) k_refit_local(DevPtrs d) {
    __shared__ float4 s_lmin[kThreads], s_lmax[kThreads];  // the block's leaves
    __shared__ float4 s_min[kThreads], s_max[kThreads];    // local internal nodes, by slot
    __shared__ int2 s_rml[kThreads];
    __shared__ int s_visit[kThreads];
    __shared__ int2 s_exit[kThreads];
    __shared__ uint32_t s_nexit, s_base;
    const int tid = threadIdx.x;
    const int B0 = blockIdx.x * kThreads, B1 = min(B0 + kThreads, d.Ttot);
    const int s = B0 + tid;
    const bool valid = s < d.Ttot;
    int c = 0, id = 0, In = 0;
    const ClothDev *cdp = nullptr;
    s_visit[tid] = 0;
    s_min[tid] = s_max[tid] = make_float4(0.f, 0.f, 0.f, 0.f);
    s_rml[tid] = make_int2(0, 0);
    if (tid == 0) s_nexit = 0;
    if (valid) {
        c = d.tcloth[s];
        cdp = &d.cloth[c];
        id = s - cdp->t_off;
        In = cdp->T - 1;
        s_lmin[tid] = __ldg(&d.nmin[cdp->n_off + In + id]);
        s_lmax[tid] = __ldg(&d.nmax[cdp->n_off + In + id]);
    }
    __syncthreads();
    if (valid && In > 0) {
        const ClothDev &cd = *cdp;
        const int base = cd.t_off - B0;  // cloth-local index -> block slot
        int pid = d.parent[cd.n_off + In + id];
        for (int guard = 0;; ++guard) {
            if (guard > cd.T) {
                atomicOr(d.err, ERR_TREE);
                break;
            }
            if (pid < 0 || pid >= In) {
                if (pid != 0) atomicOr(d.err, ERR_TREE);
                break;
            }
            const int je = __ldg(&d.nend[cd.i_off + pid]);
            const int lo = min(pid, je) + base, hi = max(pid, je) + base;
            if (lo < 0 || hi >= B1 - B0) {  // crosses a block boundary: the upper pass arrives
                const uint32_t e = atomicAdd(&s_nexit, 1u);
                s_exit[e] = make_int2(c, pid);
                break;
            }
            const int2 ch = __ldg(&d.child[cd.i_off + pid]);
            const int up = pid ? __ldg(&d.parent[cd.n_off + pid]) : 0;
            cuda::atomic_ref<int, cuda::thread_scope_block> visit(s_visit[pid + base]);
            if (visit.fetch_add(1, cuda::memory_order_acq_rel) == 0) break;
            const bool la = ch.x >= In, lb = ch.y >= In;
            const int ia = (la ? ch.x - In : ch.x) + base, ib = (lb ? ch.y - In : ch.y) + base;
            if (ia < 0 || ia >= B1 - B0 || ib < 0 || ib >= B1 - B0) {  // children outside the range: not a tree
                atomicOr(d.err, ERR_TREE);
                break;
            }
            const float4 amn = la ? s_lmin[ia] : s_min[ia], amx = la ? s_lmax[ia] : s_max[ia];
            const float4 bmn = lb ? s_lmin[ib] : s_min[ib], bmx = lb ? s_lmax[ib] : s_max[ib];
            const float4 mn = f4(vmin(xyz(amn), xyz(bmn)), 0.f), mx = f4(vmax(xyz(amx), xyz(bmx)), 0.f);
            int rl, rr;
            if (la) rl = ch.x;
            else { const int2 q = s_rml[ia]; rl = max(q.x, q.y); }
            if (lb) rr = ch.y;
            else { const int2 q = s_rml[ib]; rr = max(q.x, q.y); }
            s_min[pid + base] = mn;
            s_max[pid + base] = mx;
            s_rml[pid + base] = make_int2(rl, rr);
            d.nmin[cd.n_off + pid] = mn;
            d.nmax[cd.n_off + pid] = mx;
            d.rml[cd.i_off + pid] = make_int2(rl, rr);
            if (pid == 0) break;
            pid = up;
        }
    }
    __syncthreads();
    if (tid == 0) s_base = s_nexit ? atomicAdd(d.nrexit, s_nexit) : 0u;
    __syncthreads();
    if ((uint32_t)tid < s_nexit) d.rexit[s_base + tid] = s_exit[tid];
}
__global__ void k_refit_upper(DevPtrs d) {
    const uint32_t n = *d.nrexit;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int2 x = d.rexit[e];
        refit_climb(d, d.cloth[x.x], x.y);
    }
}

// Wide node records for the traversal: per internal node both children's
// boxes, with the child ids and rightmost leaves in the w lanes, so that one
// node visit is one contiguous 64-byte read instead of six dependent ones.
// A separate pass after the refit, not part of it: a node the refit never
// reaches (a run of >= 3 equal codes, see k_karras) still gets its record
// from its children's boxes, as the per-node reads of the traversal see them.
__global__ void k_pack_nodes(DevPtrs d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.Ttot) return;
    const ClothDev &cd = d.cloth[d.tcloth[s]];
    const int k = s - cd.t_off;
    if (k >= cd.T - 1) return;
    const int2 ch = d.child[cd.i_off + k], rm = d.rml[cd.i_off + k];
    const float4 *nmin = d.nmin + cd.n_off, *nmax = d.nmax + cd.n_off;
    const float4 a = nmin[ch.x], b = nmax[ch.x], c = nmin[ch.y], e = nmax[ch.y];
    float4 *w = d.wnode + 4 * (size_t)(cd.i_off + k);
    w[0] = make_float4(a.x, a.y, a.z, __int_as_float(ch.x));
    w[1] = make_float4(b.x, b.y, b.z, __int_as_float(rm.x));
    w[2] = make_float4(c.x, c.y, c.z, __int_as_float(ch.y));
    w[3] = make_float4(e.x, e.y, e.z, __int_as_float(rm.y));
}

// Leaf-vs-tree traversal: Collision/CudaBVH.cu:23-113.  Pairs (i, j>i) in
// left-first DFS order, at most `chunk` per leaf, the rest counted as dropped.
__global__ void k_traverse(DevPtrs d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.Ttot) return;
    const int c = d.tcloth[s];
    const ClothDev &cd = d.cloth[c];
    const int id = s - cd.t_off;
    const int In = cd.T - 1;
    if (In <= 0) { d.pair_cnt[s] = 0; return; }
    const int me = In + id;
    const int chunk = cd.chunk;
    uint32_t *out = d.pair_chunk + cd.pc_off + (int64_t)id * chunk;
    const float4 *nmin = d.nmin + cd.n_off, *nmax = d.nmax + cd.n_off;
    const int2 *child = d.child + cd.i_off, *rml = d.rml + cd.i_off;
    const float3 amin = xyz(nmin[me]), amax = xyz(nmax[me]);
    int stack[kTraverseStack];
    stack[0] = -1;
    int top = 1, node = 0, got = 0;
    uint32_t dropped = 0;
    const int guard_max = 4 * cd.T + 64;
    for (int guard = 0; guard < guard_max; ++guard) {
        const int2 ch = __ldg(&child[node]);
        const int2 rm = __ldg(&rml[node]);
        bool ol = false, orr = false;
        if (rm.x > me && overlap(amin, amax, xyz(__ldg(&nmin[ch.x])), xyz(__ldg(&nmax[ch.x])))) ol = true;
        if (rm.y > me && overlap(amin, amax, xyz(__ldg(&nmin[ch.y])), xyz(__ldg(&nmax[ch.y])))) orr = true;
        if (ol && ch.x >= In) {
            if (got < chunk) out[got++] = (uint32_t)(ch.x - In);
            else ++dropped;
        }
        if (orr && ch.y >= In) {
            if (got < chunk) out[got++] = (uint32_t)(ch.y - In);
            else ++dropped;
        }
        const bool tl = ol && ch.x < In, tr = orr && ch.y < In;
        if (!tl && !tr) {
            node = stack[--top];
        } else {
            node = tl ? ch.x : ch.y;
            if (tl && tr) {
                if (top >= kTraverseStack) { atomicOr(d.err, ERR_STACK); break; }
                stack[top++] = ch.y;
            }
        }
        if (top == 0) break;
    }
    d.pair_cnt[s] = (uint32_t)got;
    if (dropped) atomicAdd(&d.counters[3], (unsigned long long)dropped);
}



// The traversal as a packet: a left-first depth-first walk of a Karras tree
// meets the leaves in increasing index order, so leaf i's result is the
// increasing list of leaves j > i whose boxes overlap its own, cut at the
// chunk size.  A warp walks the tree once for its 32 consecutive leaves
// (spatially close in Morton order): every node record is read once for the
// warp, each lane tests its own box (and rightmost-leaf bound) against the
// two children, and the warp descends into a child when any lane needs it.
// Each lane keeps exactly the leaves it overlaps, in the walk's order, so
// every chunk is the single-leaf traversal's.  A warp whose leaves span two
// cloths walks each cloth's tree for its own lanes.
// At most 40 registers (6 blocks of 256, or 12 of 128, per SM): the walk
// waits on dependent node fetches, and 12 resident 4-warp blocks hide more of
// that latency than the 10 that 41 registers allowed.
__global__ void __launch_bounds__(kTraverseBlockMax, 6) k_traverse_packet(DevPtrs d) {
    static_assert(kTraverseStack == 64, "two stack slots per lane");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // the warp's stack in registers: slot k in lane k % 32, register k / 32
    int stk0 = 0, stk1 = 0;
    const int s = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 + lane;
    const bool valid = s < d.Ttot;
    int c = -1, me = 0, got = 0, chunk = 0;
    uint32_t dropped = 0;
    uint32_t *out = nullptr;
    float3 amin = f3(0.f, 0.f, 0.f), amax = amin;
    bool has_tree = false;
    if (valid) {
        c = d.tcloth[s];
        const ClothDev &cd = d.cloth[c];
        const int id = s - cd.t_off, In = cd.T - 1;
        has_tree = In > 0;
        me = In + id;
        chunk = cd.chunk;
        out = d.pair_chunk + cd.pc_off + (int64_t)id * chunk;
        if (has_tree) {
            amin = xyz(d.nmin[cd.n_off + me]);
            amax = xyz(d.nmax[cd.n_off + me]);
        }
    }
    unsigned pending = __ballot_sync(full, has_tree);
    bool overflow = false;
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int cc = __shfl_sync(full, c, leader);
        const bool mine = ((pending >> lane) & 1u) && c == cc;
        pending &= ~__ballot_sync(full, mine);
        const ClothDev &cd = d.cloth[cc];
        const int In = cd.T - 1;
        const float4 *W = d.wnode + 4 * (size_t)cd.i_off;
        int top = 1, node = 0;
        if (lane == 0) stk0 = -1;
        const int guard_max = 4 * cd.T + 64;
        for (int guard = 0; guard < guard_max; ++guard) {
            const float4 *r = W + 4 * (size_t)node;
            const float4 l0 = __ldg(r), l1 = __ldg(r + 1), r0 = __ldg(r + 2), r1 = __ldg(r + 3);
            const int chx = __float_as_int(l0.w), rmx = __float_as_int(l1.w);
            const int chy = __float_as_int(r0.w), rmy = __float_as_int(r1.w);
            const bool ol = mine && rmx > me && overlap(amin, amax, xyz(l0), xyz(l1));
            const bool orr = mine && rmy > me && overlap(amin, amax, xyz(r0), xyz(r1));
            if (ol && chx >= In) {
                if (got < chunk) out[got++] = (uint32_t)(chx - In);
                else ++dropped;
            }
            if (orr && chy >= In) {
                if (got < chunk) out[got++] = (uint32_t)(chy - In);
                else ++dropped;
            }
            const bool tl = chx < In && __any_sync(full, ol), tr = chy < In && __any_sync(full, orr);
            if (!tl && !tr) {
                --top;
                const int a = __shfl_sync(full, stk0, top & 31), b = __shfl_sync(full, stk1, top & 31);
                node = top < 32 ? a : b;
            } else {
                node = tl ? chx : chy;
                if (tl && tr) {
                    if (top >= kTraverseStack) { overflow = true; break; }
                    if (lane == (top & 31)) {
                        if (top < 32) stk0 = chy;
                        else stk1 = chy;
                    }
                    ++top;
                }
            }
            if (top == 0) break;
        }
        __syncwarp();
    }
    if (overflow && lane == 0) atomicOr(d.err, ERR_STACK);
    if (valid) d.pair_cnt[s] = (uint32_t)got;
    if (dropped) atomicAdd(&d.counters[3], (unsigned long long)dropped);
}


// Order-preserving compaction of the per-leaf chunks into the pair list:
// each warp takes 32 consecutive leaves, whose outputs are one contiguous
// range, and spreads that range over its lanes (output j belongs to the
// last leaf whose prefix count is <= j), so the loads are independent and
// both reads and writes are coalesced runs.
__global__ void k_pair_compact(DevPtrs d) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const int warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int base = warp0 * 32; base < d.Ttot; base += nwarps * 32) {
        const int s = base + lane;
        uint32_t n = 0;
        int t0 = 0;
        const uint32_t *src = nullptr;
        if (s < d.Ttot) {
            n = d.pair_cnt[s];
            if (n) {
                const ClothDev &cd = d.cloth[d.tcloth[s]];
                t0 = cd.t_off;
                src = d.pair_chunk + cd.pc_off + (int64_t)(s - cd.t_off) * cd.chunk;
            }
        }
        uint32_t ex = n;  // inclusive scan over the warp's leaves
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(full, ex, o);
            if (lane >= o) ex += t;
        }
        const uint32_t total = __shfl_sync(full, ex, 31);
        ex -= n;
        if (total == 0) continue;
        const uint32_t o0 = d.pair_off[base];
        for (uint32_t j0 = 0; j0 < total; j0 += 32) {
            const uint32_t j = j0 + lane;
            int L = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int cand = L + step;
                const uint32_t e = __shfl_sync(full, ex, cand & 31);
                if (cand < 32 && e <= j) L = cand;
            }
            const uint32_t exL = __shfl_sync(full, ex, L);
            const int tL = __shfl_sync(full, t0, L);
            const uint32_t *sL = reinterpret_cast<const uint32_t *>(
                __shfl_sync(full, reinterpret_cast<unsigned long long>(src), L));
            if (j < total) d.pairs[o0 + j] = make_uint2((uint32_t)(base + L), (uint32_t)tL + sL[j - exL]);
        }
    }
}
// ---------------------------------------------------------------------------
// Narrowphase.  Candidate slots of Collision/CudaCollisionDetection.cu:53-189,
// feature AABB cull of Collision/CudaPrimitiveTests.cu:427-490, CCD of
// :109-238 with Physics/CudaCubicSolver.cu:5-153 and the tests at :252-425.
// ---------------------------------------------------------------------------
// A hit's weights, normal and time (Physics::PrimitiveContact w1..w4, n, t).
// The tests write t where the reference's do (TestVF: 0; TestEE outside the
// segments: 0); the caller starts it at the candidate's -1.
struct Wts { float w0, w1, w2, w3; float3 n; float t; };

__device__ __forceinline__ float triple(float3 x21, float3 x31, float3 x41, float3 v21, float3 v31, float3 v41,
                                        float t) {
    return dot(cross(add(x21, mul(v21, t)), add(x31, mul(v31, t))), add(x41, mul(v41, t)));
}
// Physics/CudaCubicSolver.cu:131-153.  The reference evaluates f at both
// ends every iteration; f(x0) of an iteration is f(x1) of the previous one
// (same arguments, same bits), so it is carried over instead of recomputed.
// fa, fb: f(a), f(b) as the caller evaluated them (the same arguments, so
// the same bits as the reference's first-iteration evaluations).
__device__ float secant(float3 x21, float3 x31, float3 x41, float3 v21, float3 v31, float3 v41, float a, float b,
                        float fa, float fb) {
    float x0 = a, x1 = b;
    float f0 = fa;
    for (int i = 0; i < 20; ++i) {
        const float f1 = i == 0 ? fb : triple(x21, x31, x41, v21, v31, v41, x1);
        const float xc = (x0 * f1 - x1 * f0) / (f1 - f0);
        if (fabsf(xc - x1) < kEpsCubic) return xc;
        x0 = x1;
        f0 = f1;
        x1 = xc;
    }
    return -15.f;
}
__device__ __forceinline__ float3 project_on_line(float3 p, float3 e1, float3 e2) {
    const float3 ab = sub(e2, e1), ap = sub(p, e1);
    return add(e1, mul(ab, dot(ap, ab) / dot(ab, ab)));
}
__device__ __forceinline__ float3 clamp_on_line(float3 p, float3 e1, float3 e2) {
    const float d1 = dist(p, e1), d2 = dist(p, e2);
    if (fabsf(d1 + d2 - dist(e1, e2)) < kEpsPbd) return p;
    return d1 < d2 ? e1 : e2;
}

__device__ bool test_vf(float3 x4, float3 x1, float3 x2, float3 x3, float th, Wts &w) {
    const float3 x13 = sub(x1, x3), x23 = sub(x2, x3), x43 = sub(x4, x3);
    const float3 crs = cross(sub(x2, x1), sub(x3, x1));
    const float3 n = normalize(crs);
    if (fabsf(dot(x43, n)) <= th) {
        const float dt = dot(x13, x23);
        const float m11 = dot(x13, x13), m12 = dt, m21 = dt, m22 = dot(x23, x23);
        const float vr1 = dot(x13, x43), vr2 = dot(x23, x43);
        const float w2 = (m11 * vr2 - m21 * vr1) / (m11 * m22 - m21 * m12);
        const float w1 = (vr1 - m12 * w2) / m11;
        const float w3 = 1.f - w1 - w2;
        const float del = th / (len(x13) + len(x23) + len(sub(x1, x2)));
        const float lo = 0.f, hi = 1.f + del;
        if (between(w1, lo, hi) && between(w2, lo, hi) && between(w3, lo, hi)) {
            w.w0 = 1.f; w.w1 = -w1; w.w2 = -w2; w.w3 = -w3;
            w.n = n;
            w.t = 0.f;
            return true;
        }
    }
    return false;
}

__device__ bool test_ee(float3 x1, float3 x2, float3 x3, float3 x4, float th, Wts &w) {
    const float3 x21 = sub(x2, x1), x31 = sub(x3, x1), x43 = sub(x4, x3);
    const float3 crs = cross(x21, x43);
    if (len(crs) < kEpsEE) {
        const float3 m1 = add(x1, dvs(x21, 2.f)), m2 = add(x3, dvs(x43, 2.f));
        if (dist(m1, m2) <= th) {
            w.w0 = w.w1 = w.w2 = w.w3 = 0.5f;
            w.n = normalize(sub(m1, m2));
            return true;
        }
        return false;
    }
    if (is_zero(crs)) return false;
    const float dt = dot(neg(x21), x43);
    const float m11 = dot(x21, x21), m12 = dt, m21 = dt, m22 = dot(x43, x43);
    const float vr1 = dot(x21, x31), vr2 = dot(neg(x43), x31);
    float b = (m11 * vr2 - m21 * vr1) / (m11 * m22 - m21 * m12);
    float a = (vr1 - m12 * b) / m11;
    if (between(a, 0.f, 1.f) && between(b, 0.f, 1.f)) {
        const float3 cp1 = add(x1, mul(x21, a)), cp2 = add(x3, mul(x43, a));
        if (dist(cp1, cp2) <= th) {
            w.w0 = 1.f - a; w.w1 = a; w.w2 = -(1.f - b); w.w3 = -b;
            // the normal measures the second point with b (Collision/CudaPrimitiveTests.cu:305-307)
            const float3 dir = sub(add(x1, mul(x21, a)), add(x3, mul(x43, b)));
            w.n = normalize(is_zero(dir) ? crs : dir);
            return true;
        }
    } else {
        const float ac = clampf(a, 0.f, 1.f), bc = clampf(b, 0.f, 1.f);
        const float d1 = fabsf(a - ac) * len(x21), d2 = fabsf(b - bc) * len(x43);
        a = ac;
        b = bc;
        float3 cp1, cp2;
        if (d1 > d2) {
            cp1 = add(x1, mul(x21, a));
            cp2 = clamp_on_line(project_on_line(cp1, x3, x4), x3, x4);
        } else {
            cp2 = add(x3, mul(x43, b));
            cp1 = clamp_on_line(project_on_line(cp2, x1, x2), x1, x2);
        }
        if (dist(cp1, cp2) <= th) {
            w.w0 = 1.f - a; w.w1 = a; w.w2 = -(1.f - b); w.w3 = -b;
            w.n = normalize(sub(cp1, cp2));
            w.t = 0.f;
            return true;
        }
    }
    return false;
}

// A test_ee hit places both closest points on their segments (the parallel
// case uses the midpoints, the others clamp the parameters to [0,1]), up to
// a few float roundings of the coordinates, and needs their distance <= th.
// So edges whose boxes are apart by more than th plus a margin far above
// those roundings (1e-5 m + th/1000) cannot hit, and the test is skipped:
// the decision and the weights are the reference's bits either way.
__device__ __forceinline__ bool ee_far(float3 a, float3 b, float3 c, float3 d, float th) {
    const float m = th + 1e-5f + 1e-3f * th;
    return fminf(a.x, b.x) - fmaxf(c.x, d.x) > m || fminf(c.x, d.x) - fmaxf(a.x, b.x) > m ||
           fminf(a.y, b.y) - fmaxf(c.y, d.y) > m || fminf(c.y, d.y) - fmaxf(a.y, b.y) > m ||
           fminf(a.z, b.z) - fmaxf(c.z, d.z) > m || fminf(c.z, d.z) - fmaxf(a.z, b.z) > m;
}

// Particle swept box of Collision/FeatureList.cu:134-148, recomputed from
// x and x_prev (min/max are exact, so this equals the stored boxes).
struct Box { float3 lo, hi; };
__device__ __forceinline__ Box pbox(const DevPtrs &d, int v, float h) {
    if (d.vbox) return Box{xyz(d.vbox[2 * (size_t)v]), xyz(d.vbox[2 * (size_t)v + 1])};  // the same operations, once per vertex
    const float3 p = xyz(d.x[v]), q = xyz(d.xp[v]);
    return Box{subc(vmin(p, q), h), addc(vmax(p, q), h)};
}

// EE slot s: edge (s%3) of A x edge (s/3) of B; edge k of a triangle is
// (v1,v2 | bit 2), (v1,v3 | bit 0), (v2,v3 | bit 1).
__device__ __forceinline__ void edge_of(int k, int &a, int &b, int &bit) {
    if (k == 0) { a = 0; b = 1; bit = 2; }
    else if (k == 1) { a = 0; b = 2; bit = 0; }
    else { a = 1; b = 2; bit = 1; }
}

// Vertex ids of candidate slot s of a pair (A, B): VF slots 0..5 are
// (vertex s of A | face B) then (vertex s-3 of B | face A); EE slots 6..14 are
// edge (s-6)%3 of A x edge (s-6)/3 of B (Collision/CudaCollisionDetection.cu:101-187).
__device__ __forceinline__ int4 candidate_ids(const int vid[6], int s) {
    if (s < 6) {
        const int o = s < 3 ? 3 : 0;
        return make_int4(vid[s], vid[o], vid[o + 1], vid[o + 2]);
    }
    int a0, a1, ab, b0, b1, bb;
    edge_of((s - 6) % 3, a0, a1, ab);
    edge_of((s - 6) / 3, b0, b1, bb);
    return make_int4(vid[a0], vid[a1], vid[3 + b0], vid[3 + b1]);
}

// Stage 1 of the narrowphase: the candidates of one broadphase pair that
// survive feature ownership, the shared-vertex sanity checks and the feature
// AABB cull (Collision/CudaPrimitiveTests.cu:240-248, 427-490).  The checks
// commute, so the surviving set is the reference's; the six vertex boxes are
// built once per pair.
__device__ __forceinline__ uint16_t pair_filter(const DevPtrs &d, uint2 pr, bool cull) {
    const int c = d.tcloth[pr.x];
    const float h = d.cloth[c].h;
    const int4 A = d.tri_slot[pr.x], B = d.tri_slot[pr.y];
    const int fa = A.w, fb = B.w;
    const int vid[6] = {A.x, A.y, A.z, B.x, B.y, B.z};
    uint32_t want = 0;
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        const int f = s < 3 ? fa : fb;
        if (!((f >> (5 - s % 3)) & 1)) continue;
        const int pv = vid[s];
        const int o = s < 3 ? 3 : 0;
        if (pv == vid[o] || pv == vid[o + 1] || pv == vid[o + 2]) continue;
        want |= 1u << s;
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        int a0, a1, ab, b0, b1, bb;
        edge_of(s % 3, a0, a1, ab);
        edge_of(s / 3, b0, b1, bb);
        if (!(((fa >> ab) & 1) & ((fb >> bb) & 1))) continue;
        const int e1 = vid[a0], e2 = vid[a1], e3 = vid[3 + b0], e4 = vid[3 + b1];
        if (e1 == e3 || e1 == e4 || e2 == e3 || e2 == e4) continue;
        want |= 1u << (6 + s);
    }
    if (!want || !cull) return (uint16_t)want;
    // the six vertex boxes, the two face boxes and the six edge boxes once
    // (min / max are exact, so any grouping gives the reference's boxes)
    Box bx[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) bx[k] = pbox(d, vid[k], h);
    Box face[2], edge[6];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        face[t] = Box{min3(bx[3 * t].lo, bx[3 * t + 1].lo, bx[3 * t + 2].lo),
                      max3(bx[3 * t].hi, bx[3 * t + 1].hi, bx[3 * t + 2].hi)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            int a0, a1, ab;
            edge_of(k, a0, a1, ab);
            edge[3 * t + k] = Box{vmin(bx[3 * t + a0].lo, bx[3 * t + a1].lo), vmax(bx[3 * t + a0].hi, bx[3 * t + a1].hi)};
        }
    }
    uint32_t mask = 0;
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        const Box &f = face[s < 3 ? 1 : 0];
        if (((want >> s) & 1) && overlap(bx[s].lo, bx[s].hi, f.lo, f.hi)) mask |= 1u << s;
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        const Box &ea = edge[s % 3], &eb = edge[3 + s / 3];
        if (((want >> (6 + s)) & 1) && overlap(ea.lo, ea.hi, eb.lo, eb.hi)) mask |= 1u << (6 + s);
    }
    return (uint16_t)mask;
}


// Stage 1 for every pair, one thread per pair: its candidate mask, and per
// group of kPairGroup consecutive pairs (one warp iteration: the stride is a
// whole number of warps) the group's VF and EE candidate counts, whose scans
// give every group its first candidate; the number of groups at ngroups.
// cull = 0 keeps the candidates the ownership bits and the sanity checks
// leave, without the feature AABB cull (the discrete tests of
// Collision/CudaCollisionDetection.cu:191-221 apply none).
__global__ void __launch_bounds__(kThreads, 4) k_narrow_filter(DevPtrs d, const uint32_t *__restrict__ npairs,
                                                               int cull) {
    static_assert(kPairGroup == 32, "a group is one warp iteration");
    const uint32_t n = *npairs, G = (n + kPairGroup - 1) / kPairGroup;
    if (blockIdx.x == 0 && threadIdx.x == 0) *d.ngroups = G;
    const int lane = threadIdx.x & 31;
    const uint32_t end = G * kPairGroup;  // whole warps stay in the loop together (pair counts stay below 2^31)
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < end; p += gridDim.x * blockDim.x) {
        const uint16_t m = p < n ? pair_filter(d, d.pairs[p], cull != 0) : (uint16_t)0;
        if (p < n) d.pair_mask[p] = m;
        const uint32_t vf = __reduce_add_sync(0xffffffffu, (unsigned)__popc((unsigned)(m & 0x3Fu)));
        const uint32_t ee = __reduce_add_sync(0xffffffffu, (unsigned)__popc((unsigned)(m >> 6)));
        if (lane == 0) { d.grp_vf_cnt[p / kPairGroup] = vf; d.grp_ee_cnt[p / kPairGroup] = ee; }
    }
}

// First VF (or EE) candidate of pair p <= npairs: its group's offset plus the
// candidates of the pairs before it in the group; total when p starts a
// group past the last.
template <bool VF>
__device__ __forceinline__ uint32_t pair_cand_off(const DevPtrs &d, uint32_t p, uint32_t total) {
    const uint32_t g = p / kPairGroup;
    if (g >= *d.ngroups) return total;
    uint32_t o = VF ? d.grp_vf_off[g] : d.grp_ee_off[g];
    for (uint32_t q = g * kPairGroup; q < p; ++q) {
        const unsigned m = d.pair_mask[q];
        o += (uint32_t)__popc(VF ? (m & 0x3Fu) : (m >> 6));
    }
    return o;
}

// Stage 2: the surviving candidates written in the reference's order (pair,
// then slot) as the four vertex ids the CCD needs.  A warp takes 32
// consecutive pairs, whose outputs are contiguous; the warp's candidates are
// spread over all lanes (output j belongs to the last pair whose prefix count
// is <= j), so every lane writes and the writes are coalesced.
template <bool VF>
__device__ __forceinline__ void expand_kind(const DevPtrs &d, uint32_t bits, const int vid[6], uint64_t base_off) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t cnt = __popc(bits);
    uint32_t ex = cnt;  // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(full, ex, o);
        if (lane >= o) ex += t;
    }
    const uint32_t total = __shfl_sync(full, ex, 31);
    ex -= cnt;  // exclusive
    int4 *out = VF ? d.cand : d.cand_e;
    for (uint32_t j0 = 0; j0 < total; j0 += 32) {
        const uint32_t j = j0 + lane;
        int L = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int cand = L + step;
            const uint32_t e = __shfl_sync(full, ex, cand & 31);
            if (cand < 32 && e <= j) L = cand;
        }
        const uint32_t exL = __shfl_sync(full, ex, L);
        const uint32_t bL = __shfl_sync(full, bits, L);
        int v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] = __shfl_sync(full, vid[k], L);
        if (j < total) {
            uint32_t m = bL;
            for (uint32_t k = j - exL; k > 0; --k) m &= m - 1;
            const int s = (__ffs(m) - 1) + (VF ? 0 : 6);
            const uint64_t o = base_off + j;
            if (o < d.cand_cap) out[o] = candidate_ids(v, s);
            else atomicOr(d.err, ERR_CAND_OVERFLOW);
        }
    }
}

__global__ void k_narrow_expand(DevPtrs d, const uint32_t *__restrict__ npairs) {
    const uint32_t n = *npairs;
    const int lane = threadIdx.x & 31;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp0 * 32u; base < n; base += nwarps * 32u) {
        const uint32_t p = base + lane;
        const uint32_t m = p < n ? d.pair_mask[p] : 0u;
        int vid[6] = {0, 0, 0, 0, 0, 0};
        if (m) {
            const uint2 pr = d.pairs[p];
            const int4 A = d.tri_slot[pr.x], B = d.tri_slot[pr.y];
            vid[0] = A.x; vid[1] = A.y; vid[2] = A.z; vid[3] = B.x; vid[4] = B.y; vid[5] = B.z;
        }
        if (!__any_sync(0xffffffffu, m != 0u)) continue;
        expand_kind<true>(d, m & 0x3Fu, vid, d.grp_vf_off[base / kPairGroup]);
        expand_kind<false>(d, m >> 6, vid, d.grp_ee_off[base / kPairGroup]);
    }
}

// Stage 3: CCD of every candidate of one kind on x_prev and v
// (Collision/CudaPrimitiveTests.cu:109-238, Physics/CudaCubicSolver.cu:5-153).
// VF: vertex x4 against the face x1 x2 x3; EE: edges x1 x2 and x3 x4.  The
// reference collects every coplanarity time of [0,1] (the ends of the
// intervals cut at the derivative's roots where |f| < eps, and the secant
// root of every interval whose ends differ in sign), then advances the four
// positions by v t dt for each time in turn and tests after each advance
// until one test hits.  Here each warp takes 32 candidates at a time:
// (1) every lane sets up its candidate's cubic, evaluates f at the interval
// ends and queues the intervals that need a secant solve; (2) the warp runs
// the queued solves, one per lane; (3) every lane tests its times in the
// reference's order with the cumulative advance and stops at the first hit.
// The operands and operations of every piece are the reference's, so the
// decisions are the same bits; only the assignment of work to lanes differs.
constexpr int kCcdWarps = 8;
struct CcdJob { float a, b, fa, fb; };

// At most 64 registers, for 4 resident blocks per SM instead of 3 (a few
// words spill to L1): measured 0.83 -> 0.80 ms per step for VF, EE unchanged.
template <bool VF>
__global__ void __launch_bounds__(kCcdWarps * 32, 4) k_ccd_warp(DevPtrs d, const uint32_t *__restrict__ ncand) {
    __shared__ float geom[kCcdWarps][24][33];     // x1..x4 then v1..v4 (test order) per lane (padded)
    __shared__ CcdJob jobs[kCcdWarps][96];
    __shared__ uint8_t job_owner[kCcdWarps][96];  // lane << 2 | interval
    __shared__ float roots[kCcdWarps][3][32];
    __shared__ float tq[kCcdWarps][6][32];        // each lane's times to test, in the reference's order
    __shared__ int best[kCcdWarps][32];           // each lane's first hitting test (6: none)
    const uint32_t n = (uint32_t)min((uint64_t)*ncand, d.cand_cap);
    const int4 *list = VF ? d.cand : d.cand_e;
    // hit bits per group of 32 candidates (one warp iteration: base is a
    // multiple of 32); the scan of their counts orders the contacts
    uint32_t *hmask = d.hitg_mask[VF ? 0 : 1], *hcnt = d.hitg_cnt[VF ? 0 : 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) d.hitg_n[VF ? 0 : 1] = (n + 31) / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu;
    const uint32_t nwarps = gridDim.x * kCcdWarps;
    for (uint32_t base = (blockIdx.x * kCcdWarps + w) * 32u; base < n; base += nwarps * 32u) {
        const uint32_t q = base + lane;
        const bool valid = q < n;
        int4 ids = make_int4(0, 0, 0, 0);
        int ncp = -1;
        float e1 = 1.f, e2 = 1.f;
        unsigned imm = 0, sec = 0;
        float fv[4] = {0.f, 0.f, 0.f, 0.f};
        if (valid) {
            ids = list[q];
            // VF: face ids.y ids.z ids.w, vertex ids.x (x4); EE: x1..x4 = ids
            const int i1 = VF ? ids.y : ids.x, i2 = VF ? ids.z : ids.y, i3 = VF ? ids.w : ids.z, i4 = VF ? ids.x : ids.w;
            const float3 x1 = xyz(d.xp[i1]), x2 = xyz(d.xp[i2]), x3 = xyz(d.xp[i3]), x4 = xyz(d.xp[i4]);
            const float3 v1 = xyz(d.v[i1]), v2 = xyz(d.v[i2]), v3 = xyz(d.v[i3]), v4 = xyz(d.v[i4]);
            const float3 x21 = sub(x2, x1), x31 = sub(x3, x1), x41 = sub(x4, x1);
            const float3 v21 = sub(v2, v1), v31 = sub(v3, v1), v41 = sub(v4, v1);
            const float g[24] = {x1.x, x1.y, x1.z, x2.x, x2.y, x2.z, x3.x, x3.y, x3.z, x4.x, x4.y, x4.z,
                                 v1.x, v1.y, v1.z, v2.x, v2.y, v2.z, v3.x, v3.y, v3.z, v4.x, v4.y, v4.z};
#pragma unroll
            for (int k = 0; k < 24; ++k) geom[w][k][lane] = g[k];
            const float3 v21v31 = cross(v21, v31), x21v31 = cross(x21, v31), v21x31 = cross(v21, x31),
                         x21x31 = cross(x21, x31);
            const float v1v2v3 = dot(v21v31, v41), x1v2v3 = dot(x21v31, v41), v1x2v3 = dot(v21x31, v41),
                        v1v2x3 = dot(v21v31, x41), x1x2v3 = dot(x21x31, v41), x1v2x3 = dot(x21v31, x41),
                        v1x2x3 = dot(v21x31, x41);
            const float a3 = v1v2v3, b3 = x1v2v3 + v1x2v3 + v1v2x3, c3 = x1x2v3 + x1v2x3 + v1x2x3;
            const float ad = 3.f * a3, bd = 2.f * b3;
            const float disc = 4.f * (b3 * b3 - ad * c3);
            const float sq = sqrtf(disc);
            const float da = 2.f * ad;
            const float t1 = (-bd + sq) / da, t2 = (-bd - sq) / da;
            ncp = 0;
            if (disc >= kEpsCubic) {
                const bool in1 = between(t1, 0.f, 1.f), in2 = between(t2, 0.f, 1.f);
                ncp = (in1 || in2) ? ((in1 && in2) ? 2 : 1) : 0;
            } else if (fabsf(disc) < kEpsCubic) {
                ncp = between(t1, 0.f, 1.f) ? 1 : 0;
            }
            e1 = ncp >= 1 ? t1 : 1.f;
            e2 = ncp == 2 ? t2 : 1.f;
            fv[0] = triple(x21, x31, x41, v21, v31, v41, 0.f);
#pragma unroll
            for (int i = 0; i <= 2; ++i) {
                if (i > ncp) break;
                const float b = i == ncp ? 1.f : (i == 0 ? e1 : e2);
                fv[i + 1] = triple(x21, x31, x41, v21, v31, v41, b);
                if (fabsf(fv[i]) < kEpsCubic) imm |= 1u << i;
                if (fv[i] * fv[i + 1] < 0.f) sec |= 1u << i;
            }
        }
        // queue the secant solves of the warp
        int njobs = 0;
#pragma unroll
        for (int i = 0; i <= 2; ++i) {
            const bool want = (sec >> i) & 1u;
            const unsigned m = __ballot_sync(full, want);
            if (want) {
                const int pos = njobs + __popc(m & ((1u << lane) - 1u));
                const float a = i == 0 ? 0.f : (i == 1 ? e1 : e2);
                const float b = i == ncp ? 1.f : (i == 0 ? e1 : e2);
                jobs[w][pos] = CcdJob{a, b, fv[i], fv[i + 1]};
                job_owner[w][pos] = (uint8_t)(lane << 2 | i);
            }
            njobs += __popc(m);
        }
        __syncwarp();
        for (int j = lane; j < njobs; j += 32) {
            const CcdJob jb = jobs[w][j];
            const int own = job_owner[w][j] >> 2, iv = job_owner[w][j] & 3;
            // the set-up's differences, from the same operands
            const float3 p1 = f3(geom[w][0][own], geom[w][1][own], geom[w][2][own]);
            const float3 u1 = f3(geom[w][12][own], geom[w][13][own], geom[w][14][own]);
            const float3 x21 = sub(f3(geom[w][3][own], geom[w][4][own], geom[w][5][own]), p1);
            const float3 x31 = sub(f3(geom[w][6][own], geom[w][7][own], geom[w][8][own]), p1);
            const float3 x41 = sub(f3(geom[w][9][own], geom[w][10][own], geom[w][11][own]), p1);
            const float3 v21 = sub(f3(geom[w][15][own], geom[w][16][own], geom[w][17][own]), u1);
            const float3 v31 = sub(f3(geom[w][18][own], geom[w][19][own], geom[w][20][own]), u1);
            const float3 v41 = sub(f3(geom[w][21][own], geom[w][22][own], geom[w][23][own]), u1);
            roots[w][iv][own] = secant(x21, x31, x41, v21, v31, v41, jb.a, jb.b, jb.fa, jb.fb);
        }
        __syncwarp();
        // The ordered tests of every candidate (the reference advances the
        // four positions by v t dt for each time in turn and tests after each
        // advance, stopping at the first hit).  Every (candidate, time) test
        // of the warp is a job of its own, spread evenly over the lanes: a
        // job rebuilds its positions by the same sequence of advances and
        // runs the same test, so it decides the same bits.  A candidate's
        // first hit is its smallest hitting test index; its owner lane then
        // runs that test once more for the weights.
        int nt = 0;
        float hq = 0.f, dtq = 0.f;
        if (valid) {
            for (int i = 0; i <= ncp; ++i) {
                const float a = i == 0 ? 0.f : (i == 1 ? e1 : e2);
                if ((imm >> i) & 1u) tq[w][nt++][lane] = a;
                if ((sec >> i) & 1u) {
                    const float t = roots[w][i][lane];
                    if (t != -15.f) tq[w][nt++][lane] = t;
                }
            }
            const ClothDev &cd = d.cloth[d.vcloth[ids.x]];
            hq = cd.h;
            dtq = cd.dt;
        }
        best[w][lane] = 6;
        uint32_t ex = (uint32_t)nt;  // inclusive scan of the test counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(full, ex, o);
            if (lane >= o) ex += t;
        }
        const uint32_t ntests = __shfl_sync(full, ex, 31);
        ex -= (uint32_t)nt;
        __syncwarp();
        // the four vertices of lane L's candidate in test order (VF: face x1 x2 x3,
        // vertex x4), as its set-up loaded them
        auto corners = [&](int L, float3 &x1, float3 &x2, float3 &x3, float3 &x4, float3 &v1, float3 &v2,
                           float3 &v3, float3 &v4) {
            const float(*gm)[33] = geom[w];
            x1 = f3(gm[0][L], gm[1][L], gm[2][L]); x2 = f3(gm[3][L], gm[4][L], gm[5][L]);
            x3 = f3(gm[6][L], gm[7][L], gm[8][L]); x4 = f3(gm[9][L], gm[10][L], gm[11][L]);
            v1 = f3(gm[12][L], gm[13][L], gm[14][L]); v2 = f3(gm[15][L], gm[16][L], gm[17][L]);
            v3 = f3(gm[18][L], gm[19][L], gm[20][L]); v4 = f3(gm[21][L], gm[22][L], gm[23][L]);
        };
        // test m of lane L's candidate: the advances by its times 0..m, then the test
        auto run_test = [&](int L, int m, float h, float dt, Wts &wt) {
            float3 x1, x2, x3, x4, v1, v2, v3, v4;
            corners(L, x1, x2, x3, x4, v1, v2, v3, v4);
            float tt = 0.f;
            for (int k = 0; k <= m; ++k) {
                tt = tq[w][k][L] * dt;
                x1 = add(x1, mul(v1, tt));
                x2 = add(x2, mul(v2, tt));
                x3 = add(x3, mul(v3, tt));
                x4 = add(x4, mul(v4, tt));
            }
            if (!VF && ee_far(x1, x2, x3, x4, h)) return false;
            const bool r = VF ? test_vf(x4, x1, x2, x3, h, wt) : test_ee(x1, x2, x3, x4, h, wt);
            wt.t = tt;  // the contact's time (Collision/CudaPrimitiveTests.cu:174, 228)
            return r;
        };
        for (uint32_t j0 = 0; j0 < ntests; j0 += 32) {
            const uint32_t j = j0 + lane;
            int L = 0;  // owner: the last lane whose first test is <= j
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int cand = L + step;
                const uint32_t e = __shfl_sync(full, ex, cand & 31);
                if (cand < 32 && e <= j) L = cand;
            }
            const uint32_t exL = __shfl_sync(full, ex, L);
            const float h = __shfl_sync(full, hq, L), dt = __shfl_sync(full, dtq, L);
            if (j < ntests) {
                const int m = (int)(j - exL);
                Wts wt;
                if (run_test(L, m, h, dt, wt)) atomicMin(&best[w][L], m);
            }
        }
        __syncwarp();
        bool found = false;
        Wts wt;
        if (valid && best[w][lane] < 6) found = run_test(lane, best[w][lane], hq, dtq, wt);
        if (valid) {
            if (found) {
                // the contact's weights, placed at its final index by k_ccd_emit
                const uint64_t cap = VF ? d.vf_cap : d.ee_cap;
                const uint32_t slot = atomicAdd(&d.hit_n[VF ? 0 : 1], 1u);
                if (slot < cap) {
                    d.hit_q[VF ? 0 : 1][slot] = q;
                    d.hit_w[VF ? 0 : 1][slot] = make_float4(wt.w0, wt.w1, wt.w2, wt.w3);
                    if (VF && d.hit_nrm) d.hit_nrm[slot] = make_float4(wt.n.x, wt.n.y, wt.n.z, 0.f);
                    if (d.hit_tn[VF ? 0 : 1]) d.hit_tn[VF ? 0 : 1][slot] = make_float4(wt.n.x, wt.n.y, wt.n.z, wt.t);
                } else {
                    atomicOr(d.err, VF ? ERR_VF_OVERFLOW : ERR_EE_OVERFLOW);
                }
            }
        }
        const unsigned hb = __ballot_sync(full, found);
        if (lane == 0) {
            hmask[base / 32] = hb;
            hcnt[base / 32] = (uint32_t)__popc(hb);
        }
        __syncwarp();
    }
}

// The discrete tests (CudaPrimitiveTests::DCDTriangleTests,
// Collision/CudaPrimitiveTests.cu:21-94): one TestVF / TestEE of every
// candidate at x_prev, as HandleCollisionsDiscrete passes the previous
// positions (Physics/CudaDeformableBody.cpp:428).  Hits are recorded as the
// continuous kernel records them (per group of 32 candidates: the hit bits;
// k_ccd_emit places them), with t as the tests leave it.
template <bool VF>
__global__ void __launch_bounds__(kThreads) k_dcd_warp(DevPtrs d, const uint32_t *__restrict__ ncand) {
    const uint32_t n = (uint32_t)min((uint64_t)*ncand, d.cand_cap);
    const int4 *list = VF ? d.cand : d.cand_e;
    uint32_t *hmask = d.hitg_mask[VF ? 0 : 1], *hcnt = d.hitg_cnt[VF ? 0 : 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) d.hitg_n[VF ? 0 : 1] = (n + 31) / 32;
    const int lane = threadIdx.x & 31;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp0 * 32u; base < n; base += nwarps * 32u) {
        const uint32_t q = base + lane;
        bool found = false;
        if (q < n) {
            const int4 ids = list[q];
            const float h = d.cloth[d.vcloth[ids.x]].h;
            Wts wt;
            wt.t = -1.f;  // the candidate's initial time (Physics/Structs.h:122-124)
            found = VF ? test_vf(xyz(d.xp[ids.x]), xyz(d.xp[ids.y]), xyz(d.xp[ids.z]), xyz(d.xp[ids.w]), h, wt)
                       : test_ee(xyz(d.xp[ids.x]), xyz(d.xp[ids.y]), xyz(d.xp[ids.z]), xyz(d.xp[ids.w]), h, wt);
            if (found) {
                const uint64_t cap = VF ? d.vf_cap : d.ee_cap;
                const uint32_t slot = atomicAdd(&d.hit_n[VF ? 0 : 1], 1u);
                if (slot < cap) {
                    d.hit_q[VF ? 0 : 1][slot] = q;
                    d.hit_w[VF ? 0 : 1][slot] = make_float4(wt.w0, wt.w1, wt.w2, wt.w3);
                    if (d.hit_tn[VF ? 0 : 1])
                        d.hit_tn[VF ? 0 : 1][slot] = make_float4(wt.n.x, wt.n.y, wt.n.z, wt.t);
                } else {
                    atomicOr(d.err, VF ? ERR_VF_OVERFLOW : ERR_EE_OVERFLOW);
                }
            }
        }
        const unsigned hb = __ballot_sync(0xffffffffu, found);
        if (lane == 0) {
            hmask[base / 32] = hb;
            hcnt[base / 32] = (uint32_t)__popc(hb);
        }
    }
}

// Contacts of the candidates before candidate q <= n (n the kind's
// candidate count): its group's first contact plus the hits before it in
// the group.
template <bool VF>
__device__ __forceinline__ uint32_t hit_index(const DevPtrs &d, uint32_t q) {
    const int k = VF ? 0 : 1;
    const uint32_t g = q / 32, r = q % 32;
    if (g >= d.hitg_n[k]) return d.hitg_off[k][d.hitg_n[k]];
    return d.hitg_off[k][g] + (uint32_t)__popc(d.hitg_mask[k][g] & ((1u << r) - 1u));
}

// Stage 4 after k_ccd_warp: every hit written at its index in candidate order
// (the exclusive scan of the hit flags), ids from the candidate list.
template <bool VF>
__global__ void k_ccd_emit(DevPtrs d) {
    const uint64_t cap = VF ? d.vf_cap : d.ee_cap;
    const uint32_t n = (uint32_t)min((uint64_t)d.hit_n[VF ? 0 : 1], cap);
    const int4 *list = VF ? d.cand : d.cand_e;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t q = d.hit_q[VF ? 0 : 1][k];
        const uint32_t o = hit_index<VF>(d, q);
        if (o < cap) {
            if (VF) {
                d.vf_v[o] = list[q];
                d.vf_w[o] = d.hit_w[0][k];
                if (d.vf_n) d.vf_n[o] = d.hit_nrm[k];
                if (d.vf_tn) d.vf_tn[o] = d.hit_tn[0][k];
            } else {
                d.ee_v[o] = list[q];
                d.ee_w[o] = d.hit_w[1][k];
                if (d.ee_tn) d.ee_tn[o] = d.hit_tn[1][k];
            }
        } else {
            atomicOr(d.err, VF ? ERR_VF_OVERFLOW : ERR_EE_OVERFLOW);
        }
    }
}

// Per-cloth contact ranges (the VF and the EE contacts of one cloth are
// contiguous).
__global__ void k_contact_ranges(DevPtrs d, const uint32_t *__restrict__ ncv, const uint32_t *__restrict__ nce) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.C) return;
    const ClothDev &cd = d.cloth[c];
    const uint32_t nv = (uint32_t)min((uint64_t)*ncv, d.cand_cap), ne = (uint32_t)min((uint64_t)*nce, d.cand_cap);
    const uint32_t p0 = d.pair_off[cd.t_off], p1 = d.pair_off[cd.t_off + cd.T];
    const uint32_t v0 = min(pair_cand_off<true>(d, p0, nv), nv), v1 = min(pair_cand_off<true>(d, p1, nv), nv);
    const uint32_t e0 = min(pair_cand_off<false>(d, p0, ne), ne), e1 = min(pair_cand_off<false>(d, p1, ne), ne);
    d.crange[c] = make_uint4((uint32_t)min((uint64_t)hit_index<true>(d, v0), d.vf_cap),
                             (uint32_t)min((uint64_t)hit_index<true>(d, v1), d.vf_cap),
                             (uint32_t)min((uint64_t)hit_index<false>(d, e0), d.ee_cap),
                             (uint32_t)min((uint64_t)hit_index<false>(d, e1), d.ee_cap));
}

// ---------------------------------------------------------------------------
// Static triangle colliders (lc_batch_set_collider; no counterpart in the
// reference, whose sphere is analytic).  One thread per cloth vertex walks
// its cloth's collider BVH with the vertex's swept box inflated by h + m
// (m = kColliderMargin h).  For a face with unit normal n towards the free
// side (the winding given to lc_batch_set_collider) and d0 = n . a, the
// vertex's signed heights s0 = n . x_prev - d0 and s1 = n . x - d0 (x the
// prediction) make it a contact when it ends within reach of the face's
// layer (s1 < h + m) without having started far behind it (s0 > -m), and the
// point where it crosses the plane (without a crossing, its prediction) lies
// on the triangle: barycentric coordinates >= -h / perimeter, the tolerance
// of the reference's TestVF (Collision/CudaPrimitiveTests.cu:348-406).  The
// motion is the prediction's straight line, so the test is exact.  The reach
// lets the constraint act on a vertex that the solver iterations drag
// towards the face after this test, and brings back one that ended a step
// behind it; a contact above its layer is inactive, the constraint being
// one-sided.  A contact records the face and its plane (n, d0): the
// constraint n . x >= d0 + h, onto which the vertex is projected here, in
// slot order, and again at the end of every solver iteration.  The
// kColliderSlots lowest faces are kept, ascending, so the result does not
// depend on the traversal order.
// ---------------------------------------------------------------------------
// The per-face part of the test, computed once per lc_batch_set_collider
// (the same operations in the same order as a per-test evaluation, so the
// same bits): plane (n towards the free side, d0 = n . a), corner a and the
// perimeter, the edges and their dot products.
__global__ void k_collider_faces(DevPtrs d, int ntri) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const int4 tv = d.ct[t];
    const float3 a = xyz(d.cv[tv.x]), b = xyz(d.cv[tv.y]), c = xyz(d.cv[tv.z]);
    float3 nf = normalize(cross(sub(b, a), sub(c, a)));
    if (d.cloth[tv.w].coll_cw) nf = mul(nf, -1.f);
    const float3 e1 = sub(b, a), e2 = sub(c, a), e3 = sub(c, b);
    const float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2);
    float4 *g = d.cface_geo + (size_t)5 * t;
    g[0] = f4(nf, dot(nf, a));
    g[1] = f4(a, len(e1) + len(e2) + len(e3));
    g[2] = f4(e1, d00);
    g[3] = f4(e2, d11);
    g[4] = make_float4(d01, d00 * d11 - d01 * d01, 0.f, 0.f);
}
void launch_collider_faces(const DevPtrs &d, int ntri, cudaStream_t st) {
    if (ntri) k_collider_faces<<<(ntri + kThreads - 1) / kThreads, kThreads, 0, st>>>(d, ntri);
}

__device__ bool collider_hit(float3 xp, float3 x, const float4 *__restrict__ g, float h, float m) {
    const float4 pl = g[0];
    const float3 n = xyz(pl);
    const float d0 = pl.w;
    const float s0 = dot(n, xp) - d0, s1 = dot(n, x) - d0;
    if (!(s1 < h + m) || !(s0 > -m)) return false;
    const float4 ga = g[1], g1 = g[2], g2 = g[3], g3 = g[4];
    const float3 q = (s0 > 0.f && s1 < 0.f) ? add(xp, mul(sub(x, xp), s0 / (s0 - s1))) : x;
    const float3 r = sub(q, xyz(ga));
    const float d00 = g1.w, d01 = g3.x, d11 = g2.w, d20 = dot(r, xyz(g1)), d21 = dot(r, xyz(g2));
    const float den = g3.y;
    if (!(den > 0.f)) return false;
    const float wb = (d11 * d20 - d01 * d21) / den, wc = (d00 * d21 - d01 * d20) / den;
    const float wa = 1.f - wb - wc;
    const float del = h / ga.w;
    return wa >= -del && wb >= -del && wc >= -del;
}

__global__ void k_collider_query(DevPtrs d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.Vtot; i += gridDim.x * blockDim.x) {
        const ClothDev &cd = d.cloth[d.vcloth[i]];
        int n = 0;
        int face[kColliderSlots];
        float4 pln[kColliderSlots];
        const float4 x4 = d.x[i];
        const float h = cd.h;
        if (cd.coll_root >= 0) {
            const float m = kColliderMargin * h, hm = h + m;
            const float3 xi = xyz(x4), xpi = xyz(d.xp[i]);
            const float3 lo = subc(vmin(xi, xpi), hm), hi = addc(vmax(xi, xpi), hm);
            int stack[kColliderStack];
            int top = 0;
            stack[top++] = cd.coll_root;
            while (top > 0) {
                const int node = stack[--top];
                if (!overlap(lo, hi, xyz(d.cnmin[node]), xyz(d.cnmax[node]))) continue;
                const int2 ch = d.cnchild[node];
                if (ch.x >= 0) {
                    if (top + 2 > kColliderStack) { atomicOr(d.err, ERR_STACK); break; }
                    stack[top++] = ch.y;
                    stack[top++] = ch.x;
                    continue;
                }
                const int tri = -(ch.x + 1);
                const float4 *g = d.cface_geo + (size_t)5 * tri;
                if (!collider_hit(xpi, xi, g, h, m)) continue;
                // keep the kColliderSlots lowest faces, ascending
                if (n == kColliderSlots && tri > face[n - 1]) { atomicOr(d.err, ERR_COLL_OVERFLOW); continue; }
                if (n == kColliderSlots) atomicOr(d.err, ERR_COLL_OVERFLOW);
                int k = n < kColliderSlots ? n++ : kColliderSlots - 1;
                while (k > 0 && face[k - 1] > tri) {
                    face[k] = face[k - 1];
                    pln[k] = pln[k - 1];
                    --k;
                }
                face[k] = tri;
                pln[k] = g[0];
            }
        }
        d.ccnt[i] = n;
        float3 xn = xyz(x4);
        uint32_t act = 0;
        for (int k = 0; k < n; ++k) {
            d.cface[(size_t)i * kColliderSlots + k] = face[k];
            d.cw[(size_t)i * kColliderSlots + k] = pln[k];
            const float c = dot(xyz(pln[k]), xn) - pln[k].w - h;
            if (c < 0.f) {
                xn = add(xn, mul(xyz(pln[k]), -c));
                act |= 1u << k;
            }
        }
        if (x4.w == 0.f) act = 0;                  // pinned vertices do not move
        else if (n) d.x[i] = f4(xn, x4.w);
        if (d.coll_act) d.coll_act[i] = (uint8_t)act;  // the adjoint's record of the projection
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
static inline int nblk(int64_t n, int b = kThreads) { return (int)((n + b - 1) / b); }

void launch_collider(const DevPtrs &d, int grid, cudaStream_t st) {
    if (d.Vtot && d.any_collider) k_collider_query<<<grid, kThreads, 0, st>>>(d);
}
void launch_triangles(const DevPtrs &d, cudaStream_t st) {
    if (d.Ttot) k_triangles<<<nblk(d.Ttot), kThreads, 0, st>>>(d);
}
void launch_leaves_from_boxes(const DevPtrs &d, const float *bmin, const float *bmax, int T, int mode,
                              cudaStream_t st) {
    if (T) k_leaves_from_boxes<<<nblk(T), kThreads, 0, st>>>(d, bmin, bmax, T, mode);
}
void launch_sort(const DevPtrs &d, const int *tile_first, int passes, cudaStream_t st) {
    if (!d.nstiles) return;
    // One-sweep wherever the scratch exists (not in the allocation-free
    // entry, whose one tile needs no look-back) and the digit counts fit the
    // status word's 30 bits; the per-pass histogram and per-segment offsets
    // block remain for the rest.
    const bool sweep = d.sstat && d.sseg && d.Ttot <= (int64_t)kStatCount && passes <= kSortPassesMax;
    if (sweep) {
        cudaMemsetAsync(d.sseg, 0, sizeof(uint32_t) * (kSortPassesMax + (size_t)d.C * kSortPassesMax * kSortBuckets), st);
        k_sort_hist_all<<<d.nstiles, kThreads, 0, st>>>(d, d.keys, passes);
    }
    for (int p = 0; p < passes; ++p) {
        const bool even = (p & 1) == 0;
        const unsigned long long *kin = even ? d.keys : d.keys_alt;
        unsigned long long *kout = even ? d.keys_alt : d.keys;
        const uint32_t *pin = even ? d.payload : d.payload_alt;
        uint32_t *pout = even ? d.payload_alt : d.payload;
        if (sweep) {
            k_sort_scatter<true><<<d.nstiles, kThreads, 0, st>>>(d, kin, pin, kout, pout, p * kSortBits, p, tile_first);
        } else {
            k_sort_hist<<<d.nstiles, kThreads, 0, st>>>(d, kin, p * kSortBits);
            k_sort_offsets<<<d.C, kSortBuckets * kOffsetsSplit, 0, st>>>(d, tile_first);
            k_sort_scatter<false><<<d.nstiles, kThreads, 0, st>>>(d, kin, pin, kout, pout, p * kSortBits, p, tile_first);
        }
    }
}
void launch_post_sort(const DevPtrs &d, cudaStream_t st) {
    if (d.Ttot) k_post_sort<<<nblk(d.Ttot), kThreads, 0, st>>>(d);
}
void launch_karras(const DevPtrs &d, cudaStream_t st) {
    if (d.Ttot) k_karras<<<nblk(d.Ttot), kThreads, 0, st>>>(d);
}
void launch_refit(const DevPtrs &d, cudaStream_t st) {
    if (!d.Ttot) return;
    if (d.nend) {
        // the upper pass: a grid-stride loop over the arrivals left, sized to
        // be resident at once
        k_refit_local<<<nblk(d.Ttot), kThreads, 0, st>>>(d);
        k_refit_upper<<<std::min(nblk(2 * (int64_t)std::max(d.Itot, 1)), 1024), kThreads, 0, st>>>(d);
    } else {
        k_refit<<<nblk(d.Ttot), kThreads, 0, st>>>(d);
    }
}
void launch_traverse(const DevPtrs &d, int block, cudaStream_t st) {
    if (!d.Ttot) return;
    if (d.wnode) {
        k_pack_nodes<<<nblk(d.Ttot), kThreads, 0, st>>>(d);
        k_traverse_packet<<<nblk(d.Ttot, block), block, 0, st>>>(d);
    } else {
        k_traverse<<<nblk(d.Ttot, block), block, 0, st>>>(d);
    }
}
void launch_pair_compact(const DevPtrs &d, cudaStream_t st) {
    if (d.Ttot) k_pair_compact<<<nblk(d.Ttot), kThreads, 0, st>>>(d);  // one warp per 32 leaves
}
void launch_narrow(const DevPtrs &d, const uint32_t *npairs, const uint32_t *ncv, const uint32_t *nce, int grid,
                   int stage, cudaStream_t st) {
    if (stage == 0) k_narrow_filter<<<grid, kThreads, 0, st>>>(d, npairs, 1);
    else if (stage == 6) k_narrow_filter<<<grid, kThreads, 0, st>>>(d, npairs, 0);  // no feature AABB cull
    else if (stage == 7) {
        cudaMemsetAsync(d.hit_n, 0, 2 * sizeof(uint32_t), st);
        k_dcd_warp<true><<<grid, kThreads, 0, st>>>(d, ncv);
    } else if (stage == 8) {
        k_dcd_warp<false><<<grid, kThreads, 0, st>>>(d, nce);
    }
    else if (stage == 1) k_narrow_expand<<<grid, kThreads, 0, st>>>(d, npairs);
    else if (stage == 2) {
        cudaMemsetAsync(d.hit_n, 0, 2 * sizeof(uint32_t), st);
        k_ccd_warp<true><<<grid, kCcdWarps * 32, 0, st>>>(d, ncv);
    } else if (stage == 5) {
        k_ccd_warp<false><<<grid, kCcdWarps * 32, 0, st>>>(d, nce);
    } else if (stage == 3) {
        k_ccd_emit<true><<<grid, kThreads, 0, st>>>(d);
        k_ccd_emit<false><<<grid, kThreads, 0, st>>>(d);
    } else {
        k_contact_ranges<<<nblk(d.C, 128), 128, 0, st>>>(d, ncv, nce);
    }
}

}  // namespace lc
