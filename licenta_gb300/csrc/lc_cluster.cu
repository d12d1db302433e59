// lc_cluster.cu — the PBD solver of one step (CudaPBD::PBDStepSolver +
// PBDStepIntegration + DeformableUtils::WorldConstraints) with each cloth
// resident on chip in one thread-block cluster.
//
// Cluster c' owns cloth c: its CS CTAs split the cloth's vertices into CS
// contiguous ranges and keep the positions of their range (float4, w =
// inverse mass) in shared memory, double-buffered for the Jacobi update.
// Each vertex gathers the corrections of the constraints it belongs to (its
// slots, in the reference's slot order: Physics/CudaPBD.cu:146-233), reading
// the positions of vertices owned by other CTAs through distributed shared
// memory, and writes its own new position; one cluster barrier per iteration
// separates the read of iteration k from the writes of iteration k+1.  No
// atomics: every sum has a fixed order, so runs are deterministic, and the
// association follows the reference's accumulator
// ((ground + LRA) + static) + dynamic, x += acc / count (:648-659, 1690-1698).
// Set-up (ground, LRA, sphere) and integration are fused into the same launch,
// so the cloth state crosses HBM once per step.
#include <cooperative_groups.h>

#include "lc_internal.cuh"
#include "lc_pbd.cuh"

namespace cg = cooperative_groups;

namespace lc {

constexpr int kClusterBlock = 512;

// Shared memory per vertex: two position buffers (32) + ground plane height
// (4) + LRA flags (1).
constexpr int kClusterBytesPerVertex = 37;

struct ClusterArgs {
    const int *cl_cloth;     // cluster -> cloth (largest first)
    const uint32_t *nvf;     // VF contacts this step (device count)
    int chunk_cap;
};

template <int CS>
__global__ void __launch_bounds__(kClusterBlock, 1) k_solve_cluster(DevPtrs d, ClusterArgs a) {
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();
    const int c = a.cl_cloth[blockIdx.x / CS];
    const ClothDev &cd = d.cloth[c];
    const int V = cd.V, vo = cd.v_off;
    const int chunk = (V + CS - 1) / CS;
    const int lo = r * chunk;
    const int n_own = max(0, min(V, lo + chunk) - lo);
    const int tid = threadIdx.x, bs = blockDim.x;
    const int cap = a.chunk_cap;

    extern __shared__ float4 smem4[];
    float4 *buf0 = smem4;
    float4 *buf1 = smem4 + cap;
    float *gq = reinterpret_cast<float *>(smem4 + 2 * cap);
    uint8_t *lra = reinterpret_cast<uint8_t *>(gq + cap);

    auto X = [&](const float4 *xs, int li) -> float4 {
        const int o = li / chunk;
        if (o == r) return xs[li - lo];
        return cluster.map_shared_rank(xs, o)[li - o * chunk];
    };

    // ---- load + ground constraints (Physics/CudaPBD.cu:1477-1507) ----------
    const float qnan = __int_as_float(0x7fc00000);
    for (int i = tid; i < n_own; i += bs) {
        const int g = vo + lo + i;
        const float4 x4 = d.x[g];
        buf0[i] = x4;
        lra[i] = 0;
        float q = qnan;
        float4 qdbg = make_float4(0.f, 0.f, 0.f, 0.f);
        if (cd.ground_on && x4.y <= cd.ground_y + cd.h) {
            const float3 pos = xyz(x4);
            const float3 nc = f3(0.f, 1.f, 0.f);
            const float3 p0 = f3(1.f, cd.ground_y + cd.h, 1.f);
            const float3 l = sub(pos, xyz(d.xp[g]));
            const float dd = dot(sub(p0, pos), nc) / dot(l, nc);
            const float3 qc = add(mul(l, dd), pos);
            // dot(pos - qc, nc) is pos.y - qc.y when qc.x and qc.z are finite, NaN otherwise
            q = (isfinite(qc.x) && isfinite(qc.z)) ? qc.y : qnan;
            qdbg = f4(qc, 1.f);
        }
        gq[i] = q;
        if (d.dbg_ground_it) d.ground_qc[g] = qdbg;
    }
    cluster.sync();
    // ---- LRA flags (Physics/CudaPBD.cu:1571-1592) --------------------------
    if (cd.F) {
        for (int i = tid; i < n_own; i += bs) {
            const float4 x4 = buf0[i];
            uint8_t f = 0;
            const int64_t base = cd.lra_off + (int64_t)(lo + i) * cd.F;
            if (x4.w != 0.f)
                for (int j = 0; j < cd.F; ++j)
                    if (dist(xyz(x4), xyz(X(buf0, d.fixed[cd.f_off + j] - vo))) > d.lra_l0[base + j])
                        f |= (uint8_t)(1u << j);
            lra[i] = f;
            if (d.dbg_ground_it)
                for (int j = 0; j < cd.F; ++j) d.lra_flag[base + j] = (f >> j) & 1u;
        }
        cluster.sync();
    }
    // ---- analytic sphere (Physics/CudaPBD.cu:1509-1569) ---------------------
    if (cd.sphere_on) {
        const float3 sc = f3(cd.sphere_pos[0], cd.sphere_pos[1], cd.sphere_pos[2]);
        const float rad = cd.sphere_r + cd.h;
        for (int i = tid; i < n_own; i += bs) {
            const int g = vo + lo + i;
            const float4 x4 = buf0[i], p4 = d.xp[g];
            float3 dir = sub(xyz(x4), xyz(p4));
            int ret = 0;
            float3 q = f3(0.f, 0.f, 0.f);
            if (!is_zero(dir)) {
                const float l = len(dir);
                dir = dvs(dir, l);
                const float3 m = sub(xyz(p4), sc);
                const float b = dot(m, dir);
                const float cc = dot(m, m) - rad * rad;
                if (!(cc > 0.f && b > 0.f)) {
                    const float disc = b * b - cc;
                    if (!(disc < 0.f)) {
                        const float t = -b - sqrtf(disc);
                        if (t < 0.f) { q = add(xyz(p4), mul(dir, t)); ret = -1; }
                        else if (!(t > l)) { q = add(xyz(p4), mul(dir, t)); ret = 1; }
                    }
                }
            }
            if (d.dbg_sphere) d.dbg_sphere[g] = (int8_t)ret;
            if (ret == -1) {
                const float3 qs = add(sc, mul(normalize(sub(q, sc)), rad));
                const float3 ns = normalize(sub(qs, sc));
                d.xp[g] = f4(add(qs, mul(ns, 0.0001f)), p4.w);
                buf0[i] = f4(qs, x4.w);
            } else if (ret == 1) {
                const float3 ns = normalize(sub(q, sc));
                buf0[i] = f4(add(q, mul(ns, 0.0001f)), x4.w);
            }
        }
        cluster.sync();
    }

    const uint32_t nvf = (uint32_t)min((uint64_t)*a.nvf, d.vf_cap);
    const float h = cd.h;
    float4 *xa = buf0, *xb = buf1;
    for (int it = 0; it < cd.iters; ++it) {
        for (int i = tid; i < n_own; i += bs) {
            const int g = vo + lo + i;
            const float4 xi4 = xa[i];
            const float3 xi = xyz(xi4);
            float3 acc = f3(0.f, 0.f, 0.f);
            int cnt = 0;
            // ground, Physics/CudaPBD.cu:1594-1629
            const float cv = xi4.y - gq[i];
            const bool ground = cv < 0.f;
            if (ground) { acc.y = acc.y + -cv; cnt += 1; }
            if (d.dbg_ground_it) {
                const uint32_t bit = ground ? (1u << it) : 0u;
                d.dbg_ground_it[g] = it == 0 ? bit : (d.dbg_ground_it[g] | bit);
            }
            // LRA, Physics/CudaPBD.cu:1656-1688
            const uint8_t lf = lra[i];
            if (lf) {
                float3 la = f3(0.f, 0.f, 0.f);
                int lc = 0;
                const int64_t base = cd.lra_off + (int64_t)(lo + i) * cd.F;
                for (int j = 0; j < cd.F; ++j) {
                    if (!((lf >> j) & 1u)) continue;
                    const float3 diff = sub(xi, xyz(X(xa, d.fixed[cd.f_off + j] - vo)));
                    const float l = len(diff);
                    const float3 n = dvs(diff, l);
                    la = add(la, mul(n, -(l - d.lra_l0[base + j])));
                    ++lc;
                }
                acc = add(acc, la);
                cnt += lc;
            }
            // static slots, Physics/CudaPBD.cu:942-1147, 1417-1446
            {
                float3 sa = f3(0.f, 0.f, 0.f);
                const int s0 = __ldg(&d.soff[g]), s1 = __ldg(&d.soff[g + 1]);
                for (int e = s0; e < s1; ++e) {
                    const uint32_t ent = __ldg(&d.sent[e]);
                    const uint32_t k = ent & 0x1FFFFFFFu;
                    const int role = (int)((ent >> 29) & 3u);
                    float3 corr;
                    if (ent >> 31) {
                        const int4 id = __ldg(&d.b_ids[k]);
                        corr = bend_corr_pos(X(xa, id.x - vo), X(xa, id.y - vo), X(xa, id.z - vo), X(xa, id.w - vo),
                                             __ldg(&d.b_kp[k]), d.kpi_gap, role);
                    } else {
                        const int2 id = __ldg(&d.s_ids[k]);
                        const float2 par = __ldg(&d.s_par[k]);
                        corr = stretch_corr_pos(X(xa, id.x - vo), X(xa, id.y - vo), par.x, par.y, role);
                    }
                    sa = add(sa, corr);
                }
                acc = add(acc, sa);
                cnt += s1 - s0;
            }
            // dynamic VF / EE, counted when non-zero (Physics/CudaPBD.cu:1448-1475)
            {
                const uint32_t e0 = d.dyn_off[g], e1 = d.dyn_off[g + 1];
                if (e1 > e0) {
                    float3 da = f3(0.f, 0.f, 0.f);
                    int dc = 0;
                    for (uint32_t e = e0; e < e1; ++e) {
                        const uint32_t ent = d.dyn_ent[e];
                        const uint32_t ci = ent >> 2;
                        const int slot = (int)(ent & 3u);
                        const bool isvf = ci < nvf;
                        const int4 v = isvf ? d.vf_v[ci] : d.ee_v[ci - nvf];
                        const float4 w = isvf ? d.vf_w[ci] : d.ee_w[ci - nvf];
                        const float3 corr = contact_corr_pos(X(xa, v.x - vo), X(xa, v.y - vo), X(xa, v.z - vo),
                                                             X(xa, v.w - vo), w, isvf, h, slot);
                        const bool nz = !is_zero(corr);
                        if (nz) { da = add(da, corr); ++dc; }
                        if (d.dbg_dyn_nz) d.dbg_dyn_nz[(size_t)it * d.dyn_cap + ent] = nz ? 1 : 0;
                    }
                    acc = add(acc, da);
                    cnt += dc;
                }
            }
            // FinalCorrectionStep, Physics/CudaPBD.cu:1690-1698
            xb[i] = f4(add(xi, dvs(acc, (float)cnt)), xi4.w);
        }
        cluster.sync();
        float4 *t = xa;
        xa = xb;
        xb = t;
    }

    // ---- integration + world box (Physics/CudaPBD.cu:1916-1932,
    //      Physics/CudaDeformableUtils.cu:260-269) -----------------------------
    for (int i = tid; i < n_own; i += bs) {
        const int g = vo + lo + i;
        const float4 x4 = xa[i];
        float3 p = xyz(x4);
        if (x4.w == 0.f) {
            d.v[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const float4 p4 = d.xp[g];
            d.v[g] = f4(dvs(sub(p, xyz(p4)), cd.dt), 0.f);
            d.xp[g] = f4(p, p4.w);
        }
        p = f3(fminf(fmaxf(p.x, cd.wmin[0]), cd.wmax[0]), fminf(fmaxf(p.y, cd.wmin[1]), cd.wmax[1]),
               fminf(fmaxf(p.z, cd.wmin[2]), cd.wmax[2]));
        d.x[g] = f4(p, x4.w);
    }
}

size_t cluster_smem_bytes(int chunk_cap) { return (size_t)chunk_cap * kClusterBytesPerVertex + 64; }

// Largest per-CTA vertex range the device's shared memory allows.
int cluster_chunk_cap() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (optin <= 0) optin = 48 * 1024;
    return (optin - 128) / kClusterBytesPerVertex;
}

template <int CS>
static cudaError_t launch_cs(const DevPtrs &d, const ClusterArgs &a, int nclusters, cudaStream_t st) {
    const size_t smem = cluster_smem_bytes(a.chunk_cap);
    cudaError_t e = cudaFuncSetAttribute(k_solve_cluster<CS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (CS > 8) {
        e = cudaFuncSetAttribute(k_solve_cluster<CS>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nclusters * CS);
    cfg.blockDim = dim3(kClusterBlock);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve_cluster<CS>, d, a);
}

cudaError_t launch_solve_cluster(const DevPtrs &d, const ClusterArgs &a, int cs, int nclusters, cudaStream_t st) {
    if (cs == 16) return launch_cs<16>(d, a, nclusters, st);
    return launch_cs<8>(d, a, nclusters, st);
}

// How many clusters of cs CTAs the device can hold at once (0: unsupported).
int cluster_max_active(int cs, int chunk_cap) {
    const size_t smem = cluster_smem_bytes(chunk_cap);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs * 64);
    cfg.blockDim = dim3(kClusterBlock);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    cudaError_t e;
    if (cs == 16) {
        cudaFuncSetAttribute(k_solve_cluster<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_solve_cluster<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaOccupancyMaxActiveClusters(&n, k_solve_cluster<16>, &cfg);
    } else {
        cudaFuncSetAttribute(k_solve_cluster<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        e = cudaOccupancyMaxActiveClusters(&n, k_solve_cluster<8>, &cfg);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace lc
