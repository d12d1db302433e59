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
    int contact_gather;      // scatter solver: contacts gathered per owned vertex (no remote atomics)
};

// A recorded step's iterations past a cloth's own count (the tape holds the
// batch's largest): the iterate repeats and no collider slot is projected,
// as the global-memory solver records them.
__device__ __forceinline__ void record_tail(const DevPtrs &d, const ClothDev &cd, int g0, int n_own,
                                            const float4 *xs, int tid, int bs) {
    if (!d.tape_x) return;
    for (int it = cd.iters; it < d.tape_K; ++it)
        for (int i = tid; i < n_own; i += bs) {
            d.tape_x[(size_t)(it + 1) * d.Vtot + g0 + i] = xs[i];
            if (d.coll_act) d.coll_act[(size_t)(it + 1) * d.Vtot + g0 + i] = 0;
        }
}

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

    // owner CTA of local vertex li = li / chunk, as a multiply-high by
    // ceil(2^32 / chunk): exact for li, chunk < 2^16
    const uint32_t magic = (uint32_t)((0x100000000ull + chunk - 1) / chunk);
    auto X = [&](const float4 *xs, int li) -> float4 {
        const int o = (int)__umulhi((uint32_t)li, magic);
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
        if (d.dbg_ground_it || d.friction_any) d.ground_qc[g] = qdbg;
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
    if (d.tape_x)  // a recorded step: x^0 = the prediction after the set-up
        for (int i = tid; i < n_own; i += bs) d.tape_x[vo + lo + i] = buf0[i];
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
                    if ((ent >> 31) && cd.tri_bend) {
                        const int4 id = __ldg(&d.b_ids[k]);
                        corr = tri_bend_corr_pos(X(xa, id.x - vo), X(xa, id.y - vo), X(xa, id.z - vo),
                                                 __ldg(&d.b_kp[k]), __int_as_float(id.w), role);
                    } else if (ent >> 31) {
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
            float3 xn = add(xi, dvs(acc, (float)cnt));
            if (d.any_collider) {
                uint8_t *act = d.coll_act ? d.coll_act + (size_t)(it + 1) * d.Vtot + g : nullptr;
                if (xi4.w != 0.f) xn = collider_project(d, g, xn, h, act);
                else if (act) *act = 0;
            }
            xb[i] = f4(xn, xi4.w);
            if (d.tape_x) d.tape_x[(size_t)(it + 1) * d.Vtot + g] = xb[i];
        }
        cluster.sync();
        float4 *t = xa;
        xa = xb;
        xb = t;
    }
    record_tail(d, cd, vo + lo, n_own, xa, tid, bs);

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


// ---------------------------------------------------------------------------
// Scatter variant: every constraint is evaluated once per iteration by one
// thread of the cluster, which adds its corrections to the owners'
// accumulators (local or distributed shared memory).  Accumulators are
// fixed-point integers, so the sums are exact and independent of the order
// the atomics land in, and results stay deterministic.
// Shared memory per vertex: x (16) + two packed sums (16) + ground (4) + LRA
// flags (1).
// ---------------------------------------------------------------------------
// Correction sums in 32-bit fixed point: 2^25 per metre, i.e. 3e-8 m steps
// (finer than a float's spacing at 1 m) and +-64 m of range.  Two 64-bit
// words per vertex hold the four sums, so one correction costs two atomics:
//   xc = X * 2^32 + count  (the count never reaches 2^32, so it never carries
//                           into X, and X wraps like a 32-bit sum)
//   yz = Y * 2^32 + Z      (an exact 64-bit integer sum: Z is the low word
//                           read as signed, Y = (yz - Z) / 2^32)
// The decoded sums are the same integers as four separate 32-bit sums.
constexpr int kScatterBytesPerVertex = 37;
constexpr float kFix = 33554432.f;           // 2^25
constexpr float kFixInv = 1.f / 33554432.f;  // exact power of two

template <int CS>
__global__ void __launch_bounds__(kClusterBlock, 2) k_solve_cluster_scatter(DevPtrs d, ClusterArgs a) {
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
    float4 *xs = smem4;
    unsigned long long *axc = reinterpret_cast<unsigned long long *>(xs + cap);
    unsigned long long *ayz = axc + cap;
    float *gq = reinterpret_cast<float *>(ayz + cap);
    uint8_t *lra = reinterpret_cast<uint8_t *>(gq + cap);
    const uint32_t magic = (uint32_t)((0x100000000ull + chunk - 1) / chunk);
    auto owner = [&](int li) { return (int)__umulhi((uint32_t)li, magic); };
    auto X = [&](int li) -> float4 {
        const int o = owner(li);
        if (o == r) return xs[li - lo];
        return cluster.map_shared_rank(xs, o)[li - o * chunk];
    };
    auto add_corr = [&](int li, float3 v, bool count) {
        const int o = owner(li);
        const int k = li - o * chunk;
        unsigned long long *pxc = o == r ? axc : cluster.map_shared_rank(axc, o);
        unsigned long long *pyz = o == r ? ayz : cluster.map_shared_rank(ayz, o);
        const int ix = __float2int_rn(v.x * kFix), iy = __float2int_rn(v.y * kFix), iz = __float2int_rn(v.z * kFix);
        atomicAdd(pxc + k, ((unsigned long long)(uint32_t)ix << 32) + (count ? 1ull : 0ull));
        atomicAdd(pyz + k, ((unsigned long long)(uint32_t)iy << 32) + (unsigned long long)(long long)iz);
    };
    const float qnan = __int_as_float(0x7fc00000);
    for (int i = tid; i < n_own; i += bs) {
        const int g = vo + lo + i;
        const float4 x4 = d.x[g];
        xs[i] = x4;
        axc[i] = ayz[i] = 0ull;
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
            q = (isfinite(qc.x) && isfinite(qc.z)) ? qc.y : qnan;
            qdbg = f4(qc, 1.f);
        }
        gq[i] = q;
        if (d.dbg_ground_it || d.friction_any) d.ground_qc[g] = qdbg;
    }
    cluster.sync();
    if (cd.F) {
        for (int i = tid; i < n_own; i += bs) {
            const float4 x4 = xs[i];
            uint8_t f = 0;
            const int64_t base = cd.lra_off + (int64_t)(lo + i) * cd.F;
            if (x4.w != 0.f)
                for (int j = 0; j < cd.F; ++j)
                    if (dist(xyz(x4), xyz(X(d.fixed[cd.f_off + j] - vo))) > d.lra_l0[base + j]) f |= (uint8_t)(1u << j);
            lra[i] = f;
            if (d.dbg_ground_it)
                for (int j = 0; j < cd.F; ++j) d.lra_flag[base + j] = (f >> j) & 1u;
        }
        cluster.sync();
    }
    if (cd.sphere_on) {
        const float3 sc = f3(cd.sphere_pos[0], cd.sphere_pos[1], cd.sphere_pos[2]);
        const float rad = cd.sphere_r + cd.h;
        for (int i = tid; i < n_own; i += bs) {
            const int g = vo + lo + i;
            const float4 x4 = xs[i], p4 = d.xp[g];
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
                xs[i] = f4(qs, x4.w);
            } else if (ret == 1) {
                const float3 ns = normalize(sub(q, sc));
                xs[i] = f4(add(q, mul(ns, 0.0001f)), x4.w);
            }
        }
        cluster.sync();
    }
    const uint4 cr = d.crange[c];
    const uint32_t nvf_all = (uint32_t)min((uint64_t)*a.nvf, d.vf_cap);
    const float h = cd.h;
    // this CTA's share of the cloth's constraints (index order ~ vertex order)
    const int s_per = (cd.s_cnt + CS - 1) / CS, b_per = (cd.b_cnt + CS - 1) / CS;
    const int sb = cd.s_off + min(cd.s_cnt, r * s_per), se = cd.s_off + min(cd.s_cnt, (r + 1) * s_per);
    const int bb = cd.b_off + min(cd.b_cnt, r * b_per), be = cd.b_off + min(cd.b_cnt, (r + 1) * b_per);
    if (d.tape_x)  // a recorded step: x^0 = the prediction after the set-up
        for (int i = tid; i < n_own; i += bs) d.tape_x[vo + lo + i] = xs[i];
    for (int it = 0; it < cd.iters; ++it) {
        for (int k = sb + tid; k < se; k += bs) {
            const int2 id = __ldg(&d.s_ids[k]);
            const float2 par = __ldg(&d.s_par[k]);
            const int i1 = id.x - vo, i2 = id.y - vo;
            const float4 p1 = X(i1), p2 = X(i2);
            add_corr(i1, stretch_corr_pos(p1, p2, par.x, par.y, 0), false);
            add_corr(i2, stretch_corr_pos(p1, p2, par.x, par.y, 1), false);
        }
        for (int k = bb + tid; k < (cd.tri_bend ? bb : be); k += bs) {
            const int4 id = __ldg(&d.b_ids[k]);
            const float kp = __ldg(&d.b_kp[k]);
            const int li[4] = {id.x - vo, id.y - vo, id.z - vo, id.w - vo};
            const float4 p[4] = {X(li[0]), X(li[1]), X(li[2]), X(li[3])};
            float3 q[4];
            float s;
            if (bend_all_pos(p[0], p[1], p[2], p[3], kp, d.kpi_gap, q, s)) {
#pragma unroll
                for (int j = 0; j < 4; ++j) add_corr(li[j], mul(q[j], -(p[j].w * s)), false);
            }
        }
        // triangle bends (Physics/CudaPBD.cu:1149-1187), when the cloth uses them
        for (int k = bb + tid; k < (cd.tri_bend ? be : bb); k += bs) {
            const int4 id = __ldg(&d.b_ids[k]);
            const float kp = __ldg(&d.b_kp[k]), h0 = __int_as_float(id.w);
            const int li[3] = {id.x - vo, id.y - vo, id.z - vo};
            const float4 p[3] = {X(li[0]), X(li[1]), X(li[2])};
#pragma unroll
            for (int j = 0; j < 3; ++j) add_corr(li[j], tri_bend_corr_pos(p[0], p[1], p[2], kp, h0, j), false);
        }
        if (a.contact_gather) {
            // Contacts by owned vertex: each entry of the per-vertex contact
            // lists (one contact slot) is evaluated by the CTA that owns the
            // slot's vertex, whose accumulators are then local; every
            // contact is evaluated once per slot instead of once.
            const uint32_t e0 = d.dyn_off[vo + lo], e1 = d.dyn_off[vo + lo + n_own];
            for (uint32_t e = e0 + tid; e < e1; e += bs) {
                const uint32_t ent = d.dyn_ent[e];
                const uint32_t ci = ent >> 2;
                const int slot = (int)(ent & 3u);
                const bool isvf = ci < nvf_all;
                const int4 v = isvf ? d.vf_v[ci] : d.ee_v[ci - nvf_all];
                const float4 w = isvf ? d.vf_w[ci] : d.ee_w[ci - nvf_all];
                const int li[4] = {v.x - vo, v.y - vo, v.z - vo, v.w - vo};
                const float4 P[4] = {X(li[0]), X(li[1]), X(li[2]), X(li[3])};
                const float3 corr = contact_corr_pos(P[0], P[1], P[2], P[3], w, isvf, h, slot);
                const bool nz = !is_zero(corr);
                if (nz) add_corr(li[slot], corr, true);
                if (d.dbg_dyn_nz) d.dbg_dyn_nz[(size_t)it * d.dyn_cap + ent] = nz ? 1 : 0;
            }
        }
        const uint32_t nv = cr.y - cr.x, ncont = a.contact_gather ? 0u : nv + (cr.w - cr.z);
        for (uint32_t k = r * bs + tid; k < ncont; k += CS * bs) {
            const bool isvf = k < nv;
            const uint32_t gi = isvf ? cr.x + k : cr.z + (k - nv);
            const int4 v = isvf ? d.vf_v[gi] : d.ee_v[gi];
            const float4 w = isvf ? d.vf_w[gi] : d.ee_w[gi];
            const int li[4] = {v.x - vo, v.y - vo, v.z - vo, v.w - vo};
            const float4 P[4] = {X(li[0]), X(li[1]), X(li[2]), X(li[3])};
            const uint32_t ent = 4u * (isvf ? gi : nvf_all + gi);
            float3 cs[4];
            contact_all_pos(P[0], P[1], P[2], P[3], w, isvf, h, cs);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float3 corr = cs[j];
                const bool nz = !is_zero(corr);
                if (nz) add_corr(li[j], corr, true);
                if (d.dbg_dyn_nz) d.dbg_dyn_nz[(size_t)it * d.dyn_cap + ent + j] = nz ? 1 : 0;
            }
        }
        for (int i = tid; i < n_own; i += bs) {
            const float4 x4 = xs[i];
            const float cv = x4.y - gq[i];
            const bool ground = cv < 0.f;
            if (ground) {
                atomicAdd(ayz + i, (unsigned long long)(uint32_t)__float2int_rn(-cv * kFix) << 32);
                atomicAdd(axc + i, 1ull);
            }
            if (d.dbg_ground_it) {
                const uint32_t bit = ground ? (1u << it) : 0u;
                d.dbg_ground_it[vo + lo + i] = it == 0 ? bit : (d.dbg_ground_it[vo + lo + i] | bit);
            }
            const uint8_t f = lra[i];
            if (f) {
                const int64_t base = cd.lra_off + (int64_t)(lo + i) * cd.F;
                for (int j = 0; j < cd.F; ++j) {
                    if (!((f >> j) & 1u)) continue;
                    const float3 diff = sub(xyz(x4), xyz(X(d.fixed[cd.f_off + j] - vo)));
                    const float l = len(diff);
                    const float3 n = dvs(diff, l);
                    add_corr(lo + i, mul(n, -(l - d.lra_l0[base + j])), true);
                }
            }
        }
        cluster.sync();
        for (int i = tid; i < n_own; i += bs) {
            const int g = vo + lo + i;
            const unsigned long long xc = axc[i], yz = ayz[i];
            const int sx = (int)(uint32_t)(xc >> 32), sz = (int)(uint32_t)yz;
            const int sy = (int)(uint32_t)((yz - (unsigned long long)(long long)sz) >> 32);
            const float n = (float)(__ldg(&d.soff[g + 1]) - __ldg(&d.soff[g]) + (int)(uint32_t)xc);
            float4 x4 = xs[i];
            x4.x += (__int2float_rn(sx) * kFixInv) / n;
            x4.y += (__int2float_rn(sy) * kFixInv) / n;
            x4.z += (__int2float_rn(sz) * kFixInv) / n;
            if (d.any_collider) {
                uint8_t *act = d.coll_act ? d.coll_act + (size_t)(it + 1) * d.Vtot + g : nullptr;
                if (x4.w != 0.f) x4 = f4(collider_project(d, g, xyz(x4), h, act), x4.w);
                else if (act) *act = 0;
            }
            xs[i] = x4;
            if (d.tape_x) d.tape_x[(size_t)(it + 1) * d.Vtot + g] = x4;
            axc[i] = ayz[i] = 0ull;
        }
        cluster.sync();
    }
    record_tail(d, cd, vo + lo, n_own, xs, tid, bs);
    for (int i = tid; i < n_own; i += bs) {
        const int g = vo + lo + i;
        const float4 x4 = xs[i];
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

size_t cluster_smem_bytes(int chunk_cap, bool scatter) {
    return (size_t)chunk_cap * (scatter ? kScatterBytesPerVertex : kClusterBytesPerVertex) + 128;
}

// Largest per-CTA vertex range the device's shared memory allows.
int cluster_chunk_cap(bool scatter) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (optin <= 0) optin = 48 * 1024;
    return (optin - 256) / (scatter ? kScatterBytesPerVertex : kClusterBytesPerVertex);
}

template <int CS, bool SCATTER>
static cudaError_t configure(size_t smem) {
    auto k = SCATTER ? k_solve_cluster_scatter<CS> : k_solve_cluster<CS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (CS > 8) e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

static cudaLaunchConfig_t cluster_cfg(int cs, int nclusters, size_t smem, cudaStream_t st, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nclusters * cs);
    cfg.blockDim = dim3(kClusterBlock);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <int CS, bool SCATTER>
static cudaError_t launch_cs(const DevPtrs &d, const ClusterArgs &a, int nclusters, cudaStream_t st) {
    const size_t smem = cluster_smem_bytes(a.chunk_cap, SCATTER);
    cudaError_t e = configure<CS, SCATTER>(smem);
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_cfg(CS, nclusters, smem, st, attr);
    return cudaLaunchKernelEx(&cfg, SCATTER ? k_solve_cluster_scatter<CS> : k_solve_cluster<CS>, d, a);
}

cudaError_t launch_solve_cluster(const DevPtrs &d, const ClusterArgs &a, int cs, bool scatter, int nclusters,
                                 cudaStream_t st) {
    if (cs == 16) return scatter ? launch_cs<16, true>(d, a, nclusters, st) : launch_cs<16, false>(d, a, nclusters, st);
    if (cs == 4) return scatter ? launch_cs<4, true>(d, a, nclusters, st) : launch_cs<4, false>(d, a, nclusters, st);
    return scatter ? launch_cs<8, true>(d, a, nclusters, st) : launch_cs<8, false>(d, a, nclusters, st);
}

template <int CS, bool SCATTER>
static int max_active(int chunk_cap) {
    const size_t smem = cluster_smem_bytes(chunk_cap, SCATTER);
    if (configure<CS, SCATTER>(smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_cfg(CS, 64, smem, nullptr, attr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, SCATTER ? k_solve_cluster_scatter<CS> : k_solve_cluster<CS>, &cfg) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// How many clusters of cs CTAs the device can hold at once (0: unsupported).
int cluster_max_active(int cs, int chunk_cap, bool scatter) {
    if (cs == 16) return scatter ? max_active<16, true>(chunk_cap) : max_active<16, false>(chunk_cap);
    if (cs == 4) return scatter ? max_active<4, true>(chunk_cap) : max_active<4, false>(chunk_cap);
    return scatter ? max_active<8, true>(chunk_cap) : max_active<8, false>(chunk_cap);
}

}  // namespace lc
