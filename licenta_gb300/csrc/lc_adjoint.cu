// lc_adjoint.cu — reverse pass (adjoint) of one cloth step on the
// global-memory solver path, with the step's discrete decisions held fixed as
// the recorded forward step took them: the contact set and its weights, ground
// and LRA activation, and the dynamic terms counted in each Jacobi iteration.
// The analytic sphere and the wind term's vertex normals are held fixed; the
// static colliders' contact planes are fixed, their projections reversed.
//
// Given dL/d(x, x_prev, v) after the step, the kernels produce dL/d(x, x_prev,
// v) before it and add dL/dk of every stretch and bend constraint.  Order:
// integration reversed, the Jacobi iterations reversed (per constraint a
// vector-Jacobian product written to its CSR slots, then a per-vertex gather
// in a fixed order), prediction reversed, damping reversed (per-cloth sums).
#include "lc_internal.cuh"

namespace lc {

namespace {

constexpr int kAdjFixedMax = 8;  // pinned vertices per cloth reduced in shared memory
// The rescaled reverse pass: a cloth whose state gradients exceed 2^60 has all
// its accumulators multiplied by 2^-60 (contact-rich rollouts amplify the
// gradient by up to ~1e14 per 20 steps, and the float range ends near 2^128).
constexpr float kRescaleAbove = 0x1p60f;
constexpr float kRescaleBy = 0x1p-60f;

// f(d) = (|d| - l0) d/|d| (stretch, LRA and contact corrections); its
// Jacobian I - (l0/|d|)(I - n n^T) is symmetric, applied here to g.
__device__ __forceinline__ float3 f_jac(float3 d, float l, float l0, float3 g) {
    const float3 n = dvs(d, l);
    return sub(g, mul(sub(g, mul(n, dot(n, g))), l0 / l));
}

// kp = 1 - (1 - k)^(1/K) (Physics/CudaPBD.cu:277-370), so dkp/dk = (1 - kp)^(1-K) / K.
__device__ __forceinline__ float dkp_dk(float kp, int K) { return powf(1.f - kp, 1.f - (float)K) / (float)K; }

// Reverse of the bend correction (Physics/CudaPBD.cu:1024-1147) on the stable
// form of lc_pbd.cuh: ub[j] are the gradients arriving at the four
// corrections; returns the gradients of p2, p3, p4 (p1 does not enter) and kp.
__device__ void bend_vjp(float3 p2, float3 p3, float3 p4, const float w[4], float kp, float gap, const float3 ub[4],
                         float3 &g2, float3 &g3, float3 &g4, float &gkp) {
    const float3 z = f3(0.f, 0.f, 0.f);
    g2 = g3 = g4 = z;
    gkp = 0.f;
    const float3 c23 = cross(p2, p3), c24 = cross(p2, p4);
    const float l23 = len(c23), l24 = len(c24);
    if (l23 <= kEpsPbd || l24 <= kEpsPbd) return;
    const float3 n1 = dvs(c23, l23), n2 = dvs(c24, l24);
    const float3 sv = add(n1, n2), tv = sub(n1, n2);
    const float ss = dot(sv, sv), tt = dot(tv, tv);
    if (ss == 0.f) return;
    const float A = sqrtf(ss), Bq = sqrtf(tt);
    const float dphi = gap - 2.f * atan2f(A, Bq);
    const float Rt = sqrtf(ss * tt * 0.25f);
    const float term = Rt * dphi * kp;
    const float opd = 0.5f * ss;
    const float3 u = sub(sv, mul(n1, opd)), wv = sub(sv, mul(n2, opd));
    const float3 a3 = cross(p2, u), a4 = cross(p2, wv), b3 = cross(p3, u), b4 = cross(p4, wv);
    float3 q[4];
    q[2] = dvs(a3, l23);
    q[3] = dvs(a4, l24);
    q[1] = neg(add(dvs(b3, l23), dvs(b4, l24)));
    q[0] = sub(sub(neg(q[1]), q[2]), q[3]);
    const float sf = w[0] * dot(q[0], q[0]) + w[1] * dot(q[1], q[1]) + w[2] * dot(q[2], q[2]) + w[3] * dot(q[3], q[3]);
    if (sf <= kEpsPbd) return;
    const float sc = term / sf;
    float gsc = 0.f;
    float3 gq[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        gsc += -w[j] * dot(q[j], ub[j]);
        gq[j] = mul(ub[j], -w[j] * sc);
    }
    const float gterm = gsc / sf, gsf = -gsc * sc / sf;
#pragma unroll
    for (int j = 0; j < 4; ++j) gq[j] = add(gq[j], mul(q[j], 2.f * w[j] * gsf));
    gq[1] = sub(gq[1], gq[0]);
    gq[2] = sub(gq[2], gq[0]);
    gq[3] = sub(gq[3], gq[0]);
    const float3 gb3 = dvs(neg(gq[1]), l23), gb4 = dvs(neg(gq[1]), l24);
    const float gl23 = (dot(gq[1], b3) - dot(gq[2], a3)) / (l23 * l23);
    const float gl24 = (dot(gq[1], b4) - dot(gq[3], a4)) / (l24 * l24);
    const float3 ga3 = dvs(gq[2], l23), ga4 = dvs(gq[3], l24);
    float3 gu = z, gw = z;
    g2 = add(g2, cross(u, ga3)); gu = add(gu, cross(ga3, p2));
    g2 = add(g2, cross(wv, ga4)); gw = add(gw, cross(ga4, p2));
    g3 = add(g3, cross(u, gb3)); gu = add(gu, cross(gb3, p3));
    g4 = add(g4, cross(wv, gb4)); gw = add(gw, cross(gb4, p4));
    float3 gsv = add(gu, gw), gn1 = mul(gu, -opd), gn2 = mul(gw, -opd);
    float gss = -(dot(gu, n1) + dot(gw, n2)) * 0.5f, gtt = 0.f;
    const float gRt = gterm * dphi * kp, gdphi = gterm * Rt * kp;
    gkp = gterm * Rt * dphi;
    if (Rt > 0.f) {
        const float gP = gRt / (2.f * Rt);
        gss += gP * tt * 0.25f;
        gtt += gP * ss * 0.25f;
    }
    const float den = ss + tt;
    const float gA = -2.f * Bq / den * gdphi, gB = 2.f * A / den * gdphi;
    gss += gA / (2.f * A);
    if (Bq > 0.f) gtt += gB / (2.f * Bq);
    gsv = add(gsv, mul(sv, 2.f * gss));
    const float3 gtv = mul(tv, 2.f * gtt);
    gn1 = add(add(gn1, gsv), gtv);
    gn2 = sub(add(gn2, gsv), gtv);
    const float3 gc23 = add(dvs(gn1, l23), mul(n1, gl23 - dot(gn1, c23) / (l23 * l23)));
    const float3 gc24 = add(dvs(gn2, l24), mul(n2, gl24 - dot(gn2, c24) / (l24 * l24)));
    g2 = add(add(g2, cross(p3, gc23)), cross(p4, gc24));
    g3 = add(g3, cross(gc23, p2));
    g4 = add(g4, cross(gc24, p2));
}

// Block sums of N floats, partials in double, written in a fixed order.
template <int N>
__device__ __forceinline__ void block_sums(float (&v)[N], double *dst) {
    __shared__ double red[N][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float s = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[k][wid] = (double)s;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[threadIdx.x][w];
        dst[threadIdx.x] = t;
    }
}

__device__ __forceinline__ float3 in_box(float3 g, float3 p, const ClothDev &cd) {
    return f3((p.x > cd.wmin[0] && p.x < cd.wmax[0]) ? g.x : 0.f, (p.y > cd.wmin[1] && p.y < cd.wmax[1]) ? g.y : 0.f,
              (p.z > cd.wmin[2] && p.z < cd.wmax[2]) ? g.z : 0.f);
}

}  // namespace

// _FinalUpdate (Physics/CudaPBD.cu:1916-1932) and _WorldConstraints
// (Physics/CudaDeformableUtils.cu:260-269) reversed: v = (x_s - x_prev)/dt,
// x_prev' = x_s, x' = clamp(x_s); pinned vertices keep x_prev and get v = 0.
__global__ void k_adj_integrate(DevPtrs d, AdjPtrs A, float4 *a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const ClothDev &cd = d.cloth[d.vcloth[i]];
    const float4 xs = A.tape_x[(size_t)A.K * d.Vtot + i];
    const float3 gc = in_box(xyz(A.gx[i]), xyz(xs), cd);
    if (xs.w == 0.f) {
        a[i] = f4(gc, 0.f);
    } else {
        const float3 gv = xyz(A.gv[i]);
        a[i] = f4(add(add(xyz(A.gxp[i]), dvs(gv, cd.dt)), gc), 0.f);
        A.gxp[i] = f4(neg(dvs(gv, cd.dt)), 0.f);
    }
}

// Terms counted for vertex i in iteration it (Physics/CudaPBD.cu:1690-1698
// divides the summed corrections by that count) and u = dL/dx^{k+1} / count.
__global__ void k_adj_u(DevPtrs d, AdjPtrs A, const float4 *a, int it) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const ClothDev &cd = d.cloth[d.vcloth[i]];
    if (it >= cd.iters) { A.u[i] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    int cnt = d.soff[i + 1] - d.soff[i] + (int)((d.dbg_ground_it[i] >> it) & 1u);
    const int64_t base = cd.lra_off + (int64_t)(i - cd.v_off) * cd.F;
    for (int j = 0; j < cd.F; ++j) cnt += d.lra_flag[base + j] ? 1 : 0;
    const uint8_t *nz = d.dbg_dyn_nz + (size_t)it * d.dyn_cap;
    for (uint32_t e = d.dyn_off[i]; e < d.dyn_off[i + 1]; ++e) cnt += nz[d.dyn_ent[e]] ? 1 : 0;
    A.u[i] = cnt ? f4(dvs(xyz(a[i]), (float)cnt), 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Stretch (Physics/CudaPBD.cu:986-1022): corr1 = -w1 kp/ws f(x1 - x2),
// corr2 = +w2 kp/ws f(x1 - x2).
__device__ __forceinline__ void adj_stretch_one(const DevPtrs &d, const AdjPtrs &A, int it, float *gk, int c) {
    const int2 id = d.s_ids[c];
    const float2 par = d.s_par[c];
    const ClothDev &cd = d.cloth[d.vcloth[id.x]];
    float3 dd = f3(0.f, 0.f, 0.f);
    if (it < cd.iters) {
        const float4 *X = A.tape_x + (size_t)it * d.Vtot;
        const float4 x1 = X[id.x], x2 = X[id.y];
        const float ws = x1.w + x2.w;
        if (ws != 0.f) {
            const float3 dv = sub(xyz(x1), xyz(x2));
            const float l = len(dv);
            if (l > kEpsPbd) {
                const float3 comb = dvs(sub(mul(xyz(A.u[id.y]), x2.w), mul(xyz(A.u[id.x]), x1.w)), ws);
                dd = f_jac(dv, l, par.x, mul(comb, par.y));
                if (gk) gk[c] += dot(sub(dv, mul(dv, par.x / l)), comb) * dkp_dk(par.y, cd.iters);
            }
        }
    }
    A.slot[A.s_slot[2 * c]] = f4(dd, 0.f);
    A.slot[A.s_slot[2 * c + 1]] = f4(neg(dd), 0.f);
}

// Bend (Physics/CudaPBD.cu:1024-1147).
__device__ __forceinline__ void adj_bend_one(const DevPtrs &d, const AdjPtrs &A, int it, float *gk, int c) {
    const int4 id = d.b_ids[c];
    const ClothDev &cd = d.cloth[d.vcloth[id.x]];
    float3 g2 = f3(0.f, 0.f, 0.f), g3 = g2, g4 = g2;
    if (it < cd.iters) {
        const float4 *X = A.tape_x + (size_t)it * d.Vtot;
        const float4 x1 = X[id.x], x2 = X[id.y], x3 = X[id.z], x4 = X[id.w];
        const float w[4] = {x1.w, x2.w, x3.w, x4.w};
        const float3 ub[4] = {xyz(A.u[id.x]), xyz(A.u[id.y]), xyz(A.u[id.z]), xyz(A.u[id.w])};
        const float kp = d.b_kp[c];
        float gkp;
        bend_vjp(xyz(x2), xyz(x3), xyz(x4), w, kp, d.kpi_gap, ub, g2, g3, g4, gkp);
        if (gk) gk[c] += gkp * dkp_dk(kp, cd.iters);
    }
    A.slot[A.b_slot[4 * c]] = make_float4(0.f, 0.f, 0.f, 0.f);
    A.slot[A.b_slot[4 * c + 1]] = f4(g2, 0.f);
    A.slot[A.b_slot[4 * c + 2]] = f4(g3, 0.f);
    A.slot[A.b_slot[4 * c + 3]] = f4(g4, 0.f);
}

// VF / EE contacts (Physics/CudaPBD.cu:1212-1415): with the contact's
// (frozen) barycentric weights b_s and signs, n = sum_s sgn_s b_s x_s and
// corr_s = -(w_s sgn_s b_s / sum_s w_s b_s^2) f(n) with l0 = thickness; only
// the entries counted in this iteration contribute.
__device__ __forceinline__ void adj_contacts(const DevPtrs &d, const AdjPtrs &A, int it, const uint32_t *nvf_dev,
                                             const uint32_t *nee_dev, uint32_t first, uint32_t stride) {
    const uint32_t nvf = (uint32_t)min((uint64_t)*nvf_dev, d.vf_cap);
    const uint32_t nee = (uint32_t)min((uint64_t)*nee_dev, d.ee_cap);
    const uint8_t *nz = d.dbg_dyn_nz + (size_t)it * d.dyn_cap;
    for (uint32_t c = first; c < nvf + nee; c += stride) {
        const bool isvf = c < nvf;
        const int4 v4 = isvf ? d.vf_v[c] : d.ee_v[c - nvf];
        const float4 w4 = isvf ? d.vf_w[c] : d.ee_w[c - nvf];
        const int v[4] = {v4.x, v4.y, v4.z, v4.w};
        const ClothDev &cd = d.cloth[d.vcloth[v[0]]];
        float3 ub[4];
        bool any = false;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const bool t = it < cd.iters && nz[c * 4 + s] != 0;
            ub[s] = t ? xyz(A.u[v[s]]) : f3(0.f, 0.f, 0.f);
            any = any || t;
        }
        float3 out[4] = {f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f)};
        if (any) {
            const float4 *X = A.tape_x + (size_t)it * d.Vtot;
            float b[4], sg[4];
            if (isvf) {
                b[0] = 1.f; b[1] = clampf(-w4.y, 0.f, 1.f); b[2] = clampf(-w4.z, 0.f, 1.f); b[3] = clampf(-w4.w, 0.f, 1.f);
                sg[0] = 1.f; sg[1] = sg[2] = sg[3] = -1.f;
            } else {
                b[0] = w4.x; b[1] = w4.y; b[2] = -w4.z; b[3] = -w4.w;
                sg[0] = sg[1] = 1.f; sg[2] = sg[3] = -1.f;
            }
            float wv[4], den = 0.f;
            float3 nv = f3(0.f, 0.f, 0.f);
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                const float4 xs = X[v[s]];
                wv[s] = xs.w;
                den += wv[s] * b[s] * b[s];
                nv = add(nv, mul(xyz(xs), sg[s] * b[s]));
            }
            if (den != 0.f) {
                float3 comb = f3(0.f, 0.f, 0.f);
#pragma unroll
                for (int s = 0; s < 4; ++s) comb = sub(comb, mul(ub[s], wv[s] * sg[s] * b[s] / den));
                const float3 dn = f_jac(nv, len(nv), cd.h, comb);
#pragma unroll
                for (int s = 0; s < 4; ++s) out[s] = mul(dn, sg[s] * b[s]);
            }
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) A.dyn[c * 4 + s] = f4(out[s], 0.f);
    }
}

// One iteration's vector-Jacobian products in one launch: blocks [0, nbs)
// take the stretch constraints, the next nbb blocks the bends and the rest
// the contacts (grid-stride).  They write disjoint buffers (the constraints'
// CSR slots, the contact entries) from the same inputs.
constexpr int kAdjBlock = 128;
__global__ void __launch_bounds__(kAdjBlock) k_adj_constraints(DevPtrs d, AdjPtrs A, int it, float *gks, float *gkb,
                                                               const uint32_t *nvf, const uint32_t *nee, int nbs,
                                                               int nbb) {
    const int bx = blockIdx.x;
    if (bx < nbs) {
        const int c = bx * kAdjBlock + threadIdx.x;
        if (c < A.E) adj_stretch_one(d, A, it, gks, c);
    } else if (bx < nbs + nbb) {
        const int c = (bx - nbs) * kAdjBlock + threadIdx.x;
        if (c < A.B) adj_bend_one(d, A, it, gkb, c);
    } else {
        const uint32_t nbc = gridDim.x - (uint32_t)(nbs + nbb);
        adj_contacts(d, A, it, nvf, nee, (uint32_t)(bx - nbs - nbb) * kAdjBlock + threadIdx.x, nbc * kAdjBlock);
    }
}

// dL/dx^k = dL/dx^{k+1} + the vertex's CSR slots and contact entries, the
// ground term (corr.y = -(x.y - ground - h), Physics/CudaPBD.cu:1594-1629) and
// LRA (corr = -f(x - x_pinned), :1656-1688); LRA's share for the pinned vertex
// is summed per block and added with one atomic per block.
__global__ void k_adj_gather(DevPtrs d, AdjPtrs A, const float4 *__restrict__ a, float4 *__restrict__ g, int it) {
    const int c = d.vblk_cloth[blockIdx.x];
    const ClothDev &cd = d.cloth[c];
    const int i = d.vblk_start[blockIdx.x] + threadIdx.x;
    const bool valid = i < cd.v_off + cd.V;
    const bool active = it < cd.iters;
    float fx[kAdjFixedMax][3];
#pragma unroll
    for (int j = 0; j < kAdjFixedMax; ++j) fx[j][0] = fx[j][1] = fx[j][2] = 0.f;
    if (valid) {
        float3 gi = xyz(a[i]);
        if (active) {
            const float3 ui = xyz(A.u[i]);
            for (int e = d.soff[i]; e < d.soff[i + 1]; ++e) gi = add(gi, xyz(A.slot[e]));
            for (uint32_t e = d.dyn_off[i]; e < d.dyn_off[i + 1]; ++e) gi = add(gi, xyz(A.dyn[d.dyn_ent[e]]));
            if ((d.dbg_ground_it[i] >> it) & 1u) gi.y -= ui.y;
            if (cd.F) {
                const float4 *X = A.tape_x + (size_t)it * d.Vtot;
                const int64_t base = cd.lra_off + (int64_t)(i - cd.v_off) * cd.F;
                for (int j = 0; j < cd.F; ++j) {
                    if (!d.lra_flag[base + j]) continue;
                    const int fj = d.fixed[cd.f_off + j];
                    const float3 dv = sub(xyz(X[i]), xyz(X[fj]));
                    const float3 dd = f_jac(dv, len(dv), d.lra_l0[base + j], neg(ui));
                    gi = add(gi, dd);
                    if (j < kAdjFixedMax) {
                        fx[j][0] -= dd.x; fx[j][1] -= dd.y; fx[j][2] -= dd.z;
                    } else {
                        atomicAdd(&A.fixed[3 * (cd.f_off + j)], -dd.x);
                        atomicAdd(&A.fixed[3 * (cd.f_off + j) + 1], -dd.y);
                        atomicAdd(&A.fixed[3 * (cd.f_off + j) + 2], -dd.z);
                    }
                }
            }
        }
        g[i] = f4(gi, 0.f);
    }
    if (cd.F == 0 || !active) return;  // uniform per block: blocks never straddle cloths
    __shared__ float red[kThreads / 32][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nf = min(cd.F, kAdjFixedMax);
    for (int j = 0; j < nf; ++j) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float s = fx[j][k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) red[wid][k] = s;
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            float t = 0.f;
            for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w][threadIdx.x];
            if (t != 0.f) atomicAdd(&A.fixed[3 * (cd.f_off + j) + threadIdx.x], t);
        }
        __syncthreads();
    }
}

__global__ void k_adj_fixed_add(DevPtrs d, AdjPtrs A, float4 *g, int nfixed) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nfixed) return;
    const int v = d.fixed[k];
    float4 gv = g[v];
    gv.x += A.fixed[3 * k]; gv.y += A.fixed[3 * k + 1]; gv.z += A.fixed[3 * k + 2];
    g[v] = gv;
    A.fixed[3 * k] = A.fixed[3 * k + 1] = A.fixed[3 * k + 2] = 0.f;
}

// The static-collider projections of one pass reversed (lc_batch_set_collider):
// each projected slot maps x to x - (n . x - d0 - h) n, whose Jacobian
// I - n n^T is symmetric; the slots were applied in order, so their
// transposes apply last slot first.  pass 0 is the projection before the
// solver, pass it + 1 the one ending iteration it.
__global__ void k_adj_collider(DevPtrs d, float4 *a, int pass) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const uint32_t m = d.coll_act[(size_t)pass * d.Vtot + i];
    if (!m) return;
    float3 g = xyz(a[i]);
    for (int k = kColliderSlots - 1; k >= 0; --k)
        if ((m >> k) & 1u) {
            const float3 n = xyz(d.cw[(size_t)i * kColliderSlots + k]);
            g = sub(g, mul(n, dot(n, g)));
        }
    a[i] = f4(g, 0.f);
}

// ExplicitEuler reversed (x_p = x_prev + dt v_c) and the sums the damping
// reverse needs: S1 = sum dL/dv_c, S2 = sum r x dL/dv_c, r = x - xcm.
__global__ void k_adj_damp1(DevPtrs d, AdjPtrs A, const float4 *a) {
    const int c = d.vblk_cloth[blockIdx.x];
    const ClothDev &cd = d.cloth[c];
    const double *t = d.damp + (size_t)c * 16;
    const int i = d.vblk_start[blockIdx.x] + threadIdx.x;
    // the mass centre once per block: FP64 division is slow on this part
    __shared__ float cm[3];
    if (threadIdx.x < 3) cm[threadIdx.x] = (float)(t[1 + threadIdx.x] / t[0]);
    __syncthreads();
    float s[6] = {0, 0, 0, 0, 0, 0};
    if (i < cd.v_off + cd.V) {
        const float3 ai = xyz(a[i]);
        A.gxp[i] = f4(add(xyz(A.gxp[i]), ai), 0.f);
        const float3 gvc = mul(ai, cd.dt);
        A.u[i] = f4(gvc, 0.f);
        const float3 xcm = f3(cm[0], cm[1], cm[2]);
        const float3 r = sub(xyz(A.tape_xin[i]), xcm);
        const float3 cr = cross(r, gvc);
        s[0] = gvc.x; s[1] = gvc.y; s[2] = gvc.z;
        s[3] = cr.x; s[4] = cr.y; s[5] = cr.z;
    }
    block_sums<6>(s, A.red + (size_t)blockIdx.x * 8);
}

__global__ void k_adj_totals(DevPtrs d, AdjPtrs A) {
    const int c = blockIdx.x;
    if (threadIdx.x >= 6) return;
    double s = 0;
    for (int b = d.vb_first[c]; b < d.vb_first[c + 1]; ++b) s += A.red[(size_t)b * 8 + threadIdx.x];
    A.red[(size_t)A.nvblk_red * 8 + (size_t)c * 8 + threadIdx.x] = s;
}

// DampVelocities (Physics/CudaPBD.cu:411-458) reversed:
//   v_c = v_b + kd (vcm + w x r - v_b),  w = I^-1 L,  L = sum m r x v_b,
//   I = sum m (|r|^2 Id - r r^T),  r = x - xcm;  then v_b = (v + dt g)(1 - kg).
__global__ void k_adj_damp2(DevPtrs d, AdjPtrs A) {
    const int c = d.vblk_cloth[blockIdx.x];
    const ClothDev &cd = d.cloth[c];
    __shared__ float sh[24];
    if (threadIdx.x == 0) {
        const double *t = d.damp + (size_t)c * 16;
        const double *S = A.red + (size_t)A.nvblk_red * 8 + (size_t)c * 8;
        const double ms = t[0];
        const double L[3] = {t[7], t[8], t[9]};
        const double i1x = t[10], i1y = t[11], i1z = t[12], i2x = t[13], i2y = t[14], i2z = t[15];
        const double I[3][3] = {{i1y + i1z, i2x, i2y}, {i2x, i1x + i1z, i2z}, {i2y, i2z, i1x + i1y}};
        const double c00 = I[1][1] * I[2][2] - I[1][2] * I[2][1], c01 = -(I[1][0] * I[2][2] - I[1][2] * I[2][0]),
                     c02 = I[1][0] * I[2][1] - I[1][1] * I[2][0];
        const double c11 = I[0][0] * I[2][2] - I[0][2] * I[2][0], c12 = -(I[0][0] * I[2][1] - I[0][1] * I[2][0]),
                     c22 = I[0][0] * I[1][1] - I[0][1] * I[1][0];
        const double det = I[0][0] * c00 + I[0][1] * c01 + I[0][2] * c02;
        const double Iv[3][3] = {{c00 / det, c01 / det, c02 / det}, {c01 / det, c11 / det, c12 / det},
                                 {c02 / det, c12 / det, c22 / det}};
        const double kd = cd.kdamp;
        double om[3], omb[3], Lb[3];
        for (int r = 0; r < 3; ++r) om[r] = Iv[r][0] * L[0] + Iv[r][1] * L[1] + Iv[r][2] * L[2];
        for (int r = 0; r < 3; ++r) omb[r] = kd * S[3 + r];
        for (int r = 0; r < 3; ++r) Lb[r] = Iv[r][0] * omb[0] + Iv[r][1] * omb[1] + Iv[r][2] * omb[2];
        const double vcm[3] = {t[4] / ms, t[5] / ms, t[6] / ms};
        const double S1[3] = {S[0], S[1], S[2]};
        // sum of dL/dr = kd S1 x w + M vcm x Lbar (the inertia term sums to 0 about the mass centre)
        const double rs[3] = {kd * (S1[1] * om[2] - S1[2] * om[1]) + ms * (vcm[1] * Lb[2] - vcm[2] * Lb[1]),
                              kd * (S1[2] * om[0] - S1[0] * om[2]) + ms * (vcm[2] * Lb[0] - vcm[0] * Lb[2]),
                              kd * (S1[0] * om[1] - S1[1] * om[0]) + ms * (vcm[0] * Lb[1] - vcm[1] * Lb[0])};
        // Ibar = -Lbar w^T; (Ibar + Ibar^T) and its trace
        double Is[3][3];
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) Is[p][q] = -(Lb[p] * om[q] + Lb[q] * om[p]);
        const double tr = -(Lb[0] * om[0] + Lb[1] * om[1] + Lb[2] * om[2]);
        for (int k = 0; k < 3; ++k) {
            sh[k] = (float)om[k];
            sh[3 + k] = (float)Lb[k];
            sh[6 + k] = (float)(kd * S1[k] / ms);  // vcm-bar / M
            sh[9 + k] = (float)(rs[k] / ms);       // sum dL/dr / M
            sh[12 + k] = (float)(t[1 + k] / ms);   // xcm
        }
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) if (q >= p) sh[15 + p * 3 + q - (p * (p + 1)) / 2] = (float)Is[p][q];
        sh[21] = (float)(2.0 * tr);
    }
    __syncthreads();
    const int i = d.vblk_start[blockIdx.x] + threadIdx.x;
    if (i >= cd.v_off + cd.V) return;
    const float3 om = f3(sh[0], sh[1], sh[2]), Lb = f3(sh[3], sh[4], sh[5]);
    const float3 vcmb_M = f3(sh[6], sh[7], sh[8]), rs_M = f3(sh[9], sh[10], sh[11]), xcm = f3(sh[12], sh[13], sh[14]);
    // symmetric (Ibar + Ibar^T): [00 01 02; . 11 12; . . 22]
    const float s00 = sh[15], s01 = sh[16], s02 = sh[17], s11 = sh[18], s12 = sh[19], s22 = sh[20], tr2 = sh[21];
    const float kd = cd.kdamp, kg = cd.kglobal;
    const float m = d.xp[i].w;
    const float3 gvc = xyz(A.u[i]);
    const float3 r = sub(xyz(A.tape_xin[i]), xcm);
    const float3 vb = xyz(A.tape_vb[i]);
    const float3 gvb = add(add(mul(gvc, 1.f - kd), mul(vcmb_M, m)), mul(cross(Lb, r), m));
    const float3 Isr = f3(s00 * r.x + s01 * r.y + s02 * r.z, s01 * r.x + s11 * r.y + s12 * r.z,
                          s02 * r.x + s12 * r.y + s22 * r.z);
    const float3 rbar = add(add(mul(cross(gvc, om), kd), mul(cross(vb, Lb), m)), mul(sub(mul(r, tr2), Isr), m));
    A.gx[i] = f4(sub(rbar, mul(rs_M, m)), 0.f);
    A.gv[i] = f4(mul(gvb, 1.f - kg), 0.f);
}

// float3-packed (3 floats per vertex) <-> float4 gradient buffers.
// The caller's state gradients (3 packed floats per vertex) to and from the
// float4 work copies, all three arrays in one launch.
__global__ void k_adj_unpack(AdjPtrs A, const float *__restrict__ gx, const float *__restrict__ gxp,
                             const float *__restrict__ gv, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    A.gx[i] = make_float4(gx[3 * i], gx[3 * i + 1], gx[3 * i + 2], 0.f);
    A.gxp[i] = make_float4(gxp[3 * i], gxp[3 * i + 1], gxp[3 * i + 2], 0.f);
    A.gv[i] = make_float4(gv[3 * i], gv[3 * i + 1], gv[3 * i + 2], 0.f);
}

__device__ __forceinline__ float put3(float *dst, int i, float4 v) {
    dst[3 * i] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
    return fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fabsf(v.z));
}

// flag (may be null): flag[c] = 1 when a state gradient of cloth c is above
// kRescaleAbove in magnitude after the step.
__global__ void k_adj_pack(DevPtrs d, AdjPtrs A, float *__restrict__ gx, float *__restrict__ gxp,
                           float *__restrict__ gv, uint32_t *__restrict__ flag, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float m = fmaxf(fmaxf(put3(gx, i, A.gx[i]), put3(gxp, i, A.gxp[i])), put3(gv, i, A.gv[i]));
    if (flag && m > kRescaleAbove) flag[d.vcloth[i]] = 1u;
}

// Scales every accumulator of a flagged cloth by kRescaleBy (a power of two,
// so the product is exact while it stays normal), counts the scaling in
// exponent[c] and clears the flags the next call sets.  Threads [0, V) take
// vertices, [V, V+E) stretch and [V+E, V+E+B) bend constraints.
__global__ void k_adj_rescale(DevPtrs d, float *__restrict__ gx, float *__restrict__ gxp, float *__restrict__ gv,
                              float *__restrict__ gks, float *__restrict__ gkb, const uint32_t *__restrict__ flag,
                              uint32_t *__restrict__ flag_next, int32_t *__restrict__ exponent, int E, int B) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int V = d.Vtot;
    if (i < d.C) flag_next[i] = 0u;
    if (i < V) {
        const int c = d.vcloth[i];
        if (!flag[c]) return;
        if (i == d.cloth[c].v_off) exponent[c] += 1;
        for (int k = 0; k < 3; ++k) {
            gx[3 * i + k] *= kRescaleBy; gxp[3 * i + k] *= kRescaleBy; gv[3 * i + k] *= kRescaleBy;
        }
    } else if (i < (int64_t)V + E) {
        const int e = (int)(i - V);
        if (gks && flag[d.vcloth[d.s_ids[e].x]]) gks[e] *= kRescaleBy;
    } else if (i < (int64_t)V + E + B) {
        const int b = (int)(i - V - E);
        if (gkb && flag[d.vcloth[d.b_ids[b].x]]) gkb[b] *= kRescaleBy;
    }
}

// ---------------------------------------------------------------------------
static inline int nb(int64_t n, int b = kThreads) { return (int)((n + b - 1) / b); }

void launch_adj_unpack(const AdjPtrs &A, const float *gx, const float *gxp, const float *gv, int n, cudaStream_t st) {
    if (n) k_adj_unpack<<<nb(n), kThreads, 0, st>>>(A, gx, gxp, gv, n);
}
void launch_adj_pack(const DevPtrs &d, const AdjPtrs &A, float *gx, float *gxp, float *gv, uint32_t *flag, int n,
                     cudaStream_t st) {
    if (n) k_adj_pack<<<nb(n), kThreads, 0, st>>>(d, A, gx, gxp, gv, flag, n);
}
void launch_adj_rescale(const DevPtrs &d, float *gx, float *gxp, float *gv, float *gks, float *gkb,
                        const uint32_t *flag, uint32_t *flag_next, int32_t *exponent, int E, int B, cudaStream_t st) {
    const int64_t n = (int64_t)d.Vtot + E + B;
    if (n) k_adj_rescale<<<nb(n), kThreads, 0, st>>>(d, gx, gxp, gv, gks, gkb, flag, flag_next, exponent, E, B);
}

// The reverse sweep.  a, g: two float4 work buffers of Vtot entries.
void launch_adjoint(const DevPtrs &d, const AdjPtrs &A, float4 *a, float4 *g, const uint32_t *nvf, const uint32_t *nee,
                    int grid, int nfixed, float *gk_stretch, float *gk_bend, cudaStream_t st) {
    if (!d.Vtot) return;
    const bool coll = d.any_collider && d.coll_act;
    const int nbs = nb(A.E, kAdjBlock), nbb = nb(A.B, kAdjBlock);
    k_adj_integrate<<<nb(d.Vtot), kThreads, 0, st>>>(d, A, a);
    for (int it = A.K - 1; it >= 0; --it) {
        if (coll) k_adj_collider<<<nb(d.Vtot), kThreads, 0, st>>>(d, a, it + 1);
        k_adj_u<<<nb(d.Vtot), kThreads, 0, st>>>(d, A, a, it);
        k_adj_constraints<<<nbs + nbb + grid, kAdjBlock, 0, st>>>(d, A, it, gk_stretch, gk_bend, nvf, nee, nbs, nbb);
        k_adj_gather<<<d.nvblk, kThreads, 0, st>>>(d, A, a, g, it);
        if (nfixed) k_adj_fixed_add<<<nb(nfixed), kThreads, 0, st>>>(d, A, g, nfixed);
        float4 *t = a; a = g; g = t;
    }
    if (coll) k_adj_collider<<<nb(d.Vtot), kThreads, 0, st>>>(d, a, 0);
    k_adj_damp1<<<d.nvblk, kThreads, 0, st>>>(d, A, a);
    k_adj_totals<<<d.C, 32, 0, st>>>(d, A);
    k_adj_damp2<<<d.nvblk, kThreads, 0, st>>>(d, A);
}

}  // namespace lc
