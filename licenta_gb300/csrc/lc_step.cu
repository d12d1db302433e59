// lc_step.cu — PBD half of the cloth step: wind, external forces, rigid-mode
// damping and prediction (CudaPBD::PBDStepExternal), running vertex normals,
// the per-step dynamic-contact CSR, solver set-up (ground / LRA / sphere), the
// Jacobi iteration and integration (CudaPBD::PBDStepSolver /
// PBDStepIntegration, DeformableUtils::WorldConstraints).
#include "lc_internal.cuh"
#include "lc_pbd.cuh"

namespace lc {

// ---------------------------------------------------------------------------
// Host wind update of Physics/CudaPBD.cu:613-619, moved on the device so a
// captured step needs no host input.  The std::rand() draw is replaced by a
// seeded xorshift (same generator as the oracle).
// ---------------------------------------------------------------------------
__global__ void k_wind(DevPtrs d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.C) return;
    const ClothDev &cd = d.cloth[c];
    if (!cd.wind_on) return;
    ClothState st = d.cstate[c];
    const unsigned long long bit = (st.rng ^ (st.rng >> 29)) & 1ull;
    const double u = xs_uniform(st.rng);
    const double var = (double)cd.wind_var_min + u * ((double)cd.wind_var_max - (double)cd.wind_var_min);
    const float variation = (bit ? 1.f : -1.f) * (float)var;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float w = __fadd_rn(st.wind[k], __fmul_rn(cd.wind_start[k], variation));
        st.wind[k] = clampf(w, cd.wind_min[k], cd.wind_max[k]);
    }
    d.cstate[c] = st;
}

// Block-wide sums of N floats written as this block's partials (blocks never
// straddle cloths); warp sums in float, cross-warp sums in double, in a fixed
// order, so every run produces the same bits.
template <int N>
__device__ __forceinline__ void block_partials(float (&v)[N], double *dst) {
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

// Cloth totals of the block partials [k0, k0+N), one block per cloth, summed
// in a fixed order (deterministic) into d.damp[c*16 + k].
__global__ void k_cloth_totals(DevPtrs d, int k0, int N) {
    const int c = blockIdx.x;
    const int b0 = d.vb_first[c], b1 = d.vb_first[c + 1];
    __shared__ double red[16][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = 0; k < N; ++k) {
        double s = 0;
        for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) s += d.damp_part[(size_t)b * 16 + k0 + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[threadIdx.x][w];
        d.damp[(size_t)c * 16 + k0 + threadIdx.x] = t;
    }
}

// ApplyExternalForces (Physics/CudaPBD.cu:1992-2003), GlobalVelDamp (:1934-1941)
// and the mass / first-moment sums of DampVelocities (:419-435).
__global__ void k_external(DevPtrs d) {
    const int c = d.vblk_cloth[blockIdx.x];
    const ClothDev &cd = d.cloth[c];
    const int i = d.vblk_start[blockIdx.x] + threadIdx.x;
    const bool valid = i < cd.v_off + cd.V;
    float s[7] = {0, 0, 0, 0, 0, 0, 0};
    if (valid) {
        float3 vel = xyz(d.v[i]);
        const float dt = cd.dt;
        const float3 g = f3(cd.g[0], cd.g[1], cd.g[2]);
        const ClothState st = d.cstate[c];
        const float3 wind = f3(st.wind[0], st.wind[1], st.wind[2]);
        if (is_zero(wind)) {
            vel = add(vel, mul(g, dt));
        } else {
            const float3 n = xyz(d.vn[i]);
            vel = add(vel, mul(add(g, mul(mul(n, dot(normalize(wind), n)), len(wind))), dt));
        }
        vel = mul(vel, 1.f - cd.kglobal);
        d.v[i] = f4(vel, 0.f);
        const float m = d.xp[i].w;
        const float3 p = xyz(d.x[i]);
        s[0] = m;
        s[1] = p.x * m; s[2] = p.y * m; s[3] = p.z * m;
        s[4] = vel.x * m; s[5] = vel.y * m; s[6] = vel.z * m;
    }
    block_partials<7>(s, d.damp_part + (size_t)blockIdx.x * 16);
}

// ComputeL / ComputeIs (Physics/CudaPBD.cu:1955-1976): angular momentum and
// inertia about the mass centre.
__global__ void k_damp_moments(DevPtrs d) {
    const int c = d.vblk_cloth[blockIdx.x];
    const ClothDev &cd = d.cloth[c];
    const double *t = d.damp + (size_t)c * 16;
    const int i = d.vblk_start[blockIdx.x] + threadIdx.x;
    const bool valid = i < cd.v_off + cd.V;
    // the mass centre once per block: FP64 division is slow on this part
    __shared__ float cm[3];
    if (threadIdx.x < 3) cm[threadIdx.x] = (float)(t[1 + threadIdx.x] / t[0]);
    __syncthreads();
    float s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (valid) {
        const float3 xcm = f3(cm[0], cm[1], cm[2]);
        const float m = d.xp[i].w;
        const float3 r = sub(xyz(d.x[i]), xcm);
        const float3 l = cross(r, mul(xyz(d.v[i]), m));
        s[0] = l.x; s[1] = l.y; s[2] = l.z;
        s[3] = r.x * r.x * m; s[4] = r.y * r.y * m; s[5] = r.z * r.z * m;
        s[6] = -(r.x * r.y) * m; s[7] = -(r.x * r.z) * m; s[8] = -(r.y * r.z) * m;
    }
    block_partials<9>(s, d.damp_part + (size_t)blockIdx.x * 16 + 7);
}

// omega = I^-1 L (the host glm::inverse of Physics/CudaPBD.cu:447-454, here in
// double on the device), UpdateVels (:1978-1990) and ExplicitEuler (:2005-2012).
__global__ void k_damp_apply(DevPtrs d) {
    const int c = d.vblk_cloth[blockIdx.x];
    const ClothDev &cd = d.cloth[c];
    const double *a = d.damp + (size_t)c * 16;
    __shared__ float sh[9];
    if (threadIdx.x == 0) {
        const double ms = a[0];
        const double L0 = a[7], L1 = a[8], L2 = a[9];
        const double i1x = a[10], i1y = a[11], i1z = a[12], i2x = a[13], i2y = a[14], i2z = a[15];
        const double A = i1y + i1z, B = i2x, C = i2y, D = i1x + i1z, E = i2z, F = i1x + i1y;
        // symmetric [[A,B,C],[B,D,E],[C,E,F]]
        const double c00 = D * F - E * E, c01 = -(B * F - E * C), c02 = B * E - D * C;
        const double c11 = A * F - C * C, c12 = -(A * E - B * C), c22 = A * D - B * B;
        const double det = A * c00 + B * c01 + C * c02;
        sh[0] = (float)((c00 * L0 + c01 * L1 + c02 * L2) / det);
        sh[1] = (float)((c01 * L0 + c11 * L1 + c12 * L2) / det);
        sh[2] = (float)((c02 * L0 + c12 * L1 + c22 * L2) / det);
        sh[3] = (float)(a[1] / ms); sh[4] = (float)(a[2] / ms); sh[5] = (float)(a[3] / ms);
        sh[6] = (float)(a[4] / ms); sh[7] = (float)(a[5] / ms); sh[8] = (float)(a[6] / ms);
    }
    __syncthreads();
    const int i = d.vblk_start[blockIdx.x] + threadIdx.x;
    if (i >= cd.v_off + cd.V) return;
    const float3 omega = f3(sh[0], sh[1], sh[2]);
    const float3 xcm = f3(sh[3], sh[4], sh[5]);
    const float3 vcm = f3(sh[6], sh[7], sh[8]);
    const float4 x4 = d.x[i];
    const float3 r = sub(xyz(x4), xcm);
    float3 vel = xyz(d.v[i]);
    const float3 dv = sub(add(vcm, cross(omega, r)), vel);
    vel = add(vel, mul(dv, cd.kdamp));
    d.v[i] = f4(vel, 0.f);
    // ExplicitEuler (Physics/CudaPBD.cu:2005-2012), rounded after the product
    // and after the sum as the restatement does (no fused multiply-add), so
    // the predicted positions the collision stages see are reproducible.
    const float4 p = d.xp[i];
    const float dt = cd.dt;
    const float4 xn = make_float4(__fadd_rn(p.x, __fmul_rn(vel.x, dt)), __fadd_rn(p.y, __fmul_rn(vel.y, dt)),
                                  __fadd_rn(p.z, __fmul_rn(vel.z, dt)), x4.w);
    d.x[i] = xn;
    if (d.vbox) {  // the narrowphase's vertex boxes, once per vertex instead of once per pair
        d.vbox[2 * (size_t)i] = f4(subc(vmin(xyz(xn), xyz(p)), cd.h), 0.f);
        d.vbox[2 * (size_t)i + 1] = f4(addc(vmax(xyz(xn), xyz(p)), cd.h), 0.f);
    }
}

// UpdateVertexNormals (Physics/CudaDeformableUtils.cu:190-249) as a gather
// over each vertex's triangles: the running sum is kept (not zeroed) and
// renormalised, as in the reference, every step for every cloth (the wind
// term reads them and the vertex records publish them).
__global__ void k_vertex_normals(DevPtrs d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    float3 a = xyz(d.vn[i]);
    for (int k = d.vt_off[i]; k < d.vt_off[i + 1]; ++k) a = add(a, xyz(d.fn[d.vt_idx[k]]));
    d.vn[i] = f4(normalize(a), 0.f);
}

// ---------------------------------------------------------------------------
// Dynamic-contact CSR: every contact contributes 4 entries (contact*4+slot,
// VF contacts first) to its vertices; each vertex list is sorted, giving the
// order of the reference's stable sort + RLE (Physics/CudaPBD.cu:702-721).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void contact_counts(const DevPtrs &d, const uint32_t *nvf_dev, const uint32_t *nee_dev,
                                               uint32_t &nvf, uint32_t &nee) {
    nvf = min((uint64_t)*nvf_dev, d.vf_cap);
    nee = min((uint64_t)*nee_dev, d.ee_cap);
}

__global__ void k_dyn_count(DevPtrs d, const uint32_t *nvf_dev, const uint32_t *nee_dev) {
    uint32_t nvf, nee;
    contact_counts(d, nvf_dev, nee_dev, nvf, nee);
    const uint32_t n = nvf + nee;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int4 v = c < nvf ? d.vf_v[c] : d.ee_v[c - nvf];
        atomicAdd(&d.dyn_cnt[v.x], 1u);
        atomicAdd(&d.dyn_cnt[v.y], 1u);
        atomicAdd(&d.dyn_cnt[v.z], 1u);
        atomicAdd(&d.dyn_cnt[v.w], 1u);
    }
}

__global__ void k_dyn_fill(DevPtrs d, const uint32_t *nvf_dev, const uint32_t *nee_dev) {
    uint32_t nvf, nee;
    contact_counts(d, nvf_dev, nee_dev, nvf, nee);
    const uint32_t n = nvf + nee;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int4 v = c < nvf ? d.vf_v[c] : d.ee_v[c - nvf];
        const int vs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t pos = d.dyn_off[vs[s]] + atomicAdd(&d.dyn_cur[vs[s]], 1u);
            d.dyn_ent[pos] = c * 4u + (uint32_t)s;
        }
    }
}

__global__ void k_dyn_sort(DevPtrs d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const uint32_t a = d.dyn_off[i], b = d.dyn_off[i + 1];
    for (uint32_t k = a + 1; k < b; ++k) {
        const uint32_t key = d.dyn_ent[k];
        uint32_t j = k;
        while (j > a && d.dyn_ent[j - 1] > key) {
            d.dyn_ent[j] = d.dyn_ent[j - 1];
            --j;
        }
        d.dyn_ent[j] = key;
    }
}

// ---------------------------------------------------------------------------
// Solver set-up, once per step: ground (Physics/CudaPBD.cu:1477-1507) and LRA
// (:1571-1592) flags from the predicted positions.
// ---------------------------------------------------------------------------
__global__ void k_solver_setup(DevPtrs d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const int c = d.vcloth[i];
    const ClothDev &cd = d.cloth[c];
    const float4 x4 = d.x[i];
    const float3 pos = xyz(x4);
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    if (cd.ground_on && pos.y <= cd.ground_y + cd.h) {
        const float3 nc = f3(0.f, 1.f, 0.f);
        const float3 p0 = f3(1.f, cd.ground_y + cd.h, 1.f);
        const float3 l = sub(pos, xyz(d.xp[i]));
        const float dd = dot(sub(p0, pos), nc) / dot(l, nc);
        q = f4(add(mul(l, dd), pos), 1.f);
    }
    d.ground_qc[i] = q;
    if (cd.F) {
        const int local = i - cd.v_off;
        const bool pinned = x4.w == 0.f;
        for (int j = 0; j < cd.F; ++j) {
            const int64_t k = cd.lra_off + (int64_t)local * cd.F + j;
            uint8_t f = 0;
            if (!pinned && dist(pos, xyz(d.x[d.fixed[cd.f_off + j]])) > d.lra_l0[k]) f = 1;
            d.lra_flag[k] = f;
        }
    }
}

// Ray-sphere of Collision/CudaCollisionDetection.cu:529-567.
__device__ int ray_sphere(float3 p1, float3 p2, float3 c0, float rad, float3 &q) {
    float3 dir = sub(p2, p1);
    if (is_zero(dir)) return 0;
    const float l = len(dir);
    dir = dvs(dir, l);
    const float3 m = sub(p1, c0);
    const float b = dot(m, dir);
    const float c = dot(m, m) - rad * rad;
    if (c > 0.f && b > 0.f) return 0;
    const float disc = b * b - c;
    if (disc < 0.f) return 0;
    const float t = -b - sqrtf(disc);
    if (t < 0.f) { q = add(p1, mul(dir, t)); return -1; }
    if (t > l) return 0;
    q = add(p1, mul(dir, t));
    return 1;
}

// _CreateSphereConstraints (Physics/CudaPBD.cu:1509-1569): projects x / x_prev
// directly; its constraint flags are never set, so no iteration term follows.
__global__ void k_sphere(DevPtrs d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const ClothDev &cd = d.cloth[d.vcloth[i]];
    if (!cd.sphere_on) return;
    const float4 x4 = d.x[i], p4 = d.xp[i];
    const float3 sc = f3(cd.sphere_pos[0], cd.sphere_pos[1], cd.sphere_pos[2]);
    const float rad = cd.sphere_r + cd.h;
    float3 q;
    const int ret = ray_sphere(xyz(p4), xyz(x4), sc, rad, q);
    if (d.dbg_sphere) d.dbg_sphere[i] = (int8_t)ret;
    if (ret == -1) {
        const float3 qs = add(sc, mul(normalize(sub(q, sc)), rad));
        const float3 ns = normalize(sub(qs, sc));
        d.xp[i] = f4(add(qs, mul(ns, 0.0001f)), p4.w);
        d.x[i] = f4(qs, x4.w);
    } else if (ret == 1) {
        const float3 ns = normalize(sub(q, sc));
        d.x[i] = f4(add(q, mul(ns, 0.0001f)), x4.w);
    }
}

// ---------------------------------------------------------------------------
// Jacobi iteration (Physics/CudaPBD.cu:648-659) as a per-vertex gather:
// every vertex evaluates the constraints it belongs to on the positions of
// the previous iteration (xa) and writes its own update to xb.  The sum is
// associated like the reference's accumulator: ((ground + LRA) + static) +
// dynamic, then x += acc / count.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float3 stretch_corr(const DevPtrs &d, const float4 *__restrict__ xa, uint32_t k,
                                               int role) {
    const int2 id = __ldg(&d.s_ids[k]);
    const float2 par = __ldg(&d.s_par[k]);
    return stretch_corr_pos(xa[id.x], xa[id.y], par.x, par.y, role);
}

__device__ __forceinline__ float3 tri_bend_corr(const DevPtrs &d, const float4 *__restrict__ xa, uint32_t k,
                                                int role) {
    const int4 id = __ldg(&d.b_ids[k]);
    return tri_bend_corr_pos(xa[id.x], xa[id.y], xa[id.z], __ldg(&d.b_kp[k]), __int_as_float(id.w), role);
}

__device__ __forceinline__ float3 bend_corr(const DevPtrs &d, const float4 *__restrict__ xa, uint32_t k, int role) {
    const int4 id = __ldg(&d.b_ids[k]);
    return bend_corr_pos(xa[id.x], xa[id.y], xa[id.z], xa[id.w], __ldg(&d.b_kp[k]), d.kpi_gap, role);
}

__device__ __forceinline__ float3 contact_corr(const DevPtrs &d, const float4 *__restrict__ xa, uint32_t e,
                                               uint32_t nvf, float h) {
    const uint32_t c = e >> 2;
    const int slot = (int)(e & 3u);
    const bool isvf = c < nvf;
    const int4 v = isvf ? d.vf_v[c] : d.ee_v[c - nvf];
    const float4 w = isvf ? d.vf_w[c] : d.ee_w[c - nvf];
    return contact_corr_pos(xa[v.x], xa[v.y], xa[v.z], xa[v.w], w, isvf, h, slot);
}

__global__ void k_jacobi(DevPtrs d, const float4 *__restrict__ xa, float4 *__restrict__ xb, int it,
                         const uint32_t *__restrict__ nvf_dev) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const int c = d.vcloth[i];
    const ClothDev &cd = d.cloth[c];
    const float4 xi4 = xa[i];
    if (it >= cd.iters) {
        xb[i] = xi4;
        if (d.coll_act) d.coll_act[(size_t)(it + 1) * d.Vtot + i] = 0;
        return;
    }
    const float3 xi = xyz(xi4);
    float3 acc = f3(0.f, 0.f, 0.f);
    int cnt = 0;
    // ground, Physics/CudaPBD.cu:1594-1629
    const float4 q = d.ground_qc[i];
    bool ground_counted = false;
    if (q.w != 0.f) {
        const float3 nc = f3(0.f, 1.f, 0.f);
        const float cv = dot(sub(xi, xyz(q)), nc);
        if (cv < 0.f) { acc = add(acc, mul(nc, -cv)); cnt += 1; ground_counted = true; }
    }
    if (d.dbg_ground_it) {
        const uint32_t bit = ground_counted ? (1u << it) : 0u;
        d.dbg_ground_it[i] = it == 0 ? bit : (d.dbg_ground_it[i] | bit);
    }
    // LRA, Physics/CudaPBD.cu:1656-1688
    if (cd.F) {
        float3 la = f3(0.f, 0.f, 0.f);
        int lc = 0;
        const int64_t base = cd.lra_off + (int64_t)(i - cd.v_off) * cd.F;
        for (int j = 0; j < cd.F; ++j) {
            if (d.lra_flag[base + j]) {
                const float3 diff = sub(xi, xyz(xa[d.fixed[cd.f_off + j]]));
                const float l = len(diff);
                const float3 n = dvs(diff, l);
                la = add(la, mul(n, -(l - d.lra_l0[base + j])));
                ++lc;
            }
        }
        acc = add(acc, la);
        cnt += lc;
    }
    // static stretch + bend, Physics/CudaPBD.cu:942-1147, 1417-1446
    {
        float3 sa = f3(0.f, 0.f, 0.f);
        const int s0 = d.soff[i], s1 = d.soff[i + 1];
        for (int e = s0; e < s1; ++e) {
            const uint32_t ent = __ldg(&d.sent[e]);
            const uint32_t k = ent & 0x1FFFFFFFu;
            const int role = (int)((ent >> 29) & 3u);
            sa = add(sa, (ent >> 31) ? (cd.tri_bend ? tri_bend_corr(d, xa, k, role) : bend_corr(d, xa, k, role))
                                     : stretch_corr(d, xa, k, role));
        }
        acc = add(acc, sa);
        cnt += s1 - s0;
    }
    // dynamic VF / EE, Physics/CudaPBD.cu:1190-1415, 1448-1475
    {
        const uint32_t e0 = d.dyn_off[i], e1 = d.dyn_off[i + 1];
        if (e1 > e0) {
            const uint32_t nvf = (uint32_t)min((uint64_t)*nvf_dev, d.vf_cap);
            float3 da = f3(0.f, 0.f, 0.f);
            int dc = 0;
            for (uint32_t e = e0; e < e1; ++e) {
                const uint32_t ent = d.dyn_ent[e];
                const float3 corr = contact_corr(d, xa, ent, nvf, cd.h);
                const bool nz = !is_zero(corr);
                if (nz) { da = add(da, corr); ++dc; }
                if (d.dbg_dyn_nz) d.dbg_dyn_nz[(size_t)it * d.dyn_cap + ent] = nz ? 1 : 0;
            }
            acc = add(acc, da);
            cnt += dc;
        }
    }
    // FinalCorrectionStep, Physics/CudaPBD.cu:1690-1698 (no zero-count guard)
    float3 xn = add(xi, dvs(acc, (float)cnt));
    if (d.any_collider) {
        uint8_t *act = d.coll_act ? d.coll_act + (size_t)(it + 1) * d.Vtot + i : nullptr;
        if (xi4.w != 0.f) xn = collider_project(d, i, xn, cd.h, act);
        else if (act) *act = 0;
    }
    xb[i] = f4(xn, xi4.w);
}

// _FinalUpdate (Physics/CudaPBD.cu:1916-1932) then _WorldConstraints
// (Physics/CudaDeformableUtils.cu:260-269).  xs holds the solver output.
__global__ void k_integrate(DevPtrs d, const float4 *__restrict__ xs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const ClothDev &cd = d.cloth[d.vcloth[i]];
    const float4 x4 = xs[i];
    float3 p = xyz(x4);
    if (x4.w == 0.f) {
        d.v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        const float4 p4 = d.xp[i];
        d.v[i] = f4(dvs(sub(p, xyz(p4)), cd.dt), 0.f);
        d.xp[i] = f4(p, p4.w);
    }
    p = f3(fminf(fmaxf(p.x, cd.wmin[0]), cd.wmax[0]), fminf(fmaxf(p.y, cd.wmin[1]), cd.wmax[1]),
           fminf(fmaxf(p.z, cd.wmin[2]), cd.wmax[2]));
    d.x[i] = f4(p, x4.w);
}

// ---------------------------------------------------------------------------
static inline int nblk(int64_t n, int b = kThreads) { return (int)((n + b - 1) / b); }

void launch_wind(const DevPtrs &d, cudaStream_t st) { k_wind<<<nblk(d.C, 128), 128, 0, st>>>(d); }
// save_x / save_v (may be null): copies of the damping inputs (state x and the
// velocity after the global damping) for the reverse pass.
void launch_external(const DevPtrs &d, cudaStream_t st, float4 *save_x, float4 *save_v) {
    if (d.nvblk) {
        k_external<<<d.nvblk, kThreads, 0, st>>>(d);
        k_cloth_totals<<<d.C, kThreads, 0, st>>>(d, 0, 7);
        k_damp_moments<<<d.nvblk, kThreads, 0, st>>>(d);
        k_cloth_totals<<<d.C, kThreads, 0, st>>>(d, 7, 9);
        if (save_x) cudaMemcpyAsync(save_x, d.x, sizeof(float4) * (size_t)d.Vtot, cudaMemcpyDeviceToDevice, st);
        if (save_v) cudaMemcpyAsync(save_v, d.v, sizeof(float4) * (size_t)d.Vtot, cudaMemcpyDeviceToDevice, st);
        k_damp_apply<<<d.nvblk, kThreads, 0, st>>>(d);
    }
}
void launch_vertex_normals(const DevPtrs &d, cudaStream_t st) {
    if (d.Vtot) k_vertex_normals<<<nblk(d.Vtot), kThreads, 0, st>>>(d);
}
void launch_dyn(const DevPtrs &d, const uint32_t *nvf, const uint32_t *nee, int grid, int phase, cudaStream_t st) {
    if (phase == 0) k_dyn_count<<<grid, kThreads, 0, st>>>(d, nvf, nee);
    else if (phase == 1) k_dyn_fill<<<grid, kThreads, 0, st>>>(d, nvf, nee);
    else if (d.Vtot) k_dyn_sort<<<nblk(d.Vtot), kThreads, 0, st>>>(d);
}
void launch_solver_setup(const DevPtrs &d, bool sphere, cudaStream_t st) {
    if (!d.Vtot) return;
    k_solver_setup<<<nblk(d.Vtot), kThreads, 0, st>>>(d);
    if (sphere) k_sphere<<<nblk(d.Vtot), kThreads, 0, st>>>(d);
}
void launch_jacobi(const DevPtrs &d, const float4 *xa, float4 *xb, int it, const uint32_t *nvf, int block,
                   cudaStream_t st) {
    if (d.Vtot) k_jacobi<<<nblk(d.Vtot, block), block, 0, st>>>(d, xa, xb, it, nvf);
}
void launch_integrate(const DevPtrs &d, const float4 *xs, cudaStream_t st) {
    if (d.Vtot) k_integrate<<<nblk(d.Vtot), kThreads, 0, st>>>(d, xs);
}

// CudaPBD::ApplyFriction (Physics/CudaPBD.cu:770-833) for the cloths with
// useFriction, after the integration; velocities only.  Per vertex:
//  * _DampVelRigid (:1879-1912): the reference launches it with 255 threads
//    per block over ceil(V/256) blocks (:777), so it reaches only the first
//    255*ceil(V/256) vertices of a cloth; those with a ground constraint this
//    step have their normal velocity scaled by 1 - kFriction and the sum
//    reflected about the ground normal (0, 1, 0).
//  * _ApplyFrictionVF / _AccumulateFriction (:1745-1794, :1846-1877): the
//    face normals of the vertex's VF contacts summed in contact order (the
//    per-vertex contact lists are sorted by entry, as the reference's stable
//    key sort leaves them).  _ApplyFrictionEE (:1796-1845) never writes its
//    entries' vertex ids, so EE entries take no part (what the reference
//    computes for a step without EE contacts).
//  * FinalFrictionStep (:1700-1723): with a non-zero sum, the normal velocity
//    along the summed direction is scaled by (1 - kFriction)^count and the
//    sum reflected about it.
__global__ void k_friction(DevPtrs d, const uint32_t *__restrict__ nvf_dev) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const ClothDev &cd = d.cloth[d.vcloth[i]];
    if (!cd.friction) return;
    const float kf = cd.kfriction;
    float3 v = xyz(d.v[i]);
    const int li = i - cd.v_off;
    const int reach = (cd.V + 255) / 256 * 255;
    if (li < reach && d.ground_qc[i].w != 0.f) {
        const float3 n = f3(0.f, 1.f, 0.f);
        float3 vn = mul(n, dot(v, n));
        const float3 vt = sub(v, vn);
        vn = mul(vn, 1.f - kf);
        const float3 r = add(vt, vn);
        v = sub(r, mul(n, 2.f * dot(r, n)));
    }
    const uint32_t nvf4 = 4u * (uint32_t)min((uint64_t)*nvf_dev, d.vf_cap);
    float3 acc = f3(0.f, 0.f, 0.f);
    int cnt = 0;
    for (uint32_t e = d.dyn_off[i]; e < d.dyn_off[i + 1]; ++e) {
        const uint32_t ent = d.dyn_ent[e];
        if (ent >= nvf4) continue;
        acc = add(acc, xyz(d.vf_n[ent >> 2]));
        ++cnt;
    }
    if (cnt != 0 && !is_zero(acc)) {
        const float3 fn = normalize(acc);
        float3 vn = mul(fn, dot(v, fn));
        const float3 vt = sub(v, vn);
        vn = mul(vn, powf(1.f - kf, (float)cnt));
        const float3 r = add(vn, vt);
        v = sub(r, mul(fn, 2.f * dot(r, fn)));
    }
    d.v[i] = f4(v, d.v[i].w);
}

// Physics/CudaDeformableUtils.cu:327-344: position (x_prev) and running
// normal into interleaved records; nothing else of a record is touched.
__global__ void k_vertex_records(DevPtrs d, unsigned char *__restrict__ dst, int64_t stride, int pos_off,
                                 int nrm_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.Vtot) return;
    const float4 p = d.xp[i], n = d.vn[i];
    float *pp = reinterpret_cast<float *>(dst + (int64_t)i * stride + pos_off);
    float *pn = reinterpret_cast<float *>(dst + (int64_t)i * stride + nrm_off);
    pp[0] = p.x; pp[1] = p.y; pp[2] = p.z;
    pn[0] = n.x; pn[1] = n.y; pn[2] = n.z;
}

void launch_vertex_records(const DevPtrs &d, void *dst, int64_t stride, int pos_off, int nrm_off, cudaStream_t st) {
    if (d.Vtot)
        k_vertex_records<<<nblk(d.Vtot), kThreads, 0, st>>>(d, static_cast<unsigned char *>(dst), stride, pos_off,
                                                            nrm_off);
}

// Packed xyz (12 B per vertex, the caller's layout) to and from the float4
// state arrays; the w lane (mass or inverse mass) is left as it is.
__global__ void k_xyz_unpack(const float *__restrict__ src, float4 *__restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 o = dst[i];
    dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], o.w);
}
__global__ void k_xyz_pack(const float4 *__restrict__ src, float *__restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = src[i];
    dst[3 * i] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
}

void launch_xyz_unpack(const float *src, float4 *dst, int n, cudaStream_t st) {
    if (n > 0) k_xyz_unpack<<<nblk(n), kThreads, 0, st>>>(src, dst, n);
}
void launch_xyz_pack(const float4 *src, float *dst, int n, cudaStream_t st) {
    if (n > 0) k_xyz_pack<<<nblk(n), kThreads, 0, st>>>(src, dst, n);
}

void launch_friction(const DevPtrs &d, const uint32_t *nvf, cudaStream_t st) {
    if (d.Vtot) k_friction<<<nblk(d.Vtot), kThreads, 0, st>>>(d, nvf);
}

}  // namespace lc
