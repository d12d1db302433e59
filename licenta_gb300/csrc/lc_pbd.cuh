// lc_pbd.cuh — correction of one constraint slot for the vertex in that
// slot, from the positions (float4, w = inverse mass) of the constraint's
// vertices.  Shared by the global-memory Jacobi kernel (lc_step.cu) and the
// cluster-resident one (lc_cluster.cu), so both evaluate the same expressions.
#pragma once

#include "lc_internal.cuh"

namespace lc {

// Physics/CudaPBD.cu:986-1022 — stretch (distance) constraint.
__device__ __forceinline__ float3 stretch_corr_pos(float4 a, float4 b, float l0, float kp, int role) {
    const float w1 = a.w, w2 = b.w;
    const float ws = w1 + w2;
    if (ws == 0.f) return f3(0.f, 0.f, 0.f);
    const float3 diff = sub(xyz(a), xyz(b));
    const float l = len(diff);
    if (l <= kEpsPbd) return f3(0.f, 0.f, 0.f);
    const float3 n = dvs(diff, l);
    const float3 tt = dvs(mul(mul(n, l - l0), kp), ws);
    return role == 0 ? mul(tt, -w1) : mul(tt, w2);
}

// Physics/CudaPBD.cu:1024-1147 — bend constraint on the planes (0, p2, p3) and
// (0, p2, p4) of the raw positions, rest angle PI.  The reference's
// expressions cancel catastrophically near d = dot(n1, n2) = -1, which is
// where this constraint drives the cloth, so they are evaluated in an
// algebraically identical form that stays accurate in float:
//   1 + d = |n1 + n2|^2 / 2,  1 - d = |n1 - n2|^2 / 2,
//   acos(d) - PI = -2 atan2(|n1 + n2|, |n1 - n2|) (+ the gap between PI and
//   the float constant of the reference), and n2 - d n1 = s - (1 + d) n1 with
//   s = n1 + n2, so q3 = p2 x u / l23, q4 = p2 x w / l24,
//   q2 = -(p3 x u / l23 + p4 x w / l24), u = s - (1+d) n1, w = s - (1+d) n2.
__device__ __forceinline__ float3 bend_corr_pos(float4 a1, float4 a2, float4 a3, float4 a4, float kp, float kpi_gap,
                                                int role) {
    const float3 p2 = xyz(a2), p3 = xyz(a3), p4 = xyz(a4);
    const float3 c23 = cross(p2, p3), c24 = cross(p2, p4);
    const float l23 = len(c23), l24 = len(c24);
    if (l23 <= kEpsPbd || l24 <= kEpsPbd) return f3(0.f, 0.f, 0.f);
    const float3 n1 = dvs(c23, l23), n2 = dvs(c24, l24);
    const float3 sv = add(n1, n2), tv = sub(n1, n2);
    const float ss = dot(sv, sv), tt = dot(tv, tv);
    if (ss == 0.f) return f3(0.f, 0.f, 0.f);  // d == -1: phi == phi0
    const float opd = 0.5f * ss;              // 1 + d
    const float omd = 0.5f * tt;              // 1 - d
    const float dphi = kpi_gap - 2.f * atan2f(sqrtf(ss), sqrtf(tt));  // acos(d) - PI
    const float term = sqrtf(opd * omd) * dphi * kp;
    const float3 u = sub(sv, mul(n1, opd)), w = sub(sv, mul(n2, opd));
    const float3 q3 = dvs(cross(p2, u), l23);
    const float3 q4 = dvs(cross(p2, w), l24);
    const float3 q2 = neg(add(dvs(cross(p3, u), l23), dvs(cross(p4, w), l24)));
    const float3 q1 = sub(sub(neg(q2), q3), q4);
    const float sf = a1.w * dot(q1, q1) + a2.w * dot(q2, q2) + a3.w * dot(q3, q3) + a4.w * dot(q4, q4);
    if (sf <= kEpsPbd) return f3(0.f, 0.f, 0.f);
    const float ts = term / sf;
    const float wr = role == 0 ? a1.w : role == 1 ? a2.w : role == 2 ? a3.w : a4.w;
    const float3 q = role == 0 ? q1 : role == 1 ? q2 : role == 2 ? q3 : q4;
    return mul(q, -(wr * ts));
}

// Physics/CudaPBD.cu:1149-1187 — triangle bending (useTriangleBending): the
// middle vertex v of three collinear grid vertices (b0, v, b1) is kept at the
// rest distance h0 from their centroid.  Slot roles: 0 = b0, 1 = b1, 2 = v.
__device__ __forceinline__ float3 tri_bend_corr_pos(float4 b0, float4 b1, float4 v, float kp, float h0, int role) {
    const float W = b0.w + b1.w + 2.f * v.w;
    const float3 c = dvs(add(add(xyz(b0), xyz(b1)), xyz(v)), 3.f);
    const float3 hv = sub(xyz(v), c);
    const float l = len(hv);
    if (l <= kEpsPbd) return f3(0.f, 0.f, 0.f);
    const float3 term = mul(mul(dvs(hv, W), kp), 1.f - h0 / l);
    return role == 0 ? mul(term, 2.f * b0.w) : role == 1 ? mul(term, 2.f * b1.w) : mul(term, -4.f * v.w);
}

// The same bend constraint evaluated once for all four vertices: q[j] and the
// scale s such that vertex j's correction is -(w_j s) q[j].  Returns false
// when the reference returns zero corrections.
__device__ __forceinline__ bool bend_all_pos(float4 a1, float4 a2, float4 a3, float4 a4, float kp, float kpi_gap,
                                             float3 q[4], float &s) {
    const float3 p2 = xyz(a2), p3 = xyz(a3), p4 = xyz(a4);
    const float3 c23 = cross(p2, p3), c24 = cross(p2, p4);
    const float l23 = len(c23), l24 = len(c24);
    if (l23 <= kEpsPbd || l24 <= kEpsPbd) return false;
    const float3 n1 = dvs(c23, l23), n2 = dvs(c24, l24);
    const float3 sv = add(n1, n2), tv = sub(n1, n2);
    const float ss = dot(sv, sv), tt = dot(tv, tv);
    if (ss == 0.f) return false;
    const float opd = 0.5f * ss, omd = 0.5f * tt;
    const float dphi = kpi_gap - 2.f * atan2f(sqrtf(ss), sqrtf(tt));
    const float term = sqrtf(opd * omd) * dphi * kp;
    const float3 u = sub(sv, mul(n1, opd)), w = sub(sv, mul(n2, opd));
    q[2] = dvs(cross(p2, u), l23);
    q[3] = dvs(cross(p2, w), l24);
    q[1] = neg(add(dvs(cross(p3, u), l23), dvs(cross(p4, w), l24)));
    q[0] = sub(sub(neg(q[1]), q[2]), q[3]);
    const float sf = a1.w * dot(q[0], q[0]) + a2.w * dot(q[1], q[1]) + a3.w * dot(q[2], q[2]) + a4.w * dot(q[3], q[3]);
    if (sf <= kEpsPbd) return false;
    s = term / sf;
    return true;
}

// Physics/CudaPBD.cu:1212-1415 — slot `slot` of a VF contact (vertex A, face
// B C D, weights w = (1, -b0, -b1, -b2)) or an EE contact (edges A B and C D,
// weights w = (b0, b1, -b2, -b3)).
__device__ __forceinline__ float3 contact_corr_pos(float4 A, float4 B, float4 C, float4 D, float4 w, bool isvf,
                                                   float h, int slot) {
    if (isvf) {
        const float b0 = clampf(-w.y, 0.f, 1.f), b1 = clampf(-w.z, 0.f, 1.f), b2 = clampf(-w.w, 0.f, 1.f);
        const float3 q = add(add(mul(xyz(B), b0), mul(xyz(C), b1)), mul(xyz(D), b2));
        float3 n = sub(xyz(A), q);
        const float l = len(n);
        n = dvs(n, l);
        const float cc = l - h;
        float s = A.w + B.w * b0 * b0 + C.w * b1 * b1 + D.w * b2 * b2;
        if (s == 0.f) return f3(0.f, 0.f, 0.f);
        s = cc / s;
        s = cc < 0.f ? s : 0.f;
        if (slot == 0) return mul(n, -s * A.w);
        if (slot == 1) return mul(mul(neg(n), b0), -s * B.w);
        if (slot == 2) return mul(mul(neg(n), b1), -s * C.w);
        return mul(mul(neg(n), b2), -s * D.w);
    }
    const float b0 = w.x, b1 = w.y, b2 = -w.z, b3 = -w.w;
    const float3 q0 = add(mul(xyz(A), b0), mul(xyz(B), b1));
    const float3 q1 = add(mul(xyz(C), b2), mul(xyz(D), b3));
    float3 n = sub(q0, q1);
    const float l = len(n);
    n = dvs(n, l);
    const float cc = l - h;
    float s = A.w * b0 * b0 + B.w * b1 * b1 + C.w * b2 * b2 + D.w * b3 * b3;
    if (s == 0.f) return f3(0.f, 0.f, 0.f);
    s = cc / s;
    s = cc < 0.f ? s : 0.f;
    if (slot == 0) return mul(mul(n, b0), -s * A.w);
    if (slot == 1) return mul(mul(n, b1), -s * B.w);
    if (slot == 2) return mul(mul(neg(n), b2), -s * C.w);
    return mul(mul(neg(n), b3), -s * D.w);
}

// The same contact evaluated once for its four slots: out[j] equals
// contact_corr_pos(..., j) (the same expressions on the same operands).
__device__ __forceinline__ void contact_all_pos(float4 A, float4 B, float4 C, float4 D, float4 w, bool isvf, float h,
                                                float3 out[4]) {
    float3 n;
    float s;
    float b[4];
    if (isvf) {
        b[0] = 1.f;
        b[1] = clampf(-w.y, 0.f, 1.f), b[2] = clampf(-w.z, 0.f, 1.f), b[3] = clampf(-w.w, 0.f, 1.f);
        const float3 q = add(add(mul(xyz(B), b[1]), mul(xyz(C), b[2])), mul(xyz(D), b[3]));
        n = sub(xyz(A), q);
        const float l = len(n);
        n = dvs(n, l);
        const float cc = l - h;
        s = A.w + B.w * b[1] * b[1] + C.w * b[2] * b[2] + D.w * b[3] * b[3];
        if (s == 0.f) { out[0] = out[1] = out[2] = out[3] = f3(0.f, 0.f, 0.f); return; }
        s = cc / s;
        s = cc < 0.f ? s : 0.f;
        out[0] = mul(n, -s * A.w);
        out[1] = mul(mul(neg(n), b[1]), -s * B.w);
        out[2] = mul(mul(neg(n), b[2]), -s * C.w);
        out[3] = mul(mul(neg(n), b[3]), -s * D.w);
        return;
    }
    b[0] = w.x, b[1] = w.y, b[2] = -w.z, b[3] = -w.w;
    const float3 q0 = add(mul(xyz(A), b[0]), mul(xyz(B), b[1]));
    const float3 q1 = add(mul(xyz(C), b[2]), mul(xyz(D), b[3]));
    n = sub(q0, q1);
    const float l = len(n);
    n = dvs(n, l);
    const float cc = l - h;
    s = A.w * b[0] * b[0] + B.w * b[1] * b[1] + C.w * b[2] * b[2] + D.w * b[3] * b[3];
    if (s == 0.f) { out[0] = out[1] = out[2] = out[3] = f3(0.f, 0.f, 0.f); return; }
    s = cc / s;
    s = cc < 0.f ? s : 0.f;
    out[0] = mul(mul(n, b[0]), -s * A.w);
    out[1] = mul(mul(n, b[1]), -s * B.w);
    out[2] = mul(mul(neg(n), b[2]), -s * C.w);
    out[3] = mul(mul(neg(n), b[3]), -s * D.w);
}

// Static-collider contacts of vertex i (lc_batch_set_collider): each slot's
// plane (unit normal n towards the free side, d0 = n . a) is the one-sided
// constraint n . x >= d0 + h on the vertex alone (the face does not move).
// The vertex is projected onto them in slot order at the end of every solver
// iteration, after the Jacobi average: collisions are projected last, so the
// averaged stretch and bend corrections cannot pull a vertex that crossed a
// face back through it.  The caller skips pinned vertices.
// act (adjoint batches): receives the bit mask of the slots projected.
__device__ __forceinline__ float3 collider_project(const DevPtrs &d, int i, float3 x, float h,
                                                  uint8_t *act = nullptr) {
    const int nc = d.ccnt[i];
    uint32_t m = 0;
    for (int k = 0; k < nc; ++k) {
        const float4 pl = d.cw[(size_t)i * kColliderSlots + k];
        const float c = dot(xyz(pl), x) - pl.w - h;
        if (c < 0.f) {
            x = add(x, mul(xyz(pl), -c));
            m |= 1u << k;
        }
    }
    if (act) *act = (uint8_t)m;
    return x;
}

}  // namespace lc
