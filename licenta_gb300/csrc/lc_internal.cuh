// lc_internal.cuh — device-side layout and helpers shared by the cloth-step
// kernels.  All cloths of a batch live in flat arrays behind per-cloth
// offsets (ClothDev); a "slot" is a position in a cloth's current triangle
// order, which the Morton sort permutes and which persists between steps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lc/lc.h"

namespace lc {

constexpr int kThreads = 256;
constexpr int kSortBits = 8;
constexpr int kSortBuckets = 1 << kSortBits;
constexpr int kSortTile = 2048;          // keys per sort tile (256 threads x 8)
constexpr int kSortPassesMax = 8;        // 8-bit digits of a 63-bit key
constexpr int kTraverseStack = 64;       // Collision/CudaBVH.cu:38
constexpr int kTraverseBlockMax = 256;   // largest traversal block (the packet kernel is bounded for 6 of them per SM)
constexpr int kScanBlocks = 1024;        // fixed grid of the device-count scans
constexpr int kPairGroup = 32;           // consecutive pairs per narrowphase expansion warp (one per lane)
constexpr int kColliderSlots = LC_COLLIDER_SLOTS;  // static-collider contacts kept per cloth vertex and step
constexpr int kColliderStack = 64;       // collider BVH traversal stack
constexpr float kColliderMargin = 4.f;   // collider detection reach beyond the contact layer, in thicknesses

// Device error word bits (latched, reported by lc_batch_sync).
enum : uint32_t {
    ERR_VF_OVERFLOW = 1u << 0,
    ERR_EE_OVERFLOW = 1u << 1,
    ERR_STACK = 1u << 2,
    ERR_TREE = 1u << 3,
    ERR_DYN_OVERFLOW = 1u << 4,
    ERR_CAND_OVERFLOW = 1u << 5,
    ERR_COLL_OVERFLOW = 1u << 6,   // more static-collider contacts at a vertex than kColliderSlots
    ERR_SORT = 1u << 7,            // a sort look-back wait ran past its bound
};

// Per-cloth descriptor in device memory.
struct ClothDev {
    int v_off, V;          // vertices
    int t_off, T;          // triangles / slots
    int n_off;             // nodes: 2T-1 per cloth (internal 0..T-2, leaves T-1..2T-2)
    int i_off;             // internal nodes: T-1 per cloth
    int chunk;             // min(BVHChunkSize, T)
    int64_t pc_off;        // pair chunk area offset (T * chunk per cloth)
    int f_off, F;          // pinned (fixed) vertices
    int64_t lra_off;       // V * F attachment rest lengths
    int iters;             // solver iterations
    int wind_on;
    int ground_on, sphere_on;
    int tri_bend;          // bends are triangle bends (useTriangleBending): b_ids = (b0, b1, v, h0 bits)
    int friction;          // CudaPBD::ApplyFriction after the integration (useFriction)
    float kfriction;
    int morton_mode, leaf_quirk;
    float dt, h, kdamp, kglobal;
    float g[3];
    float ground_y;
    float wmin[3], wmax[3];
    float morton_origin[3], morton_scale;
    float sphere_pos[3], sphere_r;
    float wind_start[3], wind_min[3], wind_max[3];
    float wind_var_min, wind_var_max;
    int s_off, s_cnt;      // stretch constraints of the cloth (global range)
    int b_off, b_cnt;      // bend constraints
    int coll_root;         // root node of the cloth's static collider BVH, -1 without one
    int coll_cw;           // 1: the collider's faces turn clockwise seen from its free side
};

// Mutable per-cloth state that kernels update on the device (wind + RNG).
struct ClothState {
    float wind[3];
    float pad;
    unsigned long long rng;
};

// Everything a step kernel may need, passed by value.
struct DevPtrs {
    int C;                 // cloths
    int Vtot, Ttot, Ntot, Itot;
    const ClothDev *cloth;
    ClothState *cstate;
    const int *vcloth;     // vertex -> cloth
    const int *tcloth;     // slot -> cloth
    float4 *x;             // xyz, w = inverse mass
    float4 *x2;            // Jacobi double buffer
    float4 *xp;            // xyz, w = mass
    float4 *v;
    float4 *vn;            // running vertex normals
    const int4 *tri;       // original triangle -> (v1, v2, v3 global ids, features)
    uint32_t *perm;        // slot -> original triangle (global)
    uint32_t *perm_alt;
    int4 *tri_slot;        // slot -> its triangle record (tri[perm[slot]]), written after each sort
    unsigned long long *keys, *keys_alt;
    uint32_t *payload, *payload_alt;  // pre-sort slot carried through the sort
    float4 *fn;            // face normal per original triangle
    const int *vt_off;     // vertex -> incident original triangles (CSR)
    const int *vt_idx;
    float4 *nmin, *nmax;   // node AABBs
    float4 *leaf_tmp_min, *leaf_tmp_max;  // pre-sort leaf boxes (fixed mode)
    int *parent;
    int2 *child;
    int2 *rml;
    int *visit;
    int *nend;             // per internal node: the other end j of its leaf range (may be null)
    int2 *rexit;           // refit: (cloth, node) arrivals left for the upper pass (2 x internal nodes)
    uint32_t *nrexit;      // their count (cleared by k_karras)
    float4 *wnode;         // 4 per internal node: {lmin, left} {lmax, rmll} {rmin, right} {rmax, rmlr} (may be null)
    uint32_t *pair_cnt;    // per slot
    uint32_t *pair_off;    // per slot (exclusive scan), + total at [Ttot]
    uint32_t *pair_chunk;  // chunk area: j leaf (local) per entry
    uint2 *pairs;          // compacted (global slot i, global slot j)
    uint64_t pair_cap;
    uint16_t *pair_mask;   // per pair: bits 0..5 VF, 6..14 EE candidates past the AABB cull
    uint32_t *grp_vf_cnt, *grp_ee_cnt;    // per group of 32 consecutive pairs: VF / EE candidate counts
    uint32_t *grp_vf_off, *grp_ee_off;    // per group: first candidate (exclusive scans)
    uint32_t *ngroups;                    // groups of the step (device)
    int4 *cand, *cand_e;                  // VF / EE candidates: their four vertex ids, in candidate order
    uint64_t cand_cap;                    // per list
    uint32_t *hitg_mask[2];               // per group of 32 candidates (VF, EE): CCD hit bits
    uint32_t *hitg_cnt[2];                // per group: hits
    uint32_t *hitg_off[2];                // per group: first contact (exclusive scans), total at [groups]
    uint32_t *hitg_n;                     // [2] groups of the step (device)
    uint32_t *hit_q[2];                   // VF / EE hits in any order: candidate index ...
    float4 *hit_w[2];                     // ... and contact weights (capacity vf_cap / ee_cap)
    float4 *hit_nrm;                      // VF hits: unit face normal at the hit (friction; may be null)
    float4 *hit_tn[2];                    // VF / EE hits: unit normal (xyz) and time of contact (w), the
                                          // PrimitiveContact n and t (full contact records; may be null)
    uint32_t *hit_n;                      // [2] hit counts of the step
    uint4 *crange;         // per cloth: [vf0, vf1) and [ee0, ee1) contact ranges
    int4 *vf_v; float4 *vf_w;   // VF contacts (ids, weights)
    float4 *vf_n;               // VF contacts: face normal at the hit (friction; may be null)
    float4 *vf_tn, *ee_tn;      // contacts: normal and time of contact (full contact records; may be null)
    int friction_any;           // some cloth of the batch uses friction
    int4 *ee_v; float4 *ee_w;   // EE contacts
    uint64_t vf_cap, ee_cap;
    uint32_t *dyn_cnt, *dyn_off, *dyn_cur;  // per vertex dynamic-correction entries
    uint32_t *dyn_ent;
    uint64_t dyn_cap;
    // static constraints
    const int *soff;       // per vertex CSR into sent (Vtot+1)
    const uint32_t *sent;  // kind<<31 | role<<29 | constraint
    const int2 *s_ids;     // stretch (v1, v2) global ids
    const float2 *s_par;   // (l0, kp)
    const int4 *b_ids;     // bend (p1, p2, p3, p4)
    const float *b_kp;
    // LRA / ground
    const int *fixed;      // global ids of pinned vertices, per cloth at f_off
    const float *lra_l0;
    uint8_t *lra_flag;
    float4 *ground_qc;     // xyz = contact point, w = flag
    // reductions and counters
    double *damp;          // 16 per cloth
    unsigned long long *counters;  // [0] pairs [1] vf [2] ee [3] dropped
    uint32_t *err;
    uint32_t *scan_tmp;    // kScanBlocks + 1 partials
    // sort bookkeeping
    const int *stile_cloth;   // sort tile -> cloth
    const int *stile_start;   // sort tile -> first slot (global)
    int nstiles;
    uint32_t *shist;          // per tile x bucket counts / offsets
    // one-sweep scratch (both null: per-pass histograms and k_sort_offsets):
    // sseg = kSortPassesMax tile tickets, then per segment x pass x digit the
    // segment's digit totals; sstat = per pass x tile x digit look-back status
    uint32_t *sseg, *sstat;
    const int *vblk_cloth, *vblk_start;  // vertex blocks never straddle cloths
    const int *vb_first;                 // per cloth: first vertex block (C+1 entries)
    double *damp_part;                   // 16 partial sums per vertex block
    int nvblk;
    // discrete decisions of the last step, recorded only for parity checks
    uint32_t *dbg_ground_it;  // per vertex: bit it = ground term counted in iteration it
    uint8_t *dbg_dyn_nz;      // per iteration x dynamic entry: correction was non-zero
    int8_t *dbg_sphere;       // per vertex: ray-sphere outcome (-1, 0, 1)
    float kpi_gap;            // pi - (float)3.14159265359f, rest-angle offset of the bend term
    // static triangle colliders (lc_batch_set_collider), all cloths' in flat arrays
    const float4 *cv;         // collider vertices
    const int4 *ct;           // collider triangles: global vertex ids, w = cloth
    const float4 *cnmin, *cnmax;  // collider BVH node boxes
    const int2 *cnchild;      // children, or (-(triangle + 1), -1) at a leaf
    float4 *cface_geo;        // per collider triangle, 5 float4: (n, d0) (a, perimeter) (e1, d00) (e2, d11)
                              // (d01, den, -, -): its plane towards the free side and the barycentric set-up
    int *ccnt;                // per cloth vertex: collider contacts of the step (<= kColliderSlots)
    int *cface;               // per cloth vertex x slot: collider triangle (global), ascending
    float4 *cw;               // per cloth vertex x slot: the contact's plane (unit normal to the free side, n . a)
    uint8_t *coll_act;        // adjoint batches: (iterations + 1) x vertex bit masks of the collider slots
                              // projected, [0] before the solver, [it + 1] in iteration it (else null)
    int any_collider;
    float4 *tape_x;           // a recorded step on the cluster solver: (tape_K + 1) x Vtot iterates (else null)
    float4 *vbox;             // per vertex, written by the prediction: the swept box of x_prev and x widened by
                              // the thickness, lo at [2 v], hi at [2 v + 1] (may be null: computed in place)
    int tape_K;
};

// Reverse pass of one step (lc_adjoint.cu): the recorded step's tape and the
// work buffers of the reverse sweep.  Gradient buffers are float4 (w unused).
struct AdjPtrs {
    const float4 *tape_x;    // (K+1) x Vtot: solver iterates x^0 (prediction) .. x^K
    const float4 *tape_xin;  // state x at the start of the step (damping input)
    const float4 *tape_vb;   // velocity after the global damping (damping input)
    const int *s_slot;       // 2 per stretch constraint: static CSR entry of (constraint, role)
    const int *b_slot;       // 4 per bend constraint
    float4 *slot;            // per static CSR entry: the constraint's contribution to that vertex
    float4 *dyn;             // per dynamic entry (contact * 4 + vertex)
    float *fixed;            // 3 per pinned vertex: LRA contributions (block sums + atomics)
    float4 *u;               // dL/dx^{k+1} / count, per vertex
    float4 *gx, *gxp, *gv;   // state gradients: after the step on entry, before it on exit
    double *red;             // 8 per vertex block (partials), then 8 per cloth (totals)
    int nvblk_red;           // offset of the cloth totals in red
    int K;                   // solver iterations of the recorded step (max over cloths)
    int E, B;                // stretch / bend constraints of the batch
};

// ---------------------------------------------------------------------------
// float3 algebra in the operation order of Core/CudaUtils.cu:32-276.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }
__host__ __device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 neg(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 mul(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 dvs(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ float3 addc(float3 a, float s) { return f3(a.x + s, a.y + s, a.z + s); }
__host__ __device__ __forceinline__ float3 subc(float3 a, float s) { return f3(a.x - s, a.y - s, a.z - s); }
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// Length as sqrt of the dot product (stands in for the reference's norm3df).
__host__ __device__ __forceinline__ float len(float3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__host__ __device__ __forceinline__ float dist(float3 a, float3 b) { return len(sub(a, b)); }
__host__ __device__ __forceinline__ float3 normalize(float3 a) { return dvs(a, len(a)); }
__host__ __device__ __forceinline__ bool is_zero(float3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
__host__ __device__ __forceinline__ float3 vmin(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__host__ __device__ __forceinline__ float3 vmax(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__host__ __device__ __forceinline__ float3 min3(float3 a, float3 b, float3 c) { return vmin(a, vmin(b, c)); }
__host__ __device__ __forceinline__ float3 max3(float3 a, float3 b, float3 c) { return vmax(a, vmax(b, c)); }
__host__ __device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(lo, v), hi); }
__host__ __device__ __forceinline__ bool between(float v, float lo, float hi) { return v >= lo && v <= hi; }
__host__ __device__ __forceinline__ bool overlap(float3 amin, float3 amax, float3 bmin, float3 bmax) {
    bool a = amax.x < bmin.x || amin.x > bmax.x;
    bool b = amax.y < bmin.y || amin.y > bmax.y;
    bool c = amax.z < bmin.z || amin.z > bmax.z;
    return !(a || b || c);
}
__host__ __device__ __forceinline__ float4 f4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

static const float kEpsPbd = 0.00000001f;   // Physics/CudaPBD.cu:33
static const float kEpsCubic = 1.f / 1000000;  // Physics/CudaCubicSolver.cuh:12
static const float kEpsEE = 0.000000001f;   // Collision/CudaPrimitiveTests.cu:124
static const float kPi = 3.14159265359f;    // Physics/CudaPBD.cu:35

// Wind-variation RNG (replaces the reference's std::rand(); the same
// xorshift is used on both sides of every parity test).
__host__ __device__ __forceinline__ double xs_uniform(unsigned long long &s) {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace lc
