/*
 * lc.h — C ABI of the GB300 cloth-step engine (PBD + LBVH self-collision).
 *
 * Every entry point replaces one piece of the reference's GPU cloth body
 * (Tureyz/Licenta, paths relative to LicentaV2/LicentaV2/):
 *
 *   Physics::CudaDeformableBody ctor      Physics/CudaDeformableBody.h:23-24, .cpp:30-285
 *   Physics::CudaDeformableBody::FixedUpdate   Physics/CudaDeformableBody.cpp:550-627
 *   Physics::CudaDeformableBody::Update        Physics/CudaDeformableBody.cpp:629-638
 *   Physics::CudaDeformableBody::SetSpherePos  Physics/CudaDeformableBody.cpp:640-643
 *   CudaBVH::GenerateBVH2 / ComputeTreeAABBs / GetAABBCollisions
 *                                          Collision/CudaBVH.cuh:15-33, Collision/CudaBVH.cu:9-188
 *   DeformableUtils::CreateTriangleTests / CCDTriangleTests
 *                                          Collision/CudaCollisionDetection.cuh:28-46
 *
 * Conventions: plain C PODs, explicit stream (a cudaStream_t passed as void*,
 * NULL = legacy default stream), every call returns lc_status, no exception
 * crosses the boundary.  A handle is thread-compatible (one host thread at a
 * time), not thread-safe.  Device-side failures (capacity overflow, a
 * traversal stack overflow) are latched in a device error word and reported
 * by the next call that synchronises (lc_batch_sync, any *_get_* call).
 */
#ifndef LC_LC_H
#define LC_LC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lc_status {
    LC_OK = 0,
    LC_ERR_INVALID_ARG = 1,
    LC_ERR_OOM = 2,
    LC_ERR_CAPACITY_OVERFLOW = 3,
    LC_ERR_TIMEOUT = 4,            /* a bounded device-side wait gave up (a sort or look-back status
                                      that never arrived); reported by the next synchronising call */
    LC_ERR_CUDA = 5,
    LC_ERR_NOT_SUPPORTED = 6,
    LC_ERR_STACK_OVERFLOW = 7
} lc_status;

/* Morton encodings.  REF63: 21 bits per axis of x*2^21 clamped to
 * [0, 2^21-1], the live encoder of Core/CudaUtils.cu:278-287,310-325.
 * K30: 10 bits per axis (x*2^10 clamped to [0,1023]), the commented-out
 * 30-bit encoder of Core/CudaUtils.cu:289-308. */
enum { LC_MORTON_REF63 = 0, LC_MORTON_K30 = 1 };

/*
 * Cloth parameters.  The first block is field-for-field
 * Physics::ClothParams (Physics/Structs.h:23-61) minus its device vector of
 * pinned flags (passed in lc_cloth_desc.pinned instead); the second block
 * holds what the reference hard-codes or leaves implicit.
 */
typedef struct lc_cloth_params {
    float timestep;
    float kFriction;
    float kStretch;
    float kShear;            /* stored, unused by the live step (as in the reference) */
    float kBend;
    float kDamp;
    float kSpringDamp;       /* stored, unused by the live step */
    float thickness;
    float objectMass;
    float globalVelDamp;
    float strainLimit;
    float gravity[3];
    float minWindDir[3];
    float startWindDir[3];
    float maxWindDir[3];
    float windMinVariation;
    float windMaxVariation;
    int32_t windOn;
    float worldMin[3];
    float worldMax[3];
    int32_t dims[2];         /* grid rows x columns; triangle bending (useTriangleBending) walks the grid
                                with them, otherwise informational */
    int32_t solverIterations;
    int32_t ccdIterations;   /* stored, unused by the live step */
    int32_t BVHChunkSize;
    uint64_t benchmarkSample;
    int32_t useTriangleBending;
    int32_t colorContacts;
    int32_t useFriction;

    /* --- not in ClothParams --- */
    int32_t thicknessFromMesh;  /* 1: thickness = |x0 - x1| / 3 (Physics/CudaDeformableBody.cpp:86) */
    int32_t mortonMode;         /* LC_MORTON_REF63 (default) or LC_MORTON_K30 */
    int32_t refLeafAabbQuirk;   /* 1 (default): leaf k keeps the AABB of pre-sort slot k (reference behaviour) */
    int32_t groundOn;           /* 1: ground constraints at worldMin.y + thickness (reference always on) */
    float mortonOrigin[3];      /* Morton input = (p - origin) * scale; identity = (0,0,0), 1 */
    float mortonScale;
    uint64_t windSeed;          /* seeds the wind-variation draw that the reference takes from std::rand() */
    int32_t sphereOn;           /* analytic sphere of CudaPBD::SetSpherePos (Physics/CudaPBD.cu:460-472) */
    float spherePos[3];
    float sphereRadius;
} lc_cloth_params;

/* One cloth: the constructor arguments of Physics::CudaDeformableBody. */
typedef struct lc_cloth_desc {
    int32_t num_vertices;
    int32_t num_triangles;
    const float *positions;   /* 3 * num_vertices, host memory */
    const uint32_t *indices;  /* 3 * num_triangles, host memory */
    const uint8_t *pinned;    /* num_vertices flags (fixedVerts), may be NULL */
    lc_cloth_params params;
} lc_cloth_desc;

/* Capacities of the per-step device buffers; 0 picks the default. */
typedef struct lc_batch_options {
    uint64_t vf_capacity;     /* VF contacts kept per step over the whole batch (default max(8 * total triangles, 4096)) */
    uint64_t ee_capacity;     /* EE contacts kept per step (default max(8 * total triangles, 4096)) */
    int32_t use_graph;        /* 1 (default): capture one step in a CUDA graph and replay it */
    int32_t debug_capture;    /* 1: keep intermediate buffers of the last step for lc_batch_debug_get */
    int32_t solver_variant;   /* 0 = auto (cluster scatter when every cloth fits on chip, else 1),
                                 1 = per-vertex gather over global memory, 2 = cluster on-chip gather,
                                 3 = cluster on-chip scatter with fixed-point accumulators */
    int32_t block_size;       /* block size of the global-memory Jacobi kernel (0 = default) */
    uint64_t cand_capacity;   /* narrowphase candidates kept per step after the AABB cull, per kind (VF, EE);
                                 default min(15 * pair capacity, max(32 * total triangles, 4 Mi)); at most
                                 2^31 - 16 */
    int32_t adjoint;          /* 1: keep the tape and decision records lc_batch_adjoint_step needs; every step,
                                 recorded or not, runs on the batch's solver */
} lc_batch_options;

typedef struct lc_batch lc_batch;

/* Fills the reference defaults of Managers/MastersSimulationManager.cpp:33-62
 * (with gravity, dims and wind as that file sets them) plus the extension
 * defaults above. */
void lc_default_params(lc_cloth_params *out);
void lc_default_options(lc_batch_options *out);

/* Builds the device state of num_cloths independent cloths (constraints,
 * LRA, feature ownership, initial triangles/normals) — the work of the
 * CudaDeformableBody constructor and CudaPBD::Init (Physics/CudaPBD.cu:39-275)
 * for each cloth, packed behind one offset table. */
lc_status lc_batch_create(const lc_cloth_desc *descs, int32_t num_cloths,
                          const lc_batch_options *opts, lc_batch **out);
lc_status lc_batch_destroy(lc_batch *b);

/* nsteps x CudaDeformableBody::FixedUpdate for every cloth of the batch, in
 * one launch sequence per step (asynchronous on stream). */
lc_status lc_batch_step(lc_batch *b, int32_t nsteps, void *stream);

/* Waits for the stream work of the batch and reports latched device errors. */
lc_status lc_batch_sync(lc_batch *b);

/* Concurrent batches.  A group steps several batches (for example the two
 * halves of one workload) at the same time, each on a stream of the group's
 * own, forked from and joined back into the caller's stream: one batch's
 * latency-bound kernels (hierarchy build, on-chip solver) then overlap with
 * the other's.  The batches stay owned by the caller and usable on their own;
 * each must be in at most one group and be destroyed after it.  An extension
 * of lc_batch_step (Physics/CudaDeformableBody.cpp:550-627 for each cloth)
 * with no counterpart in the reference. */
typedef struct lc_group lc_group;
lc_status lc_group_create(lc_batch *const *batches, int32_t count, lc_group **out);
/* nsteps x lc_batch_step of every batch, interleaved step by step across the
 * group's streams; stream waits for all of them.  lc_batch_sync of a member
 * then waits on stream. */
lc_status lc_group_step(lc_group *g, int32_t nsteps, void *stream);
/* nsteps steps of every batch with its state moved in and out at each step,
 * for callers that keep the state on the host: on each batch's stream of the
 * group, step after step, its slice of x_in, x_prev_in, v_in (packed as
 * lc_batch_write_state takes them, the batches' cloths one after the other in
 * group order) is written, the batch steps once and its state is read into
 * the same slice of the out arrays.  The batches are joined only at the end,
 * so one batch's copies overlap the others' steps.  NULL arrays are skipped;
 * in and out may be the same arrays (each step then starts from the state the
 * previous one read back).  stream waits for all of it. */
lc_status lc_group_step_io(lc_group *g, int32_t nsteps, const float *x_in, const float *x_prev_in, const float *v_in,
                           float *x_out, float *x_prev_out, float *v_out, int32_t is_host, void *stream);
lc_status lc_group_destroy(lc_group *g);

lc_status lc_batch_num_cloths(const lc_batch *b, int32_t *out);
lc_status lc_batch_cloth_sizes(const lc_batch *b, int32_t cloth, int32_t *num_vertices,
                               int32_t *num_triangles);

/* State of one cloth as float3 arrays (3 * V floats each); any pointer may be
 * NULL.  x = m_dPositions, x_prev = m_dPrevPositions, v = m_dVelocities,
 * vn = m_dAccumulatedVertexNormals.  *_host = 1 for host memory. */
lc_status lc_batch_get_state(lc_batch *b, int32_t cloth, float *x, float *x_prev, float *v,
                             float *vn, int32_t is_host);
lc_status lc_batch_set_state(lc_batch *b, int32_t cloth, const float *x, const float *x_prev,
                             const float *v, const float *vn, int32_t is_host);

/* Triangle order (slot -> original triangle id) that persists between steps
 * because the Morton sort permutes the triangle array in place
 * (Physics/CudaDeformableUtils.cu:346-349). */
lc_status lc_batch_get_triangle_order(lc_batch *b, int32_t cloth, uint32_t *perm);
lc_status lc_batch_set_triangle_order(lc_batch *b, int32_t cloth, const uint32_t *perm);

/* Positions of every cloth, packed in cloth order (3 floats per vertex) into
 * host or device memory: the copy-out of CudaDeformableBody::Update /
 * FinalVertUpdate (Physics/CudaDeformableBody.cpp:473-495), which publishes
 * m_dPrevPositions.  Asynchronous on stream when dst is pinned or device memory. */
lc_status lc_batch_read_positions(lc_batch *b, float *dst, int32_t is_host, void *stream);

/* DeformableUtils::FinalVerticesUpdate (Physics/CudaDeformableUtils.cu:319-344,
 * called by CudaDeformableBody::FinalVertUpdate, Physics/CudaDeformableBody.cpp:473-495)
 * into a caller-owned DEVICE buffer of interleaved vertex records, for a
 * renderer or a wire format to map without a host round trip: record i of the
 * batch (cloths packed in order) starts at dst + i * stride bytes; its three
 * position floats (the published positions, x_prev) go at pos_offset and its
 * three normal floats (the running vertex normals) at normal_offset, and no
 * other byte is written.  Rendering::VertexFormat is stride 48, position 0,
 * normal 28 (Rendering/VertexFormat.h:24-30).  Offsets must be 4-byte
 * aligned, the stride a multiple of 4 and at least 12 past both offsets. */
lc_status lc_batch_write_vertex_records(lc_batch *b, void *dst, int64_t stride, int32_t pos_offset,
                                        int32_t normal_offset, void *stream);

/* Whole-batch state in one call each way, packed in cloth order (3 floats
 * per vertex per array; NULL arrays are skipped).  Asynchronous on stream;
 * host memory should be pinned.  Used by callers that keep the cloth state on
 * the host between steps.  A host array moves as one contiguous copy through
 * a staging buffer of the batch, so copies of one batch must stay ordered on
 * one stream at a time. */
lc_status lc_batch_write_state(lc_batch *b, const float *x, const float *x_prev, const float *v,
                               int32_t is_host, void *stream);
lc_status lc_batch_read_state(lc_batch *b, float *x, float *x_prev, float *v, int32_t is_host,
                              void *stream);

/* Per-phase timing of nsteps eager steps with CUDA events, using the seven
 * phase labels of the reference's GPUBenchmark (Simulation/GPUBenchmark.cu:14-77,
 * labels at Physics/CudaDeformableBody.cpp:556-594), plus the mean duration of
 * single launches of the hot kernels.  All times in milliseconds per step or
 * per launch. */
typedef struct lc_profile {
    float phase_ms[7];        /* 1 External, 2 Update Triangles, 3 Build BVH, 4 Create Triangle Tests,
                                 5 Perform Triangle Tests, 6 PBD Solver, 7 PBD Integration */
    float jacobi_ms;          /* one Jacobi iteration launch */
    float traverse_ms;        /* one traversal launch */
    float narrow_ms;          /* one narrowphase filter launch (candidate masks, counts per group of pairs) */
    float sort_ms;            /* whole segmented sort */
    float step_ms;            /* sum of the phases */
    uint32_t kernels_per_step;
    float solver_ms;          /* whole solver (set-up + iterations + integration on the cluster path) */
    int32_t solver_variant;   /* 1 = per-vertex gather, 2 = cluster on-chip */
    int32_t cluster_size;     /* CTAs per cloth on the cluster path */
    float ccd_vf_ms;          /* one vertex-face CCD launch */
    float ccd_ee_ms;          /* one edge-edge CCD launch */
} lc_profile;
lc_status lc_batch_profile(lc_batch *b, int32_t nsteps, void *stream, lc_profile *out);

/* CudaPBD::SetSpherePos for one cloth (Physics/CudaPBD.cu:460-472). */
lc_status lc_batch_set_sphere(lc_batch *b, int32_t cloth, const float pos[3], float radius);

/* Static triangle collider of one cloth (no counterpart in the reference,
 * whose only collider is the analytic sphere of CudaPBD::SetSpherePos): a
 * mesh that does not move (vertices: 3 floats each, host memory; indices: 3
 * per triangle; num_triangles = 0 removes the cloth's collider).  winding
 * names the free side: LC_WINDING_CCW when the faces turn counter-clockwise
 * seen from it ((b - a) x (c - a) points there), LC_WINDING_CW for the
 * opposite, which is how lc_mesh_icosphere winds its sphere.  Every step,
 * after the self-collision narrowphase, each cloth vertex is tested against
 * the collider triangles whose boxes meet its swept box inflated by 5 h (h
 * the cloth's thickness).  With n the face's unit normal towards the free
 * side and the vertex's heights s0 = n . (x_prev - a), s1 = n . (x - a) (x
 * the prediction), the face is a contact when s1 < 5 h, s0 > -4 h, and the
 * point where the vertex crosses the face's plane (without a crossing, the
 * prediction) lies on the triangle within the barycentric tolerance of the
 * reference's TestVF (h / perimeter, Collision/CudaPrimitiveTests.cu:
 * 348-406).  The reach beyond the contact layer lets the constraint act on a
 * vertex that the solver iterations drag towards the face, and brings back
 * one that ended a step behind it.  The hits (at most LC_COLLIDER_SLOTS per
 * vertex, the lowest triangle indices; more is a capacity error reported by
 * lc_batch_sync) are one-sided constraints n . x >= n . a + h on the vertex
 * alone.  The vertex is projected onto them, in slot order, before the first
 * solver iteration and at the end of every iteration, after the Jacobi
 * average, so collisions are projected last; pinned vertices do not move.
 * (The reference's two-sided VF projection, averaged with the other
 * corrections, leaves a vertex that crossed a face within one step on the
 * far side; a static face has a side.)  A BVH over the triangles is built on
 * the host once per call.  In batches created with adjoint the reverse pass
 * differentiates through the projections, with the contact planes held
 * fixed as the recorded step found them. */
#define LC_COLLIDER_SLOTS 8
enum { LC_WINDING_CCW = 0, LC_WINDING_CW = 1 };
lc_status lc_batch_set_collider(lc_batch *b, int32_t cloth, const float *vertices, int32_t num_vertices,
                                const uint32_t *indices, int32_t num_triangles, int32_t winding);

/* Per-constraint stiffness override (stretch: E values, bend: B values). */
lc_status lc_batch_set_stiffness(lc_batch *b, int32_t cloth, const float *k_stretch,
                                 const float *k_bend);
lc_status lc_batch_constraint_counts(const lc_batch *b, int32_t cloth, int32_t *num_stretch,
                                     int32_t *num_bend);

/* Intermediate buffers of the last step (needs options.debug_capture).
 * Writes at most cap elements into dst (host memory) and the element count
 * into *count. */
enum {
    LC_DBG_PRED_X = 1,        /* float3 per vertex: x after PBDStepExternal */
    LC_DBG_PRED_XPREV = 2,    /* float3 per vertex: x_prev after PBDStepExternal */
    LC_DBG_PRED_V = 3,        /* float3 per vertex: v after PBDStepExternal */
    LC_DBG_PERM_BEFORE = 4,   /* u32 per slot: triangle order before the sort */
    LC_DBG_MORTON = 5,        /* u64 per slot: sorted Morton codes */
    LC_DBG_PERM = 6,          /* u32 per slot: triangle order after the sort */
    LC_DBG_LEFTS = 7,         /* i32 per internal node */
    LC_DBG_RIGHTS = 8,
    LC_DBG_PARENTS = 9,       /* i32 per node (2T-1) */
    LC_DBG_RML = 10,          /* i32 pair per internal node: rightmost leaf of left/right child */
    LC_DBG_NODE_AABB = 11,    /* 6 floats per node: min xyz, max xyz */
    LC_DBG_PAIRS = 12,        /* u32 pair per broadphase pair (leaf i, leaf j) */
    LC_DBG_VF = 13,           /* lc_contact per vertex-face contact */
    LC_DBG_EE = 14,           /* lc_contact per edge-edge contact */
    LC_DBG_FEATURES = 15,     /* u8 per original triangle: ownership bits */
    /* Discrete decisions of the last step, so that a checker can replay them
     * (contact sets frozen): */
    LC_DBG_GROUND = 16,       /* u8 per vertex: ground constraint created (Physics/CudaPBD.cu:1490) */
    LC_DBG_GROUND_ACTIVE = 17,/* u32 per vertex: bit it = ground term counted in iteration it (:1612) */
    LC_DBG_LRA = 18,          /* u8 per vertex x pinned vertex: attachment active (:1588) */
    LC_DBG_DYN_ACTIVE = 19,   /* u8 per iteration x (VF contacts, then EE contacts) x 4 slots:
                                 correction non-zero, i.e. counted (:1466) */
    LC_DBG_SPHERE = 20,       /* i8 per vertex: ray-sphere outcome -1/0/1 (:1523) */
    LC_DBG_VF_NORMAL = 21,    /* float3 per vertex-face contact: face normal at the hit, which friction
                                 uses (Collision/CudaPrimitiveTests.cu:393); batches with friction only */
    LC_DBG_COLLIDER = 22      /* lc_contact per vertex x LC_COLLIDER_SLOTS: static-collider contacts of the
                                 step, v = (vertex, collider triangle or -1, 0, 0), w = the contact's plane
                                 (unit normal towards the free side, then n . a) */
};

/* A contact as the solver consumes it: the ids/weights of
 * Physics::PrimitiveContact (Physics/Structs.h:106-129). */
typedef struct lc_contact {
    int32_t v[4];
    float w[4];
} lc_contact;

lc_status lc_batch_debug_get(lc_batch *b, int32_t cloth, int32_t what, void *dst, uint64_t cap,
                             uint64_t *count);

/* Device counters of the last step: [0] pairs, [1] VF contacts, [2] EE
 * contacts, [3] pairs dropped by the per-leaf chunk cap (the reference drops
 * them silently, Collision/CudaBVH.cu:69-92). */
lc_status lc_batch_counters(lc_batch *b, uint64_t out[4]);

/* ---- launch tuning (no counterpart in the reference) ---------------------
 * Block and grid sizes of the batch's kernels and the Jacobi solver variant;
 * picked by licenta_gb300/autotune.py.  Block and grid sizes never change
 * results; the solver variant sums the Jacobi corrections differently (all
 * variants stay within the FP64 tolerance). */
typedef struct lc_tuning {
    int32_t traverse_block;        /* threads per block of the BVH traversal (32..256, multiple of 32) */
    int32_t jacobi_block;          /* threads per block of the global-memory Jacobi kernel */
    int32_t narrow_blocks_per_sm;  /* grid of the narrowphase and contact kernels, in blocks per SM */
    int32_t solver_variant;        /* 1, 2 or 3 as lc_batch_options.solver_variant (2, 3 need every cloth on chip) */
    int32_t cluster_size;          /* CTAs per cloth of the on-chip solvers: 4, 8, 16, or 0 to pick */
    int32_t contact_gather;        /* variant 3: 0 = each contact scatters its four corrections (atomics into
                                      the owners' shared memory), 1 = each owned vertex gathers its contact
                                      slots (local atomics only; every contact evaluated per slot) */
} lc_tuning;
lc_status lc_batch_get_tuning(const lc_batch *b, lc_tuning *t);
lc_status lc_batch_set_tuning(lc_batch *b, const lc_tuning *t);

/* The autotuner: every combination of the listed values (first n_* entries
 * of each list) that changes the launches and that the batch accepts is
 * timed with CUDA events over `steps` steps after `warmup` steps, each from
 * the batch's current state (saved on entry, restored before every candidate
 * and on return); the fastest is applied.  Combinations that differ only in a
 * value the chosen solver does not read (the Jacobi block of the on-chip
 * solvers, the cluster size of the global-memory one, the contact mode of
 * solvers other than 3) are timed once.  allow_variants = 0 keeps the batch's
 * solver variant (block, grid and cluster sizes never change results; the
 * variant sums corrections in another order).  NULL space takes
 * lc_default_autotune_space.  The winner goes to *best with its time per
 * step; the first trials_cap trials (configuration, ms per step) to trials,
 * their number to *num_trials.  Allocates one state buffer for the call;
 * waits for the device. */
typedef struct lc_autotune_space {
    int32_t traverse_block[8];       int32_t n_traverse_block;
    int32_t jacobi_block[8];         int32_t n_jacobi_block;
    int32_t narrow_blocks_per_sm[8]; int32_t n_narrow_blocks_per_sm;
    int32_t solver_variant[3];       int32_t n_solver_variant;
    int32_t cluster_size[4];         int32_t n_cluster_size;
    int32_t contact_gather[2];       int32_t n_contact_gather;
} lc_autotune_space;
typedef struct lc_autotune_trial {
    lc_tuning config;
    float ms_per_step;
} lc_autotune_trial;
void lc_default_autotune_space(lc_autotune_space *out);
lc_status lc_batch_autotune(lc_batch *b, const lc_autotune_space *space, int32_t steps, int32_t warmup,
                            int32_t allow_variants, void *stream, lc_tuning *best, float *best_ms,
                            lc_autotune_trial *trials, int32_t trials_cap, int32_t *num_trials);

/* ---- differentiation (no counterpart in the reference) -------------------
 * Per-constraint stiffness of the whole batch in the global constraint order
 * (cloth 0 first; lc_batch_constraint_counts gives each cloth's share), host
 * or device arrays; either may be NULL. */
lc_status lc_batch_set_constraint_stiffness(lc_batch *b, const float *k_stretch, const float *k_bend,
                                            int32_t is_host);

/* The dynamic state every later step reads (x, x_prev, v, running normals,
 * triangle order, wind state) saved to / restored from one device buffer of
 * lc_batch_state_size bytes, on stream: checkpoints of a rollout. */
lc_status lc_batch_state_size(const lc_batch *b, uint64_t *bytes);
lc_status lc_batch_save_state(lc_batch *b, void *dst, void *stream);
lc_status lc_batch_load_state(lc_batch *b, const void *src, void *stream);

/* Reverse pass of one step.  The batch (created with options.adjoint = 1)
 * must hold the state S_n before the step; the call steps it to S_{n+1}
 * exactly as lc_batch_step does, recording the step's solver iterates and
 * decisions, then runs the adjoint with those decisions held fixed (contacts
 * and their weights, ground / LRA activation, the contact terms counted in
 * each iteration; the analytic sphere and the wind's vertex normals are held
 * fixed).  gx, gx_prev, gv: device arrays, 3 floats per vertex packed in cloth
 * order, holding dL/d(x, x_prev, v) of S_{n+1} on entry and of S_n on return.
 * gk_stretch / gk_bend (device, global constraint order, may be NULL)
 * accumulate dL/dk. */
lc_status lc_batch_adjoint_step(lc_batch *b, float *gx, float *gx_prev, float *gv, float *gk_stretch,
                                float *gk_bend, void *stream);

/* lc_batch_adjoint_step for long rollouts whose gradient outgrows float
 * (contact-rich drapes amplify it by up to ~1e14 per 20 steps).  After the
 * reverse pass, every cloth c whose gx / gx_prev / gv has an entry above 2^60
 * in magnitude has all five accumulators (its vertices' entries of gx,
 * gx_prev, gv and its constraints' entries of gk_stretch, gk_bend) multiplied
 * by 2^-60, and exponent[c] (device, one int32 per cloth, zeroed by the
 * caller before the first step) is incremented; the true gradient is the
 * stored value times 2^(60 * exponent[c]).  The reverse pass is linear in
 * its seed, so the scaling is exact while values stay normal. */
lc_status lc_batch_adjoint_step_rescaled(lc_batch *b, float *gx, float *gx_prev, float *gv, float *gk_stretch,
                                         float *gk_bend, int32_t *exponent, void *stream);

/* ----- standalone LBVH (the GenerateBVH2 / ComputeTreeAABBs /
 * GetAABBCollisions chain of Collision/CudaBVH.cu over caller triangles) --- */
typedef struct lc_lbvh lc_lbvh;
/* tri_min/tri_max: 3 * T floats each (device memory); builds Morton codes of
 * the box midpoints, sorts, builds and refits the tree. */
lc_status lc_lbvh_create(int32_t max_triangles, int32_t chunk_size, int32_t morton_mode,
                         lc_lbvh **out);
lc_status lc_lbvh_build(lc_lbvh *h, const float *tri_min, const float *tri_max,
                        int32_t num_triangles, void *stream);
/* Broadphase pairs (leaf i, leaf j), i < j, in the reference's order; pairs
 * are indices into the sorted order.  out_pairs: device memory, 2 * cap u32. */
lc_status lc_lbvh_pairs(lc_lbvh *h, uint32_t *out_pairs, uint64_t cap, uint64_t *count,
                        void *stream);
lc_status lc_lbvh_sorted_ids(lc_lbvh *h, uint32_t *out_ids, void *stream);
/* Intermediate arrays of the last build, in the reference's layouts, into
 * host memory (at most cap elements; the element count goes to *count):
 * LC_DBG_MORTON (sorted codes), LC_DBG_PERM (sorted order), LC_DBG_LEFTS,
 * LC_DBG_RIGHTS, LC_DBG_PARENTS, LC_DBG_RML, LC_DBG_NODE_AABB (the arrays
 * _GenerateBVH2 and ComputeTreeAABBs write, Collision/CudaBVH.cu:128-188) and,
 * after lc_lbvh_pairs, LC_DBG_PAIRS.  Waits for the device; for parity
 * checks, not for a hot loop. */
lc_status lc_lbvh_debug_get(lc_lbvh *h, int32_t what, void *dst, uint64_t cap, uint64_t *count);
lc_status lc_lbvh_destroy(lc_lbvh *h);

/* ---- Object-level broadphase: the Collision::ICollisionMethod family ------
 * Replaces the reference's object-level methods behind ICollisionMethod
 * (Collision/ICollisionMethod.h:15-87: BVH, SweepAndPrune, SpatialGrid,
 * SpatialHashing, Collision/BVH.cpp etc.), which run on the CPU over SceneObjects.
 * Here an object is its axis-aligned box, and lc_broadphase_update (the
 * interface's Update) takes all boxes at once: box_min / box_max, 3 floats per
 * object, in device memory, which must stay valid until the
 * lc_broadphase_test that follows (TestCollision) has returned.  Every method
 * returns the same set, all pairs (a, b), a < b, of objects whose closed boxes
 * overlap (BoundingBox::Collides), with nothing dropped; the methods differ in
 * the work they do:
 *   LC_BP_BRUTE every pair;
 *   LC_BP_SAP   sorted by lower x, each object sweeps forward;
 *   LC_BP_GRID  a uniform grid of cells_per_axis^3 cells over the world box
 *               (boxes outside it are clamped into the border cells);
 *   LC_BP_HASH  an unbounded grid of cell_size cells hashed into table_size
 *               buckets (a power of two);
 *   LC_BP_BVH   a linear BVH over the box centres.
 * The reference's SweepAndPrune keeps its pair set across frames and tests
 * bounding spheres, and its SpatialHashing files objects by points of their
 * boxes; these members all report the exact box-overlap set.  The grid and
 * hash members hold up to max_entries (object, cell) entries (0: 8 per
 * object); more is LC_ERR_CAPACITY_OVERFLOW from lc_broadphase_update.
 * lc_broadphase_test writes at most cap pairs (2 uint32 each, device memory,
 * NULL with cap 0 to count only) and the full count into *count (host),
 * returning LC_ERR_CAPACITY_OVERFLOW when more exist; it synchronizes the
 * stream.  Object add / move / remove (ObjectAdded / ObjectMoved /
 * ObjectRemoved) edit the caller's box array between updates; the host
 * adapters (licenta_gb300.broadphase.CollisionMethod, lc::CollisionMethod in
 * lc_body.hpp) keep that bookkeeping.  lc_broadphase_get_criteria gives the last
 * frame's criteria (Collision/ICollisionMethod.h:61-85): structure and
 * collision times (ms, CUDA events), box tests made and the bytes held. */
enum { LC_BP_BRUTE = 0, LC_BP_SAP = 1, LC_BP_GRID = 2, LC_BP_HASH = 3, LC_BP_BVH = 4 };
typedef struct lc_broadphase_desc {
    int32_t method;
    int32_t max_objects;
    uint64_t max_entries;               /* grid / hash */
    float world_min[3], world_max[3];   /* grid */
    int32_t cells_per_axis;             /* grid, 1..1024 */
    float cell_size;                    /* hash */
    int32_t table_size;                 /* hash */
} lc_broadphase_desc;
typedef struct lc_broadphase_criteria {
    float structure_ms;                 /* last update */
    float collision_ms;                 /* last test */
    uint64_t intersection_tests;        /* box tests of the last test */
    uint64_t pairs;                     /* pairs of the last test */
    uint64_t memory_bytes;              /* device memory held */
} lc_broadphase_criteria;
typedef struct lc_broadphase lc_broadphase;
lc_status lc_broadphase_create(const lc_broadphase_desc *desc, lc_broadphase **out);
lc_status lc_broadphase_update(lc_broadphase *b, const float *box_min, const float *box_max, int32_t num_objects,
                               void *stream);
/* The boxes from host memory, copied into the handle's own device buffers
 * (which the following test reads). */
lc_status lc_broadphase_update_host(lc_broadphase *b, const float *box_min, const float *box_max,
                                    int32_t num_objects, void *stream);
lc_status lc_broadphase_test(lc_broadphase *b, uint32_t *pairs, uint64_t cap, uint64_t *count, void *stream);
/* The same into host memory (through a device staging buffer the handle grows
 * to the largest pair count it has seen). */
lc_status lc_broadphase_test_host(lc_broadphase *b, uint32_t *pairs, uint64_t cap, uint64_t *count,
                                  void *stream);
lc_status lc_broadphase_get_criteria(lc_broadphase *b, lc_broadphase_criteria *out);
lc_status lc_broadphase_destroy(lc_broadphase *b);

/* Physics::PrimitiveContact (Physics/Structs.h:106-129) as the reference's
 * contact tests leave it: vertex ids (VF: the vertex, then the face; EE: the
 * two edges), weights, time of contact and unit normal. */
typedef struct lc_primitive_contact {
    int32_t v[4];
    float w[4];
    float t;
    float n[3];
} lc_primitive_contact;

/* ----- impulse response ------------------------------------------------------
 * CudaDeformableBody::SolveCollisions (Physics/CudaDeformableBody.cpp:523-548):
 * DeformableUtils::CreateImpulses then ApplyImpulses
 * (Collision/CudaCollisionResponse.cu:11-300).  Every contact gives an
 * impulse along its normal from the penetration h - n.(sum w_i x_prev_i) and
 * the relative normal velocity, clamped and spread over its four vertices by
 * their weights; each vertex averages the impulses it received (the
 * reference's grid quirk kept: of the vertices with impulses, ranked by id,
 * only the first ceil(contacts / 256) * 256 are accumulated); then every
 * vertex that is not fixed takes v += impulse / vertex_mass and
 * x = x_prev + v timestep.  x (out), x_prev, v (in/out): device arrays of 3
 * floats per vertex; fixed: device flags; vf, ee: device contacts (as
 * lc_narrowphase_run writes them; VF first in the impulse order).  Stiffness
 * is the reference's kStretch, vertex_mass objectMass / vertex count.
 * Allocates its scratch in stream order (cudaMallocAsync) and, when there are
 * contacts, waits for the stream once to validate their vertex ids. */
lc_status lc_solve_collisions(float *x, const float *x_prev, float *v, const uint8_t *fixed, int32_t num_vertices,
                              const lc_primitive_contact *vf, uint64_t num_vf, const lc_primitive_contact *ee,
                              uint64_t num_ee, float stiffness, float vertex_mass, float timestep, float thickness,
                              void *stream);

/* ----- narrowphase on caller data ----------------------------------------
 * DeformableUtils::CreateTriangleTests followed by
 * DeformableUtils::CCDTriangleTests (mode LC_NARROW_CCD) or DCDTriangleTests
 * (mode LC_NARROW_DCD) (Collision/CudaCollisionDetection.cuh:28-46,
 * .cu:6-51, 191-221 and 223-283): for every broadphase pair (triangle i,
 * triangle j) the 6 vertex-face and 9 edge-edge candidates of
 * Collision/CudaCollisionDetection.cu:101-187 that the triangles' ownership
 * bits and the shared-vertex sanity checks keep, then
 *   CCD: the feature AABB cull on the swept vertex boxes of x and x_prev and
 *        the continuous tests of Collision/CudaPrimitiveTests.cu:96-238 on
 *        x_prev and v over one timestep (t = the hit's coplanarity time
 *        times the timestep);
 *   DCD: one TestVF / TestEE at x_prev (Collision/CudaPrimitiveTests.cu:
 *        21-94, the positions HandleCollisionsDiscrete passes), no cull (t as
 *        the tests leave it: 0, or -1 where TestEE does not write it).
 * Contacts come out in the reference's order (pair, then candidate slot), as
 * PrimitiveContact records.
 *
 * A handle owns the work buffers, sized for at most max_vertices,
 * max_triangles and max_pairs; candidate_capacity (per kind) and
 * contact_capacity (per kind) take 0 for the defaults of lc_batch_options.
 * lc_narrowphase_run takes device arrays: x, x_prev, v (3 floats per vertex:
 * predicted positions, previous positions, velocities; DCD reads x_prev
 * only, x and v may be NULL), triangles (3 vertex ids each), features (one
 * ownership byte per triangle: bits 5..3 own its vertices v1..v3, bits 2..0
 * its edges v1v2, v2v3, v3v1, as Physics::CudaTriangle::m_features; NULL
 * owns everything), pairs (2 triangle indices each, i < j as the traversal
 * emits them) and the contact outputs (device arrays of vf_cap / ee_cap
 * records).  The full contact counts go to *vf_count / *ee_count (host); more
 * contacts than a cap return LC_ERR_CAPACITY_OVERFLOW with the first cap
 * written.  An index out of range returns LC_ERR_INVALID_ARG (checked on the
 * device; the offending triangle or pair takes no part).  The call waits for
 * its stream. */
enum { LC_NARROW_CCD = 0, LC_NARROW_DCD = 1 };
typedef struct lc_narrowphase lc_narrowphase;
lc_status lc_narrowphase_create(int32_t max_vertices, int32_t max_triangles, uint64_t max_pairs,
                                uint64_t candidate_capacity, uint64_t contact_capacity, lc_narrowphase **out);
lc_status lc_narrowphase_run(lc_narrowphase *h, int32_t mode, const float *x, const float *x_prev, const float *v,
                             int32_t num_vertices, const uint32_t *triangles, const uint8_t *features,
                             int32_t num_triangles, const uint32_t *pairs, uint64_t num_pairs, float thickness,
                             float timestep, lc_primitive_contact *vf_out, uint64_t vf_cap,
                             lc_primitive_contact *ee_out, uint64_t ee_cap, uint64_t *vf_count, uint64_t *ee_count,
                             void *stream);
lc_status lc_narrowphase_destroy(lc_narrowphase *h);

/* ----- allocation-free LBVH query ---------------------------------------
 * No counterpart in the reference.  The same query as lc_lbvh_create +
 * lc_lbvh_build + lc_lbvh_pairs (+ lc_lbvh_sorted_ids), for callers that
 * cannot allocate device memory: code under a custom allocator or a fixed
 * memory pool, plugins in a process that owns the device memory, real-time
 * loops where an allocation and its implicit synchronisation are not allowed.
 * Every intermediate buffer lives in one scratch array built into the library
 * (about 0.9 MB of device memory on each GPU that loads it, kept until the
 * process exits), so sizes are limited to LC_LBVH_STATIC_MAX_TRIANGLES
 * triangles and LC_LBVH_STATIC_MAX_CHUNK pairs per leaf; larger requests
 * return LC_ERR_INVALID_ARG.  The caller passes the boxes (device memory,
 * 3 * n floats each), the pair output (device memory, 2 * cap u32; pairs
 * beyond cap are not written and the call returns
 * LC_ERR_CAPACITY_OVERFLOW with the full number in *count), *count (host) and
 * optionally the sorted triangle ids (device memory, n u32).  The first call
 * on a device looks up the scratch address and keeps it for the rest of the
 * process: after a cudaDeviceReset of that device the entry point must not be
 * called on it again.  Every call ends by copying the pair count to the host
 * and waiting for its stream, so it cannot be issued on a stream that is
 * being captured.  All calls share the scratch array and keep nothing between
 * calls that they rely on; calls that overlap on the GPU race and must be
 * serialised by the caller. */
#define LC_LBVH_STATIC_MAX_TRIANGLES 2048
#define LC_LBVH_STATIC_MAX_CHUNK 64
lc_status lc_lbvh_pairs_static(const float *tri_min, const float *tri_max, int32_t num_triangles,
                               int32_t chunk_size, int32_t morton_mode, uint32_t *out_pairs, uint64_t cap,
                               uint64_t *count, uint32_t *out_sorted_ids, void *stream);

const char *lc_last_error_string(void);
const char *lc_status_string(lc_status s);

#ifdef __cplusplus
}
#endif

#endif /* LC_LC_H */
