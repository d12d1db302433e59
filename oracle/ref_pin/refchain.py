"""The reference's collision chain, run with the reference's own kernels.

TEST INFRASTRUCTURE ONLY: generates the golden vectors that pin the oracle
(tests/golden/make_golden.py).  Nothing in the engine imports this module.

oracle/_ref/ref_kernels.cubin (built by oracle/ref_pin/build_ref.py from the
reference's sources) is loaded through the CUDA driver API (ctypes on
libcuda) and its kernels are launched in the order and with the launch
shapes of the reference's host code:

  FeatureList::UpdateFeatureAABBs       Collision/FeatureList.cu:57-70
  DeformableUtils::UpdateTrianglesContinuous
                                        Physics/CudaDeformableUtils.cu:107-118
  DeformableUtils::SortMortons          Physics/CudaDeformableUtils.cu:346-349
  CudaBVH::GenerateBVH2                 Collision/CudaBVH.cu:152-161
  CudaBVH::ComputeTreeAABBs             Collision/CudaBVH.cu:115-126
  CudaDeformableBody::CreateTriangleTests
                                        Physics/CudaDeformableBody.cpp:497-521
  DeformableUtils::CreateTriangleTests  Collision/CudaCollisionDetection.cu:6-51
  DeformableUtils::CCDTriangleTests     Collision/CudaCollisionDetection.cu:223-283

and, for the other half of the step, the prediction (PBDStepExternal with
UpdateVertexNormals), the solver (PBDStepSolver, PBDStepIntegration),
friction (ApplyFriction), the impulse response (SolveCollisions) and the
discrete triangle tests of HandleCollisionsDiscrete.

Two host-side steps stand in for the reference's CUB calls: the stable radix
sort of (Morton code, triangle) pairs (Core/CubWrappers.cuh:141-156) is a
stable host sort of the same keys, whose result is unique, and
cub::DeviceSelect::Flagged (Core/CubWrappers.cuh:84-88) is an order-preserving
host compaction.  Device buffers are torch tensors; launches go to torch's
current stream in torch's (primary) context.

Before each kernel whose memory accesses depend on data, the inputs are
checked on the host so that every access stays in bounds: the triangle
indices, no run of three equal Morton codes (there the reference's parents[]
has a write race and may leave a node without a parent, which its refit
would then follow; the two triangles of a grid quad share a box and so a
code, which its tie-break handles), a complete hierarchy in which every node
has exactly one parent, and a depth well inside the traversal's 64-entry
stack (Collision/CudaBVH.cu:38).
"""
from __future__ import annotations

import ctypes as C
import gzip
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent.parent / "_ref" / "ref_kernels.cubin"
THREADS = 256  # CudaUtils::THREADS_PER_BLOCK (Core/CudaUtils.cuh:87)
MAX_DEPTH = 56

# kernel key -> unqualified name in the reference
KERNELS = {
    "particle_aabbs": "UpdateParticleAABBs",
    "edge_aabbs": "UpdateEdgeAABBs",
    "tri_update": "_UpdateTrianglesContinuous",
    "gen_bvh": "_GenerateBVH2",
    "refit": "ComputeTreeAABBs",
    "traverse": "_GetAABBCollisions",
    "tri_tests": "CreateTriangleTests",
    "feature_aabb": "FeatureAABBTests",
    "ccd": "CCDTriangleTests",
    # PBDStepSolver and _FinalUpdate (Physics/CudaPBD.cu:632-660, :929-940)
    "ground_create": "_CreateGroundConstraints",
    "lra_create": "_CreateLRAConstraints",
    "sphere_create": "_CreateSphereConstraints",
    "ground_apply": "_ApplyGroundCorrections",
    "lra_apply": "_ApplyLRACorrections",
    "static_project": "_ProjectStaticConstraints",
    "static_project_tri": "_ProjectStaticConstraintsTriBend",
    "static_apply": "_ApplyStaticCorrections",
    "dyn_project": "_ProjectDynamicConstraints",
    "dyn_apply": "_ApplyDynamicCorrections",
    "sphere_apply": "_ApplySphereCorrections",
    "final_correction": "FinalCorrectionStep",
    "final_update": "_FinalUpdate",
    # FixedUpdate's world clamp (Physics/CudaDeformableBody.cpp:616)
    "world_clamp": "_WorldConstraints",
    # PBDStepExternal (Physics/CudaPBD.cu:610-630) with DampVelocities (:411-458)
    "external_forces": "ApplyExternalForces",
    "global_damp": "GlobalVelDamp",
    "xm_vm": "ComputeXMVMs",
    "ang_mom": "ComputeL",
    "inertia": "ComputeIs",
    "update_vels": "UpdateVels",
    "euler": "ExplicitEuler",
    # SolveCollisions (Physics/CudaDeformableBody.cpp:523-548) with
    # Collision/CudaCollisionResponse.cu:11-300, and the discrete tests of
    # HandleCollisionsDiscrete (Collision/CudaPrimitiveTests.cu:21-94)
    "create_impulses": "_CreateImpulses",
    "accumulate_impulses": "AccumulateImpulses",
    "apply_impulses": "ApplyImpulses",
    "dcd_tests": "DCDTriangleTests",
    # DeformableUtils::UpdateVertexNormals (Physics/CudaDeformableUtils.cu:190-249)
    "create_vns": "CreateVNs",
    "accumulate_vns": "AccumulateVNs",
    "normalize_vns": "NormalizeVNs",
    # CudaPBD::ApplyFriction (Physics/CudaPBD.cu:770-833)
    "damp_rigid": "_DampVelRigid",
    "apply_friction": "_ApplyFriction",
    "accumulate_friction": "_AccumulateFriction",
    "final_friction": "FinalFrictionStep",
}


class Float3(C.Structure):
    """CUDA float3 passed by value."""
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        P = C.c_void_p
        sig = {
            "cuCtxGetCurrent": [C.POINTER(P)],
            "cuModuleLoadData": [C.POINTER(P), P],
            "cuModuleGetFunctionCount": [C.POINTER(C.c_uint), P],
            "cuModuleEnumerateFunctions": [C.POINTER(P), C.c_uint, P],
            "cuFuncGetName": [C.POINTER(C.c_char_p), P],
            "cuLaunchKernel": [P, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, P,
                               C.POINTER(P), C.POINTER(P)],
            "cuModuleUnload": [P],
        }
        for name, args in sig.items():
            f = getattr(self.cu, name)
            f.argtypes = args
            f.restype = C.c_int

    def __call__(self, name, *args):
        rc = getattr(self.cu, name)(*args)
        if rc != 0:
            raise RuntimeError(f"{name} failed with CUresult {rc}")


class RefKernels:
    """The reference kernels of the collision chain, loaded from the cubin."""

    def __init__(self, cubin: Path = CUBIN):
        import torch
        gz = Path(str(cubin) + ".gz")
        if cubin.exists():
            image = cubin.read_bytes()
        elif gz.exists():
            image = gzip.decompress(gz.read_bytes())
        else:
            raise FileNotFoundError(f"{cubin} is missing: run python -m oracle.ref_pin.build_ref")
        torch.cuda.init()
        torch.empty(1, device="cuda")  # make torch's primary context current
        self.torch = torch
        self.drv = _Driver()
        ctx = C.c_void_p()
        self.drv("cuCtxGetCurrent", C.byref(ctx))
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self._image = C.create_string_buffer(image)
        self.mod = C.c_void_p()
        self.drv("cuModuleLoadData", C.byref(self.mod), C.cast(self._image, C.c_void_p))
        n = C.c_uint()
        self.drv("cuModuleGetFunctionCount", C.byref(n), self.mod)
        funcs = (C.c_void_p * n.value)()
        self.drv("cuModuleEnumerateFunctions", funcs, n.value, self.mod)
        names = {}
        for f in funcs:
            s = C.c_char_p()
            self.drv("cuFuncGetName", C.byref(s), f)
            names[s.value.decode()] = f
        self.names = sorted(names)
        self.fn = {}
        for key, ident in KERNELS.items():
            tag = f"{len(ident)}{ident}"  # the identifier as it appears in a mangled name
            hits = [m for m in names if tag in m]
            if len(hits) != 1:
                raise RuntimeError(f"kernel {ident}: {len(hits)} matches in the cubin: {hits}")
            self.fn[key] = names[hits[0]]

    def launch(self, key: str, n_threads: int, *args, block: int = THREADS, blocks: int | None = None) -> None:
        """Launches a reference kernel with `block` threads per block over
        ceil(n_threads / THREADS) blocks (the reference's own grid size),
        or `blocks` when given."""
        if n_threads <= 0:
            return
        vals = []
        for a in args:
            if isinstance(a, (C._SimpleCData, C.Structure)):
                vals.append(a)
            elif hasattr(a, "data_ptr"):
                vals.append(C.c_void_p(a.data_ptr()))
            elif a is None:
                vals.append(C.c_void_p(0))
            else:
                raise TypeError(f"argument {a!r}: pass a ctypes scalar, a tensor or None")
        params = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        if n_threads >= 1 << 31:
            raise ValueError("launch too large")
        stream = C.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        if blocks is None:
            blocks = (n_threads + THREADS - 1) // THREADS
        self.drv("cuLaunchKernel", self.fn[key], blocks, 1, 1, block, 1, 1, 0, stream, params, None)

    # ------------------------------------------------------------------
    def predict(self, x, x_prev, v, vn, masses, *, gravity, wind, dt: float, k_global: float,
                k_damp: float) -> dict:
        """CudaPBD::PBDStepExternal (Physics/CudaPBD.cu:610-630) with the
        reference's own kernels: ApplyExternalForces, then DampVelocities
        (:411-458: GlobalVelDamp, ComputeXMVMs, ComputeL, ComputeIs,
        UpdateVels), then ExplicitEuler.

        x, x_prev, v, vn: (V, 3) float32 state before the step (positions
        after the previous step's world clamp, previous positions, velocities,
        running vertex normals); masses: (V,) float32 (Physics/
        CudaDeformableBody.cpp:80-82); wind: the current wind vector
        m_crtWindDir of this step (after the host update of :613-619, which
        the restatement draws from a seeded generator in place of
        std::rand()).  Returns the predicted positions ``x`` and velocities
        ``v`` and the damping's intermediate values.

        The host work between the kernels restates DampVelocities' host code:
        the six CubWrap::ReduceSum calls (Core/CubWrappers.cuh:55-75) are
        float sums, taken here in float64 and rounded once to float32 (CUB
        sums in another order; any order differs from this by at most about
        V float roundings of the total), and glm::inverse of the float 3x3
        inertia (Dependencies/glm/detail/type_mat3x3.inl:37-56, the cofactor
        matrix over the determinant) with the matrix-vector product of glm's
        column-major mat3 (the same file's operator*), in float32."""
        torch = self.torch
        f32 = np.float32
        x = np.ascontiguousarray(x, f32)
        V = x.shape[0]
        arrs = [np.ascontiguousarray(a, f32).reshape(V, 3) for a in (x_prev, v, vn)]
        m = np.ascontiguousarray(masses, f32).reshape(V)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        d_x, d_xp, d_v, d_vn, d_m = dev(x), dev(arrs[0]), dev(arrs[1]), dev(arrs[2]), dev(m)
        aux1 = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        aux2 = torch.zeros_like(aux1)
        n = C.c_int(V)
        f3 = lambda a: Float3(*[float(f32(q)) for q in a])

        def rsum(t):  # CubWrap::ReduceSum of float / float3 values
            a = t.cpu().numpy().astype(np.float64)
            return a.sum(axis=0).astype(f32)

        self.launch("external_forces", V, n, d_v, d_vn, f3(gravity), f3(wind), C.c_float(dt))
        self.launch("global_damp", V, n, d_v, C.c_float(k_global))
        mass_sum = f32(rsum(d_m))
        self.launch("xm_vm", V, n, d_x, d_v, d_m, aux1, aux2)
        torch.cuda.synchronize()
        xcm = (rsum(aux1) / mass_sum).astype(f32)
        vcm = (rsum(aux2) / mass_sum).astype(f32)
        self.launch("ang_mom", V, n, d_x, f3(xcm), aux2, aux1)
        torch.cuda.synchronize()
        L = rsum(aux1)
        self.launch("inertia", V, n, d_x, f3(xcm), d_m, aux1, aux2)
        torch.cuda.synchronize()
        i1, i2 = rsum(aux1), rsum(aux2)
        # glm::mat3 I(col0, col1, col2) of Physics/CudaPBD.cu:447-449
        I = np.array([[i1[1] + i1[2], i2[0], i2[1]],
                      [i2[0], i1[0] + i1[2], i2[2]],
                      [i2[1], i2[2], i1[0] + i1[1]]], dtype=f32)  # I[col][row]
        omega = _glm_mat3_mul(_glm_inverse3(I), L)
        self.launch("update_vels", V, n, d_x, f3(omega), f3(xcm), f3(vcm), C.c_float(k_damp), d_v)
        self.launch("euler", V, n, d_xp, d_v, d_x, C.c_float(dt))
        torch.cuda.synchronize()
        return dict(x=d_x.cpu().numpy(), v=d_v.cpu().numpy(), mass_sum=mass_sum, xcm=xcm, vcm=vcm, L=L,
                    inertia=I, omega=omega)

    def vertex_normals(self, x, x_prev, triangles, vn, thickness: float) -> np.ndarray:
        """DeformableUtils::UpdateVertexNormals (Physics/CudaDeformableUtils.cu:
        190-249) as FixedUpdate runs it (Physics/CudaDeformableBody.cpp:
        562-567): _UpdateTrianglesContinuous writes each triangle's unit face
        normal from the predicted positions x into the triangle array (still
        in its pre-sort slot order), CreateVNs copies it to the triangle's
        three vertices, AccumulateVNs adds them into the running normals vn
        (never zeroed) with float atomicAdd and NormalizeVNs renormalises.
        x, x_prev: (V, 3) float32; triangles: (T, 3) vertex ids in slot
        order; vn: (V, 3) running normals before the step.  Returns the
        running normals after it.  The atomic sums' order is the GPU's, so
        results agree with an ordered sum up to float rounding."""
        torch = self.torch
        f32 = np.float32
        x = np.ascontiguousarray(x, f32)
        V = x.shape[0]
        tris = np.ascontiguousarray(triangles, np.int64)
        T = tris.shape[0]
        if T < 1 or tris.min() < 0 or tris.max() >= V:
            raise ValueError("triangle index out of range")
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        tri = np.zeros((T, 7), dtype=np.int32)
        tri[:, :3] = tris
        d_tri = dev(tri)
        nodes = 2 * T - 1
        mort = torch.zeros(T, dtype=torch.int64, device="cuda")
        nmin = torch.zeros((nodes, 3), dtype=torch.float32, device="cuda")
        nmax = torch.zeros_like(nmin)
        self.launch("tri_update", T, C.c_int(T), dev(x), dev(np.ascontiguousarray(x_prev, f32)), d_tri, mort,
                    nmin, nmax, C.c_float(thickness))
        raw = torch.zeros((3 * T, 3), dtype=torch.float32, device="cuda")
        raw_ids = torch.zeros(3 * T, dtype=torch.int32, device="cuda")
        acc = dev(np.ascontiguousarray(vn, f32).reshape(V, 3))
        self.launch("create_vns", T, C.c_int(T), d_tri, raw, raw_ids)
        self.launch("accumulate_vns", 3 * T, C.c_int(3 * T), raw, raw_ids, acc)
        self.launch("normalize_vns", V, C.c_int(V), acc)
        torch.cuda.synchronize()
        return acc.cpu().numpy()

    # ------------------------------------------------------------------
    def collide(self, x, x_prev, v, triangles, features, thickness: float, dt: float, chunk: int = 64,
                prefill: dict | None = None) -> dict:
        """One pass of the reference's collision stages.

        x, x_prev, v: (V, 3) float32 predicted positions, previous positions
        and velocities; triangles: (T, 3) vertex ids in the current slot
        order; features: (T,) feature bytes of those triangles.  Returns the
        sorted Morton codes, the sort order (new slot -> old slot), the
        hierarchy, node boxes, rightmost leaves, broadphase pairs and the
        compacted VF / EE contacts.

        ComputeTreeAABBs (Collision/CudaBVH.cu:128-149) releases a parent with
        atomicExch but writes the child's box and rightmost leaf without a
        fence, so the second arrival at a node can read a child's box before
        it is visible (stale zeros, or a float3 half written).  ``prefill``
        (internal-node boxes ``node_min`` / ``node_max`` of shape (2T-1, 3)
        and ``rmll`` / ``rmlr`` of shape (T-1,)) seeds the internal entries
        before the refit runs: the kernel still computes and writes every
        internal node, but a read that races now returns the seeded value.
        Seeded with the restatement's values, an output node equal to the
        seed shows that the reference's formula, applied to children that
        already agree, gives the same value (induction from the leaves,
        which the refit never writes).
        """
        torch = self.torch
        f32, i32 = np.float32, np.int32
        x = np.ascontiguousarray(x, f32)
        xp = np.ascontiguousarray(x_prev, f32)
        vel = np.ascontiguousarray(v, f32)
        tris = np.ascontiguousarray(triangles, np.int64)
        V, T = x.shape[0], tris.shape[0]
        if T < 2 or V < 3 or V > 8192:
            raise ValueError("need 2 <= T and 3 <= V <= 8192")
        if tris.min() < 0 or tris.max() >= V:
            raise ValueError("triangle index out of range")
        chunk = min(chunk, T)  # Physics/CudaDeformableBody.cpp:233
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        h = C.c_float(thickness)

        # Collision/FeatureList.cu:12-55 — unique edges and the V x V edge map.
        emap = np.full(V * V, -1, dtype=i32)
        e1, e2 = [], []
        for t in range(T):
            for j in range(3):
                a, b = int(tris[t, j]), int(tris[t, (j + 1) % 3])
                lo, hi = min(a, b), max(a, b)
                if emap[lo * V + hi] == -1:
                    emap[lo * V + hi] = len(e1)
                    e1.append(lo)
                    e2.append(hi)
        E = len(e1)
        d_x, d_xp, d_v = dev(x), dev(xp), dev(vel)
        d_emap, d_e1, d_e2 = dev(emap), dev(np.array(e1, i32)), dev(np.array(e2, i32))
        pmin = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        pmax = torch.zeros_like(pmin)
        emin = torch.zeros((E, 3), dtype=torch.float32, device="cuda")
        emax = torch.zeros_like(emin)
        self.launch("particle_aabbs", V, C.c_int(V), d_x, d_xp, h, pmin, pmax)
        self.launch("edge_aabbs", E, C.c_int(E), pmin, pmax, d_e1, d_e2, h, emin, emax)

        # Physics/Structs.h:176-188 — CudaTriangle {int v1, v2, v3; char
        # features; float3 normal} = 28 bytes, as 7 int32 words.
        tri = np.zeros((T, 7), dtype=i32)
        tri[:, :3] = tris
        tri[:, 3] = np.asarray(features, np.uint8).astype(i32)
        d_tri = dev(tri)
        nodes = 2 * T - 1
        mort = torch.zeros(T, dtype=torch.int64, device="cuda")
        nmin = torch.zeros((nodes, 3), dtype=torch.float32, device="cuda")
        nmax = torch.zeros_like(nmin)
        self.launch("tri_update", T, C.c_int(T), d_x, d_xp, d_tri, mort, nmin, nmax, h)
        torch.cuda.synchronize()

        # Stable sort of the codes with the triangle payload; the boxes stay.
        keys = mort.cpu().numpy().view(np.uint64)
        order = np.argsort(keys, kind="stable")
        skeys = keys[order]
        if skeys.size > 2 and np.any((skeys[2:] == skeys[1:-1]) & (skeys[1:-1] == skeys[:-2])):
            raise ValueError("three equal Morton codes in a row: the reference hierarchy would race")
        tri_sorted = d_tri.cpu().numpy()[order]  # the payload carries the new face normals
        d_tri = dev(tri_sorted)
        d_keys = dev(skeys.view(np.int64))

        In = T - 1
        lefts = torch.zeros(In, dtype=torch.int32, device="cuda")
        rights = torch.zeros_like(lefts)
        parents = torch.zeros(nodes, dtype=torch.int32, device="cuda")
        visited = torch.zeros(In, dtype=torch.int32, device="cuda")
        self.launch("gen_bvh", In, C.c_int(In), d_keys, lefts, rights, parents, visited)
        torch.cuda.synchronize()
        L, R, Pa = lefts.cpu().numpy(), rights.cpu().numpy(), parents.cpu().numpy()
        depth = _check_tree(L, R, Pa, T)
        if depth > MAX_DEPTH:
            raise ValueError(f"hierarchy depth {depth} too close to the 64-entry traversal stack")

        rmll = torch.zeros(In, dtype=torch.int32, device="cuda")
        rmlr = torch.zeros_like(rmll)
        if prefill is not None:
            nmin[:In] = torch.from_numpy(np.ascontiguousarray(prefill["node_min"][:In], f32)).cuda()
            nmax[:In] = torch.from_numpy(np.ascontiguousarray(prefill["node_max"][:In], f32)).cuda()
            rmll.copy_(torch.from_numpy(np.ascontiguousarray(prefill["rmll"], i32)))
            rmlr.copy_(torch.from_numpy(np.ascontiguousarray(prefill["rmlr"], i32)))
        self.launch("refit", T, C.c_int(T), lefts, rights, parents, visited, nmin, nmax, rmll, rmlr)

        cols = torch.zeros((T * chunk, 2), dtype=torch.int32, device="cuda")
        flags = torch.zeros(T * chunk, dtype=torch.uint8, device="cuda")
        self.launch("traverse", T, C.c_int(T), lefts, rights, nmin, nmax, rmll, rmlr, cols, flags,
                    C.c_int(chunk), C.c_uint64(1))
        torch.cuda.synchronize()
        pairs = cols[flags.bool()].contiguous()
        P = pairs.shape[0]
        if P and (int(pairs.min()) < 0 or int(pairs.max()) >= T):
            raise RuntimeError("pair index out of range")

        out = dict(morton=skeys, order=order.astype(i32), lefts=L, rights=R, parents=Pa,
                   node_min=nmin.cpu().numpy(), node_max=nmax.cpu().numpy(),
                   rmll=rmll.cpu().numpy(), rmlr=rmlr.cpu().numpy(), pairs=pairs.cpu().numpy())
        if P == 0:
            out["vf"] = out["ee"] = np.zeros((0, 12), i32)
            return out

        # PrimitiveContact {int v1..v4; float w1..w4, t; float3 n} = 12 words.
        vf = torch.zeros((6 * P, 12), dtype=torch.int32, device="cuda")
        ee = torch.zeros((9 * P, 12), dtype=torch.int32, device="cuda")
        vff = torch.ones(6 * P, dtype=torch.uint8, device="cuda")
        eef = torch.ones(9 * P, dtype=torch.uint8, device="cuda")
        self.launch("tri_tests", P, C.c_int(P), d_tri, pairs, vf, vff, ee, eef)
        self.launch("feature_aabb", 15 * P, C.c_int(V), pmin, pmax, d_emap, d_e1, d_e2, emin, emax, None, None, None,
                    vf, vff, C.c_uint64(6 * P), ee, eef, C.c_uint64(9 * P))
        torch.cuda.synchronize()
        vf = vf[vff.bool()].contiguous()
        ee = ee[eef.bool()].contiguous()
        for c in (vf, ee):
            if c.shape[0] and (int(c[:, :4].min()) < 0 or int(c[:, :4].max()) >= V):
                raise RuntimeError("candidate vertex out of range")
        nvf, nee = vf.shape[0], ee.shape[0]
        vff = torch.zeros(max(nvf, 1), dtype=torch.uint8, device="cuda")
        eef = torch.zeros(max(nee, 1), dtype=torch.uint8, device="cuda")
        self.launch("ccd", nvf + nee, d_tri, d_xp, d_v, vf, vff, C.c_uint64(nvf), ee, eef, C.c_uint64(nee),
                    h, C.c_float(dt))
        torch.cuda.synchronize()
        out["vf"] = vf[vff[:nvf].bool()].cpu().numpy()
        out["ee"] = ee[eef[:nee].bool()].cpu().numpy()
        return out

    # ------------------------------------------------------------------
    def solve_collisions(self, x, x_prev, v, fixed, vf, ee, *, stiffness: float, vertex_mass: float, dt: float,
                         thickness: float) -> dict:
        """CudaDeformableBody::SolveCollisions with the reference's kernels:
        CreateImpulses (Collision/CudaCollisionResponse.cu:11-140: the
        accumulators cleared, _CreateImpulses over the contacts, the CUB
        stable sort by vertex id, run-length encoding and exclusive sum of the
        counts on the host, AccumulateImpulses launched over the contacts'
        grid as the reference launches it) then ApplyImpulses (:262-300).
        x, x_prev, v: (V, 3) float32 positions, previous positions and
        velocities (the reference passes m_dPrevPositions as the impulses'
        positions; a fixed vertex keeps x); fixed: (V,) flags; vf, ee: (N, 12) int32
        PrimitiveContact records.  Returns the new positions ``x``, the
        velocities ``v`` and the accumulated impulses."""
        torch = self.torch
        f32, i32 = np.float32, np.int32
        xp = np.ascontiguousarray(x_prev, f32)
        V = xp.shape[0]
        vel = np.ascontiguousarray(v, f32).reshape(V, 3)
        vf = np.ascontiguousarray(vf, i32).reshape(-1, 12)
        ee = np.ascontiguousarray(ee, i32).reshape(-1, 12)
        for c in (vf, ee):
            if len(c) and (c[:, :4].min() < 0 or c[:, :4].max() >= V):
                raise ValueError("contact vertex out of range")
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        d_xp, d_v = dev(xp), dev(vel)
        d_x = dev(np.ascontiguousarray(x, f32).reshape(V, 3))
        acc = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        nvf, nee = len(vf), len(ee)
        C_ = nvf + nee
        if C_:
            ids = torch.zeros(4 * C_, dtype=torch.int32, device="cuda")
            vals = torch.zeros((4 * C_, 3), dtype=torch.float32, device="cuda")
            flags = torch.zeros(4 * C_, dtype=torch.uint8, device="cuda")
            self.launch("create_impulses", C_, d_xp, d_v, dev(vf if nvf else np.zeros((1, 12), i32)), C.c_uint64(nvf),
                        dev(ee if nee else np.zeros((1, 12), i32)), C.c_uint64(nee), ids, vals, flags,
                        C.c_float(stiffness), C.c_float(vertex_mass), C.c_float(dt), C.c_float(thickness))
            torch.cuda.synchronize()
            h_ids = ids.cpu().numpy().view(np.uint32)
            order = np.argsort(h_ids, kind="stable")
            sids = h_ids[order]
            starts = np.flatnonzero(np.r_[True, sids[1:] != sids[:-1]]).astype(i32)
            runs = len(starts)
            blocks = (C_ + THREADS - 1) // THREADS  # the contacts' grid (:132-136)
            self.launch("accumulate_impulses", runs, C.c_int(runs), dev(sids[starts].view(i32)), dev(starts),
                        dev(vals.cpu().numpy()[order]), C.c_uint64(4 * C_), acc, blocks=blocks)
        self.launch("apply_impulses", V, C.c_int(V), d_x, d_xp, d_v, acc, dev(np.asarray(fixed) != 0),
                    C.c_float(vertex_mass), C.c_float(dt))
        torch.cuda.synchronize()
        return dict(x=d_x.cpu().numpy(), v=d_v.cpu().numpy(), impulses=acc.cpu().numpy())

    def dcd(self, positions, triangles, features, pairs, thickness: float) -> dict:
        """HandleCollisionsDiscrete's tests (Physics/CudaDeformableBody.cpp:
        419-438) on given broadphase pairs: CreateTriangleTests
        (Collision/CudaCollisionDetection.cu:6-189) then DCDTriangleTests
        (Collision/CudaPrimitiveTests.cu:21-94: the sanity checks and TestVF /
        TestEE at the positions, no feature AABB cull) and the compaction.
        positions: (V, 3) float32 (the reference passes m_dPrevPositions);
        triangles: (T, 3) in the slot order the pairs index; features: (T,)
        their ownership bytes; pairs: (P, 2).  Returns the VF / EE contacts
        as (N, 12) PrimitiveContact records."""
        torch = self.torch
        f32, i32 = np.float32, np.int32
        pos = np.ascontiguousarray(positions, f32)
        V = pos.shape[0]
        tris = np.ascontiguousarray(triangles, np.int64).reshape(-1, 3)
        T = tris.shape[0]
        pr = np.ascontiguousarray(pairs, i32).reshape(-1, 2)
        P = pr.shape[0]
        if tris.min() < 0 or tris.max() >= V or (P and (pr.min() < 0 or pr.max() >= T)):
            raise ValueError("index out of range")
        if P == 0:
            return dict(vf=np.zeros((0, 12), i32), ee=np.zeros((0, 12), i32))
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        tri = np.zeros((T, 7), dtype=i32)
        tri[:, :3] = tris
        tri[:, 3] = np.asarray(features, np.uint8).astype(i32)
        vf = torch.zeros((6 * P, 12), dtype=torch.int32, device="cuda")
        ee = torch.zeros((9 * P, 12), dtype=torch.int32, device="cuda")
        vff = torch.ones(6 * P, dtype=torch.uint8, device="cuda")
        eef = torch.ones(9 * P, dtype=torch.uint8, device="cuda")
        self.launch("tri_tests", P, C.c_int(P), dev(tri), dev(pr), vf, vff, ee, eef)
        self.launch("dcd_tests", 15 * P, dev(tri), dev(pos), vf, vff, C.c_uint64(6 * P), ee, eef, C.c_uint64(9 * P),
                    C.c_float(thickness))
        torch.cuda.synchronize()
        return dict(vf=vf[vff.bool()].cpu().numpy(), ee=ee[eef.bool()].cpu().numpy())

    # ------------------------------------------------------------------
    def solve(self, x, x_prev, topo: dict, vf, ee, *, iterations: int, k_stretch: float, k_bend: float,
              thickness: float, ground_y: float, dt: float, sphere: tuple | None = None,
              world: tuple | None = None) -> dict:
        """PBDStepSolver followed by PBDStepIntegration (Physics/CudaPBD.cu:
        632-667), run with the reference's own solver kernels.

        x, x_prev: (V, 3) float32 predicted and previous positions; topo: the
        static topology in the oracle's layout (oracle_ffi.Oracle.topology:
        stretch ends, rest lengths, bend vertices, the per-vertex slot CSR,
        pinned ids, attachment lengths, inverse masses, pinned flags); vf, ee:
        (N, 12) int32 PrimitiveContact records (Physics/Structs.h:106-129);
        sphere: (centre, radius) or None; world: (min corner, max corner).
        Returns the positions after the solver iterations (``x``), the
        velocities and previous positions after _FinalUpdate (``v``,
        ``x_prev``), the positions after the world clamp of
        Physics/CudaDeformableUtils.cu:251-267 (``x_end``), and how many
        ground constraints and attachments the step activated.

        The host work between launches restates the reference's host code:
        the per-iteration clears of the accumulators, and for the contact
        corrections the stable key sort, run-length encoding and exclusive
        sum of Physics/CudaPBD.cu:711-721 (CUB there, numpy here; a stable
        sort's result is unique).
        """
        torch = self.torch
        f32, i32 = np.float32, np.int32
        x = np.ascontiguousarray(x, f32)
        xp = np.ascontiguousarray(x_prev, f32)
        V = x.shape[0]
        s12 = np.asarray(topo["s12"], i32).reshape(-1, 2)
        bq = np.asarray(topo["b"], i32).reshape(-1, 4)
        soff = np.asarray(topo["soff"], i32)
        sent = np.asarray(topo["sent"], i32)
        fixed = np.asarray(topo["fixed"], i32)
        E, B, S, F = len(s12), len(bq), len(sent), len(fixed)
        tri = bool(topo.get("tri_bend", False))
        nb_roles = 3 if tri else 4
        if x.shape != (V, 3) or xp.shape != (V, 3) or len(soff) != V + 1 or soff[0] != 0 or soff[-1] != S \
                or np.any(np.diff(soff) < 0):
            raise ValueError("state and slot offsets do not match")
        for a in (s12, bq[:, :nb_roles], fixed):
            if a.size and (a.min() < 0 or a.max() >= V):
                raise ValueError("vertex id out of range")
        # Slot of each (constraint, role): the inverse of the CSR entries.
        kind, role, cid = (sent >> 30) & 1, (sent >> 28) & 3, sent & 0x0FFFFFFF
        so = np.full((E, 2), -1, i32)
        bo = np.full((B, 4), -1, i32)
        slots = np.arange(S, dtype=i32)
        st, bd = kind == 0, kind == 1
        if np.any(cid[st] >= E) or np.any(role[st] > 1) or np.any(cid[bd] >= B):
            raise ValueError("slot entry out of range")
        so[cid[st], role[st]] = slots[st]
        bo[cid[bd], role[bd]] = slots[bd]
        if np.any(role[bd] >= nb_roles):
            raise ValueError("slot entry out of range")
        if (so < 0).any() or (bo[:, :nb_roles] < 0).any():
            raise ValueError("a constraint end has no slot")
        vf = np.ascontiguousarray(vf, i32).reshape(-1, 12)
        ee = np.ascontiguousarray(ee, i32).reshape(-1, 12)
        for c in (vf, ee):
            if len(c) and (c[:, :4].min() < 0 or c[:, :4].max() >= V):
                raise ValueError("contact vertex out of range")
        nvf, nee = len(vf), len(ee)
        N = nvf + nee

        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        d_x, d_xp = dev(x), dev(xp)
        d_invm = dev(np.asarray(topo["invm"], f32))
        d_fixedv = dev(np.asarray(topo["pinned"], np.uint8) != 0)
        d_s1, d_s2 = dev(s12[:, 0]), dev(s12[:, 1])
        d_s1o, d_s2o = dev(so[:, 0]), dev(so[:, 1])
        d_sl0 = dev(np.asarray(topo["sl0"], np.float64).astype(f32))
        d_b = [dev(bq[:, j]) for j in range(4)]
        d_bo = [dev(bo[:, j]) for j in range(4)]
        d_phi0 = dev(np.full(max(B, 1), np.float32(3.14159265359), f32))  # Physics/CudaPBD.cu:35,368
        d_h0 = dev(np.asarray(topo.get("h0", np.zeros(max(B, 1))), np.float64).astype(f32) if B else np.zeros(1, f32))
        d_soff = dev(soff)
        cor = torch.zeros((max(S, 1), 3), dtype=torch.float32, device="cuda")
        d_fixed = dev(fixed if F else np.zeros(1, i32))
        d_l0 = dev(np.asarray(topo["lra_l0"], np.float64).reshape(V, F).astype(f32) if F else np.zeros(1, f32))
        lflag = torch.zeros(max(V * F, 1), dtype=torch.bool, device="cuda")
        gq = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        gn = torch.zeros_like(gq)
        gflag = torch.zeros(V, dtype=torch.bool, device="cuda")
        acc = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        cnt = torch.zeros(V, dtype=torch.int32, device="cuda")
        h, it = C.c_float(thickness), C.c_int(iterations)

        self.launch("ground_create", V, C.c_int(V), d_x, d_xp, d_invm, C.c_float(ground_y), h, gq, gn, gflag)
        if F:
            self.launch("lra_create", V * F, C.c_int(V), C.c_int(F), d_x, d_fixedv, d_fixed, d_l0, lflag)
        if sphere is not None:
            sq, sn = torch.zeros_like(gq), torch.zeros_like(gq)
            sflag = torch.zeros(V, dtype=torch.bool, device="cuda")
            centre, radius = sphere
            self.launch("sphere_create", V, C.c_int(V), d_x, d_xp, d_invm, Float3(*[float(q) for q in centre]),
                        C.c_float(radius), h, sq, sn, sflag)
        if N:
            d_vf = dev(vf if nvf else np.zeros((1, 12), i32))
            d_ee = dev(ee if nee else np.zeros((1, 12), i32))
            raw_ids = torch.zeros(4 * N, dtype=torch.int32, device="cuda")
            raw_vals = torch.zeros((4 * N, 3), dtype=torch.float32, device="cuda")
        for _ in range(iterations):
            acc.zero_()
            cnt.zero_()
            self.launch("ground_apply", V, C.c_int(V), d_x, d_invm, gflag, gq, gn, acc, cnt)
            if F:
                self.launch("lra_apply", V, C.c_int(V), C.c_int(F), d_x, d_invm, d_fixed, d_l0, lflag, acc, cnt)
            if tri:  # Physics/CudaPBD.cu:840-851
                self.launch("static_project_tri", E + B, C.c_int(E), C.c_int(B), it, d_x, d_invm, d_s1, d_s2, d_s1o,
                            d_s2o, C.c_float(k_stretch), d_sl0, *d_b[:3], *d_bo[:3], C.c_float(k_bend), d_h0, cor)
            else:
                self.launch("static_project", E + B, C.c_int(E), C.c_int(B), it, d_x, d_invm, d_s1, d_s2, d_s1o, d_s2o,
                            C.c_float(k_stretch), d_sl0, *d_b, *d_bo, C.c_float(k_bend), d_phi0, cor)
            self.launch("static_apply", V, C.c_int(V), cor, d_soff, acc, cnt)
            if N:
                self.launch("dyn_project", N, d_x, d_xp, d_invm, h, d_vf, C.c_uint64(nvf), d_ee, C.c_uint64(nee),
                            raw_ids, raw_vals)
                torch.cuda.synchronize()
                ids = raw_ids.cpu().numpy().view(np.uint32)
                if ids.max() >= V:
                    raise RuntimeError("correction id out of range")
                order = np.argsort(ids, kind="stable")
                sids = ids[order]
                starts = np.flatnonzero(np.r_[True, sids[1:] != sids[:-1]]).astype(i32)
                runs = len(starts)
                d_uniq = dev(sids[starts].astype(np.uint32).view(i32))
                d_pref = dev(starts)
                d_vals = dev(raw_vals.cpu().numpy()[order])
                self.launch("dyn_apply", runs, C.c_int(runs), d_uniq, d_pref, d_vals, C.c_uint64(4 * N), acc, cnt)
            if sphere is not None:
                self.launch("sphere_apply", V, C.c_int(V), d_x, h, sflag, sq, sn, acc, cnt)
            self.launch("final_correction", V, C.c_int(V), acc, cnt, d_x)
        torch.cuda.synchronize()
        x_solved = d_x.cpu().numpy().copy()
        d_v = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        self.launch("final_update", V, C.c_int(V), d_x, d_xp, d_v, d_fixedv, C.c_float(dt))
        if world is not None:
            lo, hi = world
            self.launch("world_clamp", V, C.c_int(V), d_x, Float3(*[float(q) for q in lo]),
                        Float3(*[float(q) for q in hi]))
        torch.cuda.synchronize()
        return dict(x=x_solved, v=d_v.cpu().numpy(), x_prev=d_xp.cpu().numpy(), x_end=d_x.cpu().numpy(),
                    ground=gflag.cpu().numpy().astype(np.uint8),
                    ground_flags=int(gflag.sum()), lra_flags=int(lflag[:V * F].sum()) if F else 0)

    # ------------------------------------------------------------------
    def friction(self, v, ground, vf, k_friction: float) -> np.ndarray:
        """CudaPBD::ApplyFriction (Physics/CudaPBD.cu:770-833) with the
        reference's kernels on velocities v (V, 3) after _FinalUpdate, the
        step's ground-constraint flags and its VF contacts (N, 12) int32
        PrimitiveContact records, whose normals the kernels read.

        _DampVelRigid runs with the reference's launch shape, 255 threads per
        block over ceil(V/256) blocks (:777).  _ApplyFriction gets no EE
        contacts: its EE half leaves the vertex ids of its entries unwritten
        (:1796-1845), which with EE contacts present would sort and
        accumulate whatever ids the buffer held.  The CUB sort, run-length
        encoding and exclusive sum (:813-818) run on the host.  Returns the
        velocities after FinalFrictionStep."""
        torch = self.torch
        f32, i32 = np.float32, np.int32
        vel = np.ascontiguousarray(v, f32)
        V = vel.shape[0]
        ground = np.ascontiguousarray(ground, np.uint8).reshape(V)
        vf = np.ascontiguousarray(vf, i32).reshape(-1, 12)
        if len(vf) and (vf[:, :4].min() < 0 or vf[:, :4].max() >= V):
            raise ValueError("contact vertex out of range")
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        d_v = dev(vel)
        d_g = dev(ground != 0)
        d_gn = dev(np.tile(np.array([0, 1, 0], f32), (V, 1)))  # ground normals (Physics/CudaPBD.cu:1492)
        kf = C.c_float(k_friction)
        blocks = (V + THREADS - 1) // THREADS
        self.launch("damp_rigid", V, C.c_int(V), d_v, kf, d_g, d_gn, None, None, block=THREADS - 1, blocks=blocks)
        acc = torch.zeros((V, 3), dtype=torch.float32, device="cuda")
        cnt = torch.zeros(V, dtype=torch.int32, device="cuda")
        N = len(vf)
        if N:
            d_vf = dev(vf)
            ids = torch.zeros(4 * N, dtype=torch.int32, device="cuda")
            vals = torch.zeros((4 * N, 3), dtype=torch.float32, device="cuda")
            self.launch("apply_friction", N, d_v, kf, d_vf, C.c_uint64(N), None, C.c_uint64(0), ids, vals)
            torch.cuda.synchronize()
            h_ids = ids.cpu().numpy().view(np.uint32)
            order = np.argsort(h_ids, kind="stable")
            sids = h_ids[order]
            starts = np.flatnonzero(np.r_[True, sids[1:] != sids[:-1]]).astype(i32)
            runs = len(starts)
            self.launch("accumulate_friction", runs, C.c_int(runs), kf, dev(sids[starts].view(i32)), dev(starts),
                        dev(vals.cpu().numpy()[order]), C.c_uint64(4 * N), acc, cnt)
        self.launch("final_friction", V, C.c_int(V), kf, acc, cnt, d_v)
        torch.cuda.synchronize()
        return d_v.cpu().numpy()


def _glm_inverse3(m: np.ndarray) -> np.ndarray:
    """glm::inverse of a float mat3 (Dependencies/glm/detail/type_mat3x3.inl
    :37-56): the transposed cofactor matrix times the reciprocal of the
    determinant, every operation rounded to float32.  m and the result are
    indexed [column][row] as glm stores them."""
    f = np.float32
    m = np.asarray(m, f)
    a = lambda c, r: f(m[c, r])
    one_over_det = f(1) / (a(0, 0) * (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2))
                           - a(1, 0) * (a(0, 1) * a(2, 2) - a(2, 1) * a(0, 2))
                           + a(2, 0) * (a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2)))
    inv = np.empty((3, 3), f)
    inv[0, 0] = +(a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) * one_over_det
    inv[1, 0] = -(a(1, 0) * a(2, 2) - a(2, 0) * a(1, 2)) * one_over_det
    inv[2, 0] = +(a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1)) * one_over_det
    inv[0, 1] = -(a(0, 1) * a(2, 2) - a(2, 1) * a(0, 2)) * one_over_det
    inv[1, 1] = +(a(0, 0) * a(2, 2) - a(2, 0) * a(0, 2)) * one_over_det
    inv[2, 1] = -(a(0, 0) * a(2, 1) - a(2, 0) * a(0, 1)) * one_over_det
    inv[0, 2] = +(a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2)) * one_over_det
    inv[1, 2] = -(a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2)) * one_over_det
    inv[2, 2] = +(a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1)) * one_over_det
    return inv


def _glm_mat3_mul(m: np.ndarray, v) -> np.ndarray:
    """glm's mat3 * vec3 for a column-major m[column][row]: row r of the
    result is m[0][r] v.x + m[1][r] v.y + m[2][r] v.z, summed left to right
    in float32."""
    f = np.float32
    v = np.asarray(v, f)
    return np.array([f(m[0, r]) * v[0] + f(m[1, r]) * v[1] + f(m[2, r]) * v[2] for r in range(3)], f)


def _check_tree(L, R, Pa, T) -> int:
    """Every node below the root has its parent; returns the depth."""
    In = T - 1
    nodes = 2 * T - 1
    if L.min() < 0 or R.min() < 0 or L.max() >= nodes or R.max() >= nodes:
        raise ValueError("child index out of range")
    seen = np.zeros(nodes, dtype=np.int32)
    depth = np.zeros(nodes, dtype=np.int32)
    stack = [0]
    while stack:
        n = stack.pop()
        seen[n] += 1
        if n < In:
            for c in (int(L[n]), int(R[n])):
                if Pa[c] != n:
                    raise ValueError("parent link missing")
                depth[c] = depth[n] + 1
                stack.append(c)
    if not np.all(seen == 1):
        raise ValueError("hierarchy does not reach every node exactly once")
    return int(depth.max())


def contact_fields(c: np.ndarray):
    """(ids (n,4) int32, weights (n,4) float32, t (n,) float32, normal (n,3))."""
    c = np.ascontiguousarray(c, np.int32)
    f = c.view(np.float32)
    return c[:, :4].copy(), f[:, 4:8].copy(), f[:, 8].copy(), f[:, 9:12].copy()
