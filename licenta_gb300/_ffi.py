"""ctypes view of the C ABI in include/lc/lc.h.

The structures below mirror lc.h field for field.  Loading fails loudly: the
engine has no CPU fallback, so a missing or unbuilt library is an error.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_lib" / "liblicenta_gb300.so"

LC_OK = 0
LC_ERR_INVALID_ARG = 1
LC_ERR_CAPACITY_OVERFLOW = 3
LC_ERR_NOT_SUPPORTED = 6
STATUS_NAMES = {
    0: "LC_OK", 1: "LC_ERR_INVALID_ARG", 2: "LC_ERR_OOM", 3: "LC_ERR_CAPACITY_OVERFLOW",
    4: "LC_ERR_TIMEOUT", 5: "LC_ERR_CUDA", 6: "LC_ERR_NOT_SUPPORTED", 7: "LC_ERR_STACK_OVERFLOW",
}
LC_MORTON_REF63 = 0
LC_MORTON_K30 = 1
LC_NARROW_CCD = 0
LC_NARROW_DCD = 1
LC_BP_BRUTE, LC_BP_SAP, LC_BP_GRID, LC_BP_HASH, LC_BP_BVH = 0, 1, 2, 3, 4


class BroadphaseDesc(C.Structure):
    _fields_ = [("method", C.c_int32), ("max_objects", C.c_int32), ("max_entries", C.c_uint64),
                ("world_min", C.c_float * 3), ("world_max", C.c_float * 3), ("cells_per_axis", C.c_int32),
                ("cell_size", C.c_float), ("table_size", C.c_int32)]


class BroadphaseCriteria(C.Structure):
    _fields_ = [("structure_ms", C.c_float), ("collision_ms", C.c_float), ("intersection_tests", C.c_uint64),
                ("pairs", C.c_uint64), ("memory_bytes", C.c_uint64)]


LC_WINDING_CCW = 0
LC_WINDING_CW = 1
COLLIDER_SLOTS = 8

DBG = dict(PRED_X=1, PRED_XPREV=2, PRED_V=3, PERM_BEFORE=4, MORTON=5, PERM=6, LEFTS=7, RIGHTS=8,
           PARENTS=9, RML=10, NODE_AABB=11, PAIRS=12, VF=13, EE=14, FEATURES=15, GROUND=16,
           GROUND_ACTIVE=17, LRA=18, DYN_ACTIVE=19, SPHERE=20, VF_NORMAL=21, COLLIDER=22)

F3 = C.c_float * 3


class ClothParams(C.Structure):
    """lc_cloth_params (Physics::ClothParams, Physics/Structs.h:23-61, plus extensions)."""
    _fields_ = [
        ("timestep", C.c_float), ("kFriction", C.c_float), ("kStretch", C.c_float), ("kShear", C.c_float),
        ("kBend", C.c_float), ("kDamp", C.c_float), ("kSpringDamp", C.c_float), ("thickness", C.c_float),
        ("objectMass", C.c_float), ("globalVelDamp", C.c_float), ("strainLimit", C.c_float),
        ("gravity", F3), ("minWindDir", F3), ("startWindDir", F3), ("maxWindDir", F3),
        ("windMinVariation", C.c_float), ("windMaxVariation", C.c_float), ("windOn", C.c_int32),
        ("worldMin", F3), ("worldMax", F3), ("dims", C.c_int32 * 2), ("solverIterations", C.c_int32),
        ("ccdIterations", C.c_int32), ("BVHChunkSize", C.c_int32), ("benchmarkSample", C.c_uint64),
        ("useTriangleBending", C.c_int32), ("colorContacts", C.c_int32), ("useFriction", C.c_int32),
        ("thicknessFromMesh", C.c_int32), ("mortonMode", C.c_int32), ("refLeafAabbQuirk", C.c_int32),
        ("groundOn", C.c_int32), ("mortonOrigin", F3), ("mortonScale", C.c_float), ("windSeed", C.c_uint64),
        ("sphereOn", C.c_int32), ("spherePos", F3), ("sphereRadius", C.c_float),
    ]


class ClothDesc(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int32), ("num_triangles", C.c_int32),
        ("positions", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_uint32)),
        ("pinned", C.POINTER(C.c_uint8)), ("params", ClothParams),
    ]


class BatchOptions(C.Structure):
    _fields_ = [
        ("vf_capacity", C.c_uint64), ("ee_capacity", C.c_uint64), ("use_graph", C.c_int32),
        ("debug_capture", C.c_int32), ("solver_variant", C.c_int32), ("block_size", C.c_int32),
        ("cand_capacity", C.c_uint64), ("adjoint", C.c_int32),
    ]


class Tuning(C.Structure):
    _fields_ = [("traverse_block", C.c_int32), ("jacobi_block", C.c_int32), ("narrow_blocks_per_sm", C.c_int32),
                ("solver_variant", C.c_int32), ("cluster_size", C.c_int32), ("contact_gather", C.c_int32)]


class AutotuneSpace(C.Structure):
    _fields_ = [("traverse_block", C.c_int32 * 8), ("n_traverse_block", C.c_int32),
                ("jacobi_block", C.c_int32 * 8), ("n_jacobi_block", C.c_int32),
                ("narrow_blocks_per_sm", C.c_int32 * 8), ("n_narrow_blocks_per_sm", C.c_int32),
                ("solver_variant", C.c_int32 * 3), ("n_solver_variant", C.c_int32),
                ("cluster_size", C.c_int32 * 4), ("n_cluster_size", C.c_int32),
                ("contact_gather", C.c_int32 * 2), ("n_contact_gather", C.c_int32)]


class AutotuneTrial(C.Structure):
    _fields_ = [("config", Tuning), ("ms_per_step", C.c_float)]


class Profile(C.Structure):
    _fields_ = [("phase_ms", C.c_float * 7), ("jacobi_ms", C.c_float), ("traverse_ms", C.c_float),
                ("narrow_ms", C.c_float), ("sort_ms", C.c_float), ("step_ms", C.c_float),
                ("kernels_per_step", C.c_uint32), ("solver_ms", C.c_float), ("solver_variant", C.c_int32),
                ("cluster_size", C.c_int32), ("ccd_vf_ms", C.c_float), ("ccd_ee_ms", C.c_float)]


PHASES = ("1. PBD External", "2. Update Triangles", "3. Build BVH", "4. Create Triangle Tests",
          "5. Perform Triangle Tests", "6. PBD Solver", "7. PBD Integration")


class Contact(C.Structure):
    _fields_ = [("v", C.c_int32 * 4), ("w", C.c_float * 4)]


# Every entry point of include/lc/lc.h: name -> (restype, argtypes).
VP = C.c_void_p
SIGNATURES = {
    "lc_default_params": (None, [C.POINTER(ClothParams)]),
    "lc_default_options": (None, [C.POINTER(BatchOptions)]),
    "lc_batch_create": (C.c_int, [C.POINTER(ClothDesc), C.c_int32, C.POINTER(BatchOptions), C.POINTER(VP)]),
    "lc_batch_set_constraint_stiffness": (C.c_int, [VP, VP, VP, C.c_int32]),
    "lc_batch_get_tuning": (C.c_int, [VP, C.POINTER(Tuning)]),
    "lc_default_autotune_space": (None, [C.POINTER(AutotuneSpace)]),
    "lc_batch_autotune": (C.c_int, [VP, C.POINTER(AutotuneSpace), C.c_int32, C.c_int32, C.c_int32, VP,
                                    C.POINTER(Tuning), C.POINTER(C.c_float), C.POINTER(AutotuneTrial), C.c_int32,
                                    C.POINTER(C.c_int32)]),
    "lc_batch_set_tuning": (C.c_int, [VP, C.POINTER(Tuning)]),
    "lc_batch_write_vertex_records": (C.c_int, [VP, VP, C.c_int64, C.c_int32, C.c_int32, VP]),
    "lc_group_create": (C.c_int, [C.POINTER(VP), C.c_int32, C.POINTER(VP)]),
    "lc_group_step": (C.c_int, [VP, C.c_int32, VP]),
    "lc_group_step_io": (C.c_int, [VP, C.c_int32, VP, VP, VP, VP, VP, VP, C.c_int32, VP]),
    "lc_group_destroy": (C.c_int, [VP]),
    "lc_batch_state_size": (C.c_int, [VP, C.POINTER(C.c_uint64)]),
    "lc_batch_save_state": (C.c_int, [VP, VP, VP]),
    "lc_batch_load_state": (C.c_int, [VP, VP, VP]),
    "lc_batch_adjoint_step": (C.c_int, [VP, VP, VP, VP, VP, VP, VP]),
    "lc_batch_adjoint_step_rescaled": (C.c_int, [VP, VP, VP, VP, VP, VP, VP, VP]),
    "lc_batch_destroy": (C.c_int, [VP]),
    "lc_batch_step": (C.c_int, [VP, C.c_int32, VP]),
    "lc_batch_sync": (C.c_int, [VP]),
    "lc_batch_num_cloths": (C.c_int, [VP, C.POINTER(C.c_int32)]),
    "lc_batch_cloth_sizes": (C.c_int, [VP, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lc_batch_get_state": (C.c_int, [VP, C.c_int32, VP, VP, VP, VP, C.c_int32]),
    "lc_batch_set_state": (C.c_int, [VP, C.c_int32, VP, VP, VP, VP, C.c_int32]),
    "lc_batch_get_triangle_order": (C.c_int, [VP, C.c_int32, VP]),
    "lc_batch_set_triangle_order": (C.c_int, [VP, C.c_int32, VP]),
    "lc_batch_read_positions": (C.c_int, [VP, VP, C.c_int32, VP]),
    "lc_batch_set_sphere": (C.c_int, [VP, C.c_int32, C.POINTER(C.c_float), C.c_float]),
    "lc_batch_set_collider": (C.c_int, [VP, C.c_int32, VP, C.c_int32, VP, C.c_int32, C.c_int32]),
    "lc_broadphase_create": (C.c_int, [VP, C.POINTER(C.c_void_p)]),
    "lc_broadphase_update": (C.c_int, [VP, VP, VP, C.c_int32, VP]),
    "lc_broadphase_update_host": (C.c_int, [VP, VP, VP, C.c_int32, VP]),
    "lc_broadphase_test": (C.c_int, [VP, VP, C.c_uint64, C.POINTER(C.c_uint64), VP]),
    "lc_broadphase_test_host": (C.c_int, [VP, VP, C.c_uint64, C.POINTER(C.c_uint64), VP]),
    "lc_broadphase_get_criteria": (C.c_int, [VP, VP]),
    "lc_broadphase_destroy": (C.c_int, [VP]),
    "lc_batch_set_stiffness": (C.c_int, [VP, C.c_int32, VP, VP]),
    "lc_batch_constraint_counts": (C.c_int, [VP, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lc_batch_debug_get": (C.c_int, [VP, C.c_int32, C.c_int32, VP, C.c_uint64, C.POINTER(C.c_uint64)]),
    "lc_batch_counters": (C.c_int, [VP, C.c_uint64 * 4]),
    "lc_batch_write_state": (C.c_int, [VP, VP, VP, VP, C.c_int32, VP]),
    "lc_batch_read_state": (C.c_int, [VP, VP, VP, VP, C.c_int32, VP]),
    "lc_batch_profile": (C.c_int, [VP, C.c_int32, VP, C.c_void_p]),
    "lc_lbvh_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(VP)]),
    "lc_lbvh_build": (C.c_int, [VP, VP, VP, C.c_int32, VP]),
    "lc_lbvh_pairs": (C.c_int, [VP, VP, C.c_uint64, C.POINTER(C.c_uint64), VP]),
    "lc_lbvh_sorted_ids": (C.c_int, [VP, VP, VP]),
    "lc_lbvh_debug_get": (C.c_int, [VP, C.c_int32, VP, C.c_uint64, C.POINTER(C.c_uint64)]),
    "lc_lbvh_destroy": (C.c_int, [VP]),
    "lc_narrowphase_create": (C.c_int, [C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_uint64,
                                        C.POINTER(VP)]),
    "lc_narrowphase_run": (C.c_int, [VP, C.c_int32, VP, VP, VP, C.c_int32, VP, VP, C.c_int32, VP, C.c_uint64, C.c_float,
                                     C.c_float, VP, C.c_uint64, VP, C.c_uint64, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint64), VP]),
    "lc_narrowphase_destroy": (C.c_int, [VP]),
    "lc_solve_collisions": (C.c_int, [VP, VP, VP, VP, C.c_int32, VP, C.c_uint64, VP, C.c_uint64, C.c_float,
                                      C.c_float, C.c_float, C.c_float, VP]),
    "lc_lbvh_pairs_static": (C.c_int, [VP, VP, C.c_int32, C.c_int32, C.c_int32, VP, C.c_uint64,
                                       C.POINTER(C.c_uint64), VP, VP]),
    "lc_last_error_string": (C.c_char_p, []),
    "lc_status_string": (C.c_char_p, [C.c_int]),
    "lc_morton3d": (C.c_uint64, [C.c_float, C.c_float, C.c_float, C.c_int32]),
    "lc_mesh_grid": (C.c_int32, [C.c_int32, C.c_int32, VP]),
    "lc_mesh_icosphere": (C.c_int32, [C.c_int32, VP, VP]),
}

_lib = None


class LcError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {detail}".strip())


def lib() -> C.CDLL:
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"CUDA engine not built: {LIB_PATH} is missing (run licenta_gb300._build.build())")
        L = C.CDLL(str(LIB_PATH), mode=os.RTLD_LOCAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != LC_OK:
        detail = lib().lc_last_error_string()
        raise LcError(status, where, detail.decode() if detail else "")


def default_params() -> ClothParams:
    p = ClothParams()
    lib().lc_default_params(C.byref(p))
    return p


def default_options() -> BatchOptions:
    o = BatchOptions()
    lib().lc_default_options(C.byref(o))
    return o
