"""Parity of the CUDA engine against the oracle, through the C ABI.

Collision stages (Morton codes, sorted order, Karras topology, refit boxes,
rightmost-leaf bookkeeping, pairs, VF/EE contacts) must be bit-exact against
the FP32 mirror run on the GPU's own predicted positions.  Positions must stay
within 1e-5 m (relative to the 1 m cloth extent) of the FP64 oracle after
every step, each step starting from the GPU's state (teacher forcing) with the
GPU's contact set frozen in the oracle.  A step that misses the bound is
excused only if one of its bends passed within rounding of the reference's
d -> 1 singularity (oracle.parity.conditioning_bound), and at most one step
in twenty may be.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from licenta_gb300 import ClothBatch, Lbvh, _ffi, scenes
from oracle import parity
from oracle.oracle_ffi import Oracle

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5  # metres, on a 1 m cloth: the 1e-5 relative bound


def run_parity(*args, **kw):
    worst, contacts, _, _ = parity.run_parity(*args, tol=POS_TOL, **kw)
    return worst, contacts


@pytest.mark.parametrize("variant,gather", [(1, 0), (2, 0), (3, 0), (3, 1)],
                         ids=["gather", "cluster", "scatter", "scatter-contact-gather"])
def test_small_cloth_parity_through_contacts(variant, gather):
    worst, contacts = run_parity([scenes.small_cloth(seed=0)], steps=60, variant=variant, contact_gather=gather)
    assert contacts > 0, "the run should reach self-contact"


def test_parity_windy_k30_and_fixed_leaf_mode():
    a = scenes.small_cloth(seed=5, n=20)
    scenes.set_constant_wind(a.params, (1.5, 0.0, -1.0))
    b = scenes.small_cloth(seed=6, n=24)
    b.params.mortonMode = _ffi.LC_MORTON_REF63
    b.params.refLeafAabbQuirk = 0
    run_parity([a, b], steps=25)


def test_k30_batch_parity():
    a = scenes.small_cloth(seed=7, n=18)
    a.params.mortonMode = _ffi.LC_MORTON_K30
    b = scenes.small_cloth(seed=8, n=21)
    b.params.mortonMode = _ffi.LC_MORTON_K30
    run_parity([a, b], steps=20)


@pytest.mark.parametrize("variant", [1, 2, 3], ids=["gather", "cluster", "scatter"])
def test_sphere_and_mesh_thickness_parity(variant):
    s = scenes.large_cloth(seed=2, n=40)
    run_parity([s], steps=40, check_every=3, variant=variant)


@pytest.mark.parametrize("variant", [1, 3], ids=["gather", "scatter"])
def test_friction_parity(variant):
    """CudaPBD::ApplyFriction: a hanging cloth that folds onto itself (VF
    contact normals) and an unpinned cloth landing on a raised ground (the
    ground's rigid damping), velocities against the FP64 oracle every step."""
    hang = scenes.small_cloth(seed=0, n=24)
    hang.params.useFriction = 1
    hang.params.kFriction = 0.3
    flat = scenes.small_cloth(seed=3, n=20)
    flat.pinned[:] = 0
    flat.params.worldMin[1] = 0.9
    flat.params.useFriction = 1
    worst, contacts = run_parity([hang, flat], steps=70, check_every=5, variant=variant, friction=True)
    assert contacts > 0


@pytest.mark.parametrize("variant", [1, 2, 3], ids=["gather", "cluster", "scatter"])
def test_triangle_bending_parity(variant):
    """useTriangleBending: triangle bends (Physics/CudaPBD.cu:474-509,
    1149-1187) in place of the dihedral ones, next to a dihedral cloth."""
    tri = scenes.small_cloth(seed=12, n=28)
    tri.params.useTriangleBending = 1
    run_parity([tri, scenes.small_cloth(seed=13, n=16)], steps=150, check_every=10, variant=variant)


def test_vertex_records(cuda):
    """lc_batch_write_vertex_records into Rendering::VertexFormat records
    (48 B): position = published x_prev, normal = running vertex normal, and
    the color and uv bytes of every record untouched."""
    torch = cuda
    specs = [scenes.small_cloth(seed=1, n=12), scenes.small_cloth(seed=2, n=9)]
    b = ClothBatch(specs)
    b.step(5)
    V = sum(sp.num_vertices for sp in specs)
    buf = torch.full((V * 48,), 0xAB, dtype=torch.uint8, device="cuda")
    b.write_vertex_records(buf.data_ptr())
    b.sync()
    rec = buf.cpu().numpy().view(np.float32).reshape(V, 12)
    raw = buf.cpu().numpy().reshape(V, 48)
    off = 0
    for c, sp in enumerate(specs):
        st = b.get_state(c)
        n = sp.num_vertices
        assert np.array_equal(rec[off:off + n, 0:3], st["x_prev"])
        assert np.array_equal(rec[off:off + n, 7:10], st["vn"])
        off += n
    assert np.all(raw[:, 12:28] == 0xAB) and np.all(raw[:, 40:48] == 0xAB)
    L = _ffi.lib()
    assert L.lc_batch_write_vertex_records(b._h, C.c_void_p(buf.data_ptr()), 48, 0, 8, None) == 1  # overlap
    host = np.zeros(V * 12, np.float32)
    assert L.lc_batch_write_vertex_records(b._h, host.ctypes.data_as(C.c_void_p), 48, 0, 28, None) == 1
    b.close()


def test_uneven_batch_parity():
    specs = scenes.batched_cloths(seed=11, count=5, n_min=5, n_max=40)
    run_parity(specs, steps=15, check_every=2)


def test_batch_equals_individual_runs():
    specs = scenes.batched_cloths(seed=3, count=4, n_min=8, n_max=30)
    together = ClothBatch(specs)
    together.step(12)
    together.sync()
    for c, s in enumerate(specs):
        alone = ClothBatch([s])
        alone.step(12)
        alone.sync()
        a, b = together.get_state(c), alone.get_state(0)
        assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["v"], b["v"])
        assert np.array_equal(together.triangle_order(c), alone.triangle_order(0))
        alone.close()
    together.close()


def test_graph_replay_equals_eager():
    s = scenes.small_cloth(seed=9, n=24)
    g = ClothBatch([s], use_graph=True)
    e = ClothBatch([s], use_graph=False)
    g.step(30)
    e.step(30)
    g.sync()
    e.sync()
    assert np.array_equal(g.get_state(0)["x"], e.get_state(0)["x"])
    g.close()
    e.close()


@pytest.mark.parametrize("variant", [1, 2, 3], ids=["gather", "cluster", "scatter"])
def test_runs_are_bitwise_reproducible(variant):
    specs = scenes.batched_cloths(seed=4, count=3, n_min=10, n_max=48)
    out = []
    for _ in range(2):
        b = ClothBatch(specs, solver_variant=variant)
        b.step(40)
        b.sync()
        out.append([b.get_state(c)["x"] for c in range(len(specs))])
        b.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_cluster_and_gather_solvers_agree():
    s = scenes.small_cloth(seed=12, n=28)
    g = ClothBatch([s], solver_variant=1)
    k = ClothBatch([s], solver_variant=2)
    for step in range(15):
        g.step(1)
        k.step(1)
        a, b = g.get_state(0), k.get_state(0)
        assert np.abs(a["x"] - b["x"]).max() <= 1e-5
        k.set_state(0, **a)  # teacher forcing: both continue from the same state
        k.set_triangle_order(0, g.triangle_order(0))
    g.close()
    k.close()


def test_cluster_profile_reports_variant():
    specs = scenes.batched_cloths(seed=5, count=6, n_min=16, n_max=64)
    b = ClothBatch(specs)
    b.step(2)
    p = b.profile(1)
    assert p["solver_variant"] == 3 and p["cluster_size"] in (4, 8, 16)
    assert p["kernels_per_step"] > 10 and p["step_ms"] > 0
    b.close()


def test_contact_capacity_overflow_is_reported_not_faulted():
    s = scenes.small_cloth(seed=0)
    b = ClothBatch([s], vf_capacity=1, ee_capacity=1)
    with pytest.raises(_ffi.LcError) as ei:
        b.step(60)
        b.sync()
    assert ei.value.status == 3
    # the handle stays usable after the report
    b.sync()
    b.close()


def test_standalone_lbvh_pairs_equal_brute_force(cuda):
    torch = cuda
    lo, hi = scenes.random_triangle_boxes(4000, seed=1)
    lo_t = torch.from_numpy(lo).cuda()
    hi_t = torch.from_numpy(hi).cuda()
    h = Lbvh(4000, chunk_size=64)
    h.build(lo_t.data_ptr(), hi_t.data_ptr(), 4000)
    cap = 4000 * 64
    out = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    n = h.pairs(out.data_ptr(), cap)
    ids = torch.empty(4000, dtype=torch.int32, device="cuda")
    h.sorted_ids(ids.data_ptr())
    torch.cuda.synchronize()
    pairs = out[:n].cpu().numpy()
    order = ids.cpu().numpy()
    got = {tuple(sorted((int(order[i]), int(order[j])))) for i, j in pairs}
    assert len(got) == n
    ov = ~((hi[:, None, :] < lo[None, :, :]) | (lo[:, None, :] > hi[None, :, :])).any(-1)
    iu = np.triu_indices(4000, 1)
    want = set(zip(iu[0][ov[iu]].tolist(), iu[1][ov[iu]].tolist()))
    assert got == want
    h.close()


def test_malformed_hierarchy_reads_current_boxes():
    """Runs of >= 3 equal Morton codes leave internal nodes, the root among
    them, unreached by the refit (scenes.equal_code_cloth).  The traversal's
    node records must then hold the boxes the reference's per-node reads see
    in this step, not records left from an earlier step: the cloth steps twice
    with its loose triangles spread apart (a well-formed hierarchy), then takes
    the near-coincident state and one more step, checked bit-exact (codes,
    hierarchy, boxes, pairs, contacts) against the oracle."""
    bad = scenes.equal_code_cloth()
    good = scenes.equal_code_cloth(offset=(0.0, 0.0, 0.0))
    n0 = good.num_vertices - 12
    good.positions[n0:] += np.repeat(np.arange(4, dtype=np.float32) * 0.01, 3)[:, None] * np.float32([1, 0, 0])
    batch = ClothBatch([good], debug_capture=True)
    batch.step(2)
    batch.sync()
    assert np.any(batch.debug(0, "NODE_AABB")[0] != 0), "the spread-out state builds a well-formed hierarchy"
    vn = batch.get_state(0)["vn"]
    batch.set_state(0, x=bad.positions, x_prev=bad.positions, v=np.zeros_like(bad.positions), vn=vn)
    o32 = Oracle([bad], fp64=False)
    pre = parity.capture_pre(batch, 0)
    batch.step(1)
    batch.sync()
    parity.check_collision(batch, 0, o32, pre[0]["vn"], tag="malformed hierarchy")
    assert np.all(batch.debug(0, "NODE_AABB")[0] == 0), "the root stays unreached in the near-coincident state"
    o32.close()
    batch.close()


def test_body_interface_fixed_update_and_update():
    from licenta_gb300 import CudaDeformableBody
    s = scenes.small_cloth(seed=2, n=16)
    verts = s.positions.copy()
    body = CudaDeformableBody(verts, s.indices, s.params, s.pinned.astype(bool))
    for _ in range(10):
        body.FixedUpdate()
    body.Update()
    st = body.batch.get_state(0)
    assert np.array_equal(verts, st["x_prev"])
    assert not np.array_equal(verts, s.positions)
