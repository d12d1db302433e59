"""Generate the golden vectors of the collision stages from the reference's
own kernels.

Runs on a machine with a GPU, after ``python -m oracle.ref_pin.build_ref``
has built oracle/_ref/ref_kernels.cubin from the reference checkout and
``__graft_entry__.build()`` has built the engine and the oracle:

    python tests/golden/make_golden.py OUTDIR

Each case steps a seeded cloth with the FP32 oracle to a chosen step and
takes the state before the next step (positions, previous positions,
velocities, running vertex normals, the triangle order before the Morton
sort).  From that state the reference's own kernels run the whole step
(oracle/ref_pin/refchain.py): the prediction (PBDStepExternal: external
forces with gravity and wind, the rigid-mode damping, explicit Euler), the
running vertex normals (UpdateVertexNormals), the collision chain on the
predicted state, the solver chain (PBDStepSolver, _FinalUpdate and the world
clamp) with the contacts its collision chain found, and the friction kernels
(CudaPBD::ApplyFriction) on the solver's velocities.
The inputs and the reference's outputs go to OUTDIR/<case>.npz; the tests
hold the oracle (tests/test_golden_cpu.py) and the engine
(tests/test_golden_gpu.py) to them bit for bit.  The script also prints how
the FP32 oracle compares, so a run shows at once whether the pin holds.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

import golden_cases  # noqa: E402
from oracle.oracle_ffi import Oracle  # noqa: E402
from oracle.ref_pin.refchain import RefKernels  # noqa: E402


def main(outdir: str) -> int:
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    ref = RefKernels()
    bad = 0
    for case in golden_cases.CASES:
        spec = golden_cases.make_spec(case)
        o = Oracle([spec], fp64=False)
        if case["steps"]:
            o.step(case["steps"], threads=1)
        pre = {k: a.astype(np.float32) for k, a in o.get_state(0).items()}
        pre_wind, pre_rng = o.wind(0)
        o.step_one(0)
        wind = o.wind(0)[0].astype(np.float32)  # this step's wind, after its update
        perm = o.debug(0, "PERM_BEFORE").astype(np.int64)
        feats = o.debug(0, "FEATURES")
        h = o.thickness(0)
        p = spec.params
        dt = float(p.timestep)
        chunk = int(p.BVHChunkSize)
        tris = spec.indices.astype(np.int64)[perm]
        # the reference's prediction from the pre-step state; its output is
        # the collision stages' input below
        pred = ref.predict(pre["x"], pre["x_prev"], pre["v"], pre["vn"], golden_cases.masses(spec),
                           gravity=tuple(p.gravity), wind=tuple(wind), dt=dt, k_global=float(p.globalVelDamp),
                           k_damp=float(p.kDamp))
        x, xp, v = pred["x"], pre["x_prev"], pred["v"]
        data = dict(x=x, x_prev=xp, v=v, perm_before=perm.astype(np.int32), features=feats,
                    thickness=np.float32(h), dt=np.float32(dt), chunk=np.int32(chunk),
                    meta=np.array(json.dumps(case)),
                    pre_x=pre["x"], pre_x_prev=pre["x_prev"], pre_v=pre["v"], pre_vn=pre["vn"], wind=wind,
                    pre_wind=pre_wind.astype(np.float32), pre_rng=np.uint64(pre_rng),
                    ref_vn=ref.vertex_normals(x, xp, tris, pre["vn"], h),
                    oracle_pred_x=o.debug(0, "PRED_X"), oracle_pred_v=o.debug(0, "PRED_V"))
        # As the reference runs: its refit may read a child before the
        # child's box is visible (kept as evidence, not compared).
        raw = ref.collide(x, xp, v, tris, feats[perm], h, dt, chunk)
        data.update({"raw_" + k: raw[k] for k in ("node_min", "node_max", "rmll", "rmlr", "pairs")})
        # With the internal nodes seeded so that a racing read is harmless.
        r = ref.collide(x, xp, v, tris, feats[perm], h, dt, chunk, prefill=golden_cases.oracle_refit(spec, data))
        data.update({"ref_" + k: val for k, val in r.items()})
        if not spec.params.groundOn:
            raise ValueError("the reference always projects ground constraints: keep groundOn")
        sol = ref.solve(x, xp, vf=r["vf"], ee=r["ee"], **golden_cases.solver_inputs(spec, data, o))
        data.update({"ref_solve_" + k: sol[k] for k in ("x", "v", "x_prev", "x_end")})
        # the reference's other pipeline on the same state: SolveCollisions
        # (impulses from the continuous contacts, with their normals) and the
        # discrete tests of HandleCollisionsDiscrete at x_prev on the same pairs
        imp = ref.solve_collisions(x, xp, v, spec.pinned, r["vf"], r["ee"], **golden_cases.impulse_params(spec, h))
        data["ref_impulse_x"], data["ref_impulse_v"] = imp["x"], imp["v"]
        slot = perm[r["order"].astype(np.int64)]
        dcd = ref.dcd(xp, spec.indices.astype(np.int64)[slot], feats[slot], r["pairs"], h)
        data["ref_dcd_vf"], data["ref_dcd_ee"] = dcd["vf"], dcd["ee"]
        # friction (CudaPBD::ApplyFriction) on the solver's velocities with the
        # step's ground flags and VF contacts
        data["ref_ground"] = sol["ground"]
        data["ref_friction_v"] = ref.friction(sol["v"], sol["ground"], r["vf"], float(spec.params.kFriction))
        raced = int(np.sum(np.any(raw["node_min"] != r["node_min"], axis=1) | np.any(raw["node_max"] != r["node_max"],
                                                                                        axis=1)))
        np.savez_compressed(out / f"{case['name']}.npz", **data)
        o.close()
        # how the FP32 oracle compares on the same inputs
        diffs = golden_cases.compare_oracle(spec, data)
        sdiff = golden_cases.compare_oracle_solver(spec, data)
        fdiff = golden_cases.compare_oracle_friction(spec, data)
        pdiff = golden_cases.compare_oracle_prediction(spec, data)
        print(f"{case['name']}: prediction vs oracle {pdiff}")
        print(f"{case['name']}: dcd vf={len(dcd['vf'])} ee={len(dcd['ee'])}; response and contact records vs oracle "
              f"{golden_cases.compare_oracle_response(spec, data)}")
        print(f"{case['name']}: T={len(perm)} pairs={len(r['pairs'])} vf={len(r['vf'])} ee={len(r['ee'])} "
              f"ground={sol['ground_flags']} lra={sol['lra_flags']} solver vs FP32 oracle {sdiff} friction {fdiff} "
              f"nodes raced in the unseeded refit={raced} "
              f"oracle {'agrees' if not diffs else 'DIFFERS: ' + ', '.join(diffs)}")
        bad += bool(diffs)
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).resolve().parent)))
