"""Paper A (the reference's examples/paperA_centre_crease/CB_n80_t0.5_xi10.json): the centre
crease grown in a very thin sheet (t/L = 0.0025; 80 x 80 cells, 57,600 face Gauss points, order-3
RKPM at rho = 6h with up to 113 neighbours, 19,683 dofs, Kt = 10 D) by ProgressiveCreasing with
LineSearch Newton steps, node coordinates of the reference's own mesh (tests/golden/
make_paper_a.py).

The initial solve and the first CGB_PAPER_A_STEPS tip moves (default 2; 20 complete the crease) run
three ways, every KKT solve by the same
dense FP32 LU + FP64 GMRES on the GPU:
- the oracle's assembly (the CPU restatement, FP64, static thread split);
- the GPU's FP64 assembly: the same Newton iteration counts, energies within 1e-8;
- the GPU's mixed assembly with two FP64 refinements of every Newton step (the FP32 tangent
  alone, or with one refinement, does not converge on this plate): it converges, and reaches the
  FP64 states (energies within 1e-6), over the first 10 tip moves at most.
Measured on GB300 with CGB_PAPER_A_STEPS=20 (the whole crease): the GPU's FP64 run has the
oracle's Newton iteration count at every one of the 21 solves, energies within 2e-9, in 36 s
against the oracle's 119 s; the mixed run needs 5-49 iterations per move and finds no equilibrium
at the 17th.
CGB_PAPER_A_REPORT=<json path> writes the steps and timings.
"""
import json
import os
import time

import numpy as np
import pytest

from curvami_gb300 import creasing as PC
from curvami_gb300 import solver as S

import creasing_helpers as H

STEPS = int(os.environ.get("CGB_PAPER_A_STEPS", "2"))
# The mixed arm converges for the first 16 tip moves (with up to 49 Newton iterations) and
# finds no equilibrium at the 17th; it is checked over the first 10.
MIXED_STEPS = 10
KEYS = ("step", "a", "b", "newton_iters", "substeps", "E_mem", "E_ben", "E_hin", "theta_mean_deg", "theta_max_deg")


class _Stop(Exception):
    pass


def _run(plate, case, refine=0, max_steps=STEPS):
    solver = S.ContinuationSolver(kkt="device_mixed", refine_steps=refine, **case.solver_args)
    steps = []

    def on_conv(k, x, rec):
        steps.append({key: rec[key] for key in KEYS if key in rec})
        if k >= max_steps:
            raise _Stop()

    t0 = time.perf_counter()
    stopped = ""
    try:
        res = PC.run(solver, plate, np.zeros(3 * len(case.plate.node_xy)), [case.line], cfg=case.config,
                     on_converged=on_conv)
        stopped = res.stopped
    except _Stop:
        pass
    return {"steps": steps, "stopped": stopped, "seconds": time.perf_counter() - t0}


@pytest.mark.gpu
def test_paper_a_first_steps(tmp_path):
    import __graft_entry__ as ge
    from curvami_gb300.api import Context, PlateModel
    from oracle import Oracle

    ge.build()
    case = H.paper_a_case(str(tmp_path / "cb_n80.msh"))
    o = Oracle(native=True)
    oplate = H.OracleCreasingPlate(o, case.plate, case.spec, case.point_bcs, static_schedule=True)
    import torch

    out = {"oracle": _run(oplate, case)}
    ctx = Context(0)
    for name, mixed, refine in (("gpu_fp64", False, 0), ("gpu_mixed_refined2", True, 2)):
        model = PlateModel(case.plate, ctx)
        plate = PC.GpuCreasingPlate(model, case.point_bcs, [case.spec], exact_tangent=True, mixed=mixed)
        out[name] = _run(plate, case, refine, STEPS if not mixed else min(STEPS, MIXED_STEPS))
        del plate, model
    print(json.dumps(out))
    report = os.environ.get("CGB_PAPER_A_REPORT")
    if report:
        with open(report, "w") as f:
            json.dump(out, f, indent=1)
    # Records: the initial solve (step 0, the crease's first segment at each side of the centre)
    # and one per tip move; the crease is complete after 20 moves.
    n_rec = min(STEPS, 20) + 1
    ref = out["oracle"]["steps"]
    assert len(ref) == n_rec and out["oracle"]["stopped"] == ""
    for name, tol in (("gpu_fp64", 1e-8), ("gpu_mixed_refined2", 1e-6)):
        run = out[name]["steps"]
        assert len(run) == (n_rec if name == "gpu_fp64" else min(STEPS, MIXED_STEPS) + 1), name
        assert out[name]["stopped"] == "", name
        for r, g in zip(run, ref):
            if name == "gpu_fp64":
                assert r["newton_iters"] == g["newton_iters"], (name, r, g)
            for k in ("E_mem", "E_ben", "E_hin", "theta_mean_deg"):
                assert r[k] == pytest.approx(g[k], rel=tol, abs=1e-20), (name, r["step"], k)
