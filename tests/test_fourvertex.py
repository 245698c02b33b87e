"""The reference's square-twist example through the GPU assembly: examples/fourvertex/
ST-nx61nf30-TRBL-Kt5-p0.json on SquareTwistFiner.msh (from the fixtures of
tests/golden/make_fourvertex.py), read by curvami_gb300.runconfig as main.cpp reads it
(cubic basis at rho = 6h, four elastic driver creases with Kt = 5 and targets of +-180 deg,
two cuts through the vertex, three point supports, E = 1.2e7, t = 0.01), and driven by
TargetDirectedArcLength with the file's settings (ds 0.1, dsmax 0.75, max_iters 30, psi 0).

The first CGB_FOURVERTEX_STEPS (default 3) steps over the GPU's FP64 assembly are compared with
the same steps over the oracle's assembly (shape functions, stage B and the hinge of the CPU
restatement): the same accepted steps with the same corrector iteration counts, loads within
1e-8 and fold angles within 1e-6 deg. The mixed assembly (FP32 tangent) stays on the same path
(fold angles against the load within 1e-3 deg of the oracle's), with more corrector iterations.
Every arm solves its KKT systems with the same dense FP64 LU on the GPU, standing in for MUMPS.
CGB_FOURVERTEX_REPORT=<json path> writes the steps and timings. Measured on GB300 with
CGB_FOURVERTEX_STEPS=8 (to 13 deg of fold): FP64 iterations 4/5/5/6/6/6/6/7 on both sides, loads
within 6e-10, angles within 3.4e-9 deg.
"""
import json
import math
import os
import sys
import time

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_fourvertex  # noqa: E402
from curvami_gb300 import runconfig as RC  # noqa: E402
from oracle import Oracle  # noqa: E402

from arclength_helpers import oracle_arc_problem  # noqa: E402

STEPS = int(os.environ.get("CGB_FOURVERTEX_STEPS", "3"))


def square_twist():
    cfg, xy, els = make_fourvertex.load()
    return RC.from_elements(cfg, xy, els)


def test_square_twist_config_reads_like_main_cpp():
    """CPU: the configuration as main.cpp builds it (folds in file order, valley signs, the
    two cuts through the vertex, the point supports u v w / v w / w, rho = 6h)."""
    rc = square_twist()
    p = rc.plate
    assert [f.crease_tag for f in rc.folds] == [6, 5, 8, 7]
    assert all(f.driver and not f.rigid and f.stiffness == 5.0 and f.sign == 1.0 for f in rc.folds)
    assert [round(math.degrees(f.angle_target)) for f in rc.folds] == [180, 180, 180, -180]
    assert len(p.creases) == 2 and all(len(c["vertices"]) == 59 for c in p.creases)
    assert [len(f.left.xy) for f in p.folds] == [29, 29, 29, 29]
    assert p.order == 3 and p.n_nodes == 61 * 61 and len(p.faces.xy) == 60 * 60 * 9
    assert p.rho == pytest.approx(6.0 * 2.0 / 60.0, rel=1e-9)
    bcs = [(d.bc.active_u, d.bc.active_v, d.bc.active_w) for d in rc.points]
    assert bcs == [(True, True, True), (False, True, True), (False, False, True)]
    s = rc.solver
    assert (s["ds"], s["dsmax"], s["dsmin"], s["max_iters"], s["psi"], s["max_load"], s["target_tol_deg"]) == \
        (0.1, 0.75, 0.001, 30, 0.0, 500.0, 1.0)
    assert [d.fold for d in rc.drivers()] == [0, 1, 2, 3]


def run(rc, prob):
    sol = rc.arc_length_solver(kmax=STEPS, kkt="device")
    sol.states = []
    t0 = time.perf_counter()
    sol.target_directed_arc_length(prob, 0.0, np.zeros(prob.ns), rc.solver["max_load"], rc.drivers(),
                                   target_tol_deg=rc.solver["target_tol_deg"],
                                   on_converged=lambda k, lam, x, ang: sol.states.append((lam, x.copy())))
    return sol, time.perf_counter() - t0


def equilibrium_residual(rc, prob, lam, x):
    """max |P (F_int(x) - lam F_follower(x))| over the dofs: TargetDirectedArcLength's residual
    (the follower load sum r_i ComputeFoldGradient_i, r_i the drivers' travel scaled to
    max |r_i| = 1) with the constraint forces projected out (P = I - J^T (J J^T)^-1 J over the
    independent constraint rows)."""
    from curvami_gb300 import solver as S

    sol = rc.arc_length_solver()
    _, J_all = prob.constraints(x)
    sol.initialize_topology(J_all)
    _, J = sol._constraints(prob, x)
    drivers = rc.drivers()
    r = np.array([d.angle_target - d.angle_start * d.fold_sign for d in drivers])
    r /= np.abs(r).max()
    F = sum(ri * sol._fold_gradient(prob, d.fold, x) for ri, d in zip(r, drivers))
    return float(np.abs(S._Projector(J).project(prob.internal_force(x) - lam * F)).max())


@pytest.mark.gpu
def test_square_twist_first_steps_match_oracle():
    import __graft_entry__ as ge
    import curvami_gb300 as cg

    ge.build()
    rc = square_twist()
    o = Oracle(native=True)
    prob_o = oracle_arc_problem(o, rc.plate, rc.points, exact_tangent=rc.solver["fold_exact_tangent"])
    ref, t_ref = run(rc, prob_o)
    ctx = cg.Context(0)
    model = cg.PlateModel(rc.plate, ctx)
    out = {"oracle": {"seconds": t_ref, "steps": [vars(s) for s in ref.steps], "failed": ref.failed_steps}}
    runs = {}
    for name, mixed in (("gpu_fp64", False), ("gpu_mixed", True)):
        sol, t = run(rc, RC.gpu_problem(rc, model, mixed=mixed, deterministic=not mixed))
        runs[name] = sol
        out[name] = {"seconds": t, "steps": [vars(s) for s in sol.steps], "failed": sol.failed_steps,
                     "timing": sol.timing}
    # Every arm's converged states as equilibria of the oracle's FP64 problem.
    for name, sol in [("oracle", ref)] + list(runs.items()):
        out[name]["oracle_residual"] = [equilibrium_residual(rc, prob_o, lam, x) for lam, x in sol.states]
    print(json.dumps(out))
    report = os.environ.get("CGB_FOURVERTEX_REPORT")
    if report:
        with open(report, "w") as f:
            json.dump(out, f, indent=1)
    assert len(ref.steps) == STEPS and ref.failed_steps == 0
    # FP64: the oracle's steps, iteration for iteration.
    sol = runs["gpu_fp64"]
    assert len(sol.steps) == len(ref.steps) and sol.failed_steps == 0
    for a, b in zip(sol.steps, ref.steps):
        assert a.iterations == b.iterations, (a, b)
        assert abs(a.load - b.load) <= 1e-8 * abs(b.load), (a, b)
        assert max(abs(x - y) for x, y in zip(a.angles, b.angles)) <= 1e-6, (a, b)
    # Mixed: the FP32 tangent makes the corrector converge linearly, so it takes more
    # iterations and ASLA picks other step lengths. Its first step (the same ds) is the
    # oracle's, and every converged state is an equilibrium of the oracle's FP64 problem: the
    # projected residual within 1e-6 (the run's own test is max |R + J^T mu| <= tol_force =
    # 1e-8 on the GPU's FP64 residual; the orthogonal projection is bounded by the 2-norm of
    # that, at most sqrt(n_dofs) x 1e-8).
    sol = runs["gpu_mixed"]
    assert len(sol.steps) == STEPS and sol.failed_steps == 0
    assert max(abs(x - y) for x, y in zip(sol.steps[0].angles, ref.steps[0].angles)) <= 1e-5
    for name in ("oracle", "gpu_fp64", "gpu_mixed"):
        assert max(out[name]["oracle_residual"]) <= 1e-6, (name, out[name]["oracle_residual"])
