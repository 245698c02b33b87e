"""KinematicArcLength over the GPU assembly against the same driver over the oracle.

The four-crease plate of tests/arclength_helpers.py, the drivers' rest angle moved toward
150 deg with the exact fold gradient and the exact hinge tangent, 10 continuation steps:
- FP64 GPU assembly: the same accepted steps with the same corrector iteration counts, mu
  within 1e-9 and fold angles within 1e-7 deg of the oracle run;
- mixed GPU assembly (FP32 tangent, FP64 residual): every step converges to the same
  residual tolerance; the fold angles at each step's mu lie on the oracle's path within
  0.05 deg (linear interpolation between the oracle's steps).
"""
import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import arclength as A
from curvami_gb300 import solver as S
from oracle import Oracle

from arclength_helpers import four_crease_case, oracle_arc_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as ge

    ge.build()
    yield cg.Context(0)


def _run(prob, drivers, kmax=10):
    sol = A.ArcLengthSolver(kmax=kmax, max_iters=30, dsmax=2.0, exact_fold_gradient=True)
    sol.kinematic_arc_length(prob, np.zeros(prob.ns), drivers)
    return sol


def test_kinematic_arc_length_gpu_matches_oracle(ctx):
    o = Oracle(native=True)
    p, doms, drivers = four_crease_case(target_deg=150.0)
    ref = _run(oracle_arc_problem(o, p, doms), drivers)
    model = cg.PlateModel(p, ctx=ctx)
    g64 = _run(S.gpu_problem(model, points=doms, exact_hinge=True), drivers)
    assert len(g64.steps) == len(ref.steps) == 10 and g64.failed_steps == ref.failed_steps == 0
    for a, b in zip(g64.steps, ref.steps):
        assert a.iterations == b.iterations
        assert abs(a.load - b.load) <= 1e-9
        assert np.abs(np.subtract(a.angles, b.angles)).max() <= 1e-7
    mx = _run(S.gpu_problem(model, points=doms, exact_hinge=True, mixed=True), drivers)
    assert mx.failed_steps == 0 and len(mx.steps) == 10
    mus = np.array([0.0] + [s.load for s in ref.steps])
    ang = np.array([[0.0] * 4] + [s.angles for s in ref.steps])
    worst = 0.0
    for st in mx.steps:
        if st.load > mus[-1]:
            break
        for f in range(4):
            worst = max(worst, abs(st.angles[f] - np.interp(st.load, mus, ang[:, f])))
    print("mixed: iterations", [s.iterations for s in mx.steps], "oracle", [s.iterations for s in ref.steps],
          "worst angle deviation from the oracle path (deg)", worst)
    assert worst <= 0.05
