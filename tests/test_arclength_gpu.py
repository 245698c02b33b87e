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


def test_mixed_kkt_solve_on_device():
    """The FP32-LU + FP64-refinement KKT solve against SciPy's sparse LU on arc-length KKT
    matrices of the four-crease plate (flat and folded states): relative error <= 1e-8
    (the matrices' condition numbers reach 3e8, so an FP64 direct solve is itself only
    accurate to about 1e-8)."""
    import scipy.sparse.linalg as spla

    import scipy.sparse as sp

    o = Oracle(native=True)
    p, doms, drivers = four_crease_case(target_deg=150.0)
    prob = oracle_arc_problem(o, p, doms)
    sol = A.ArcLengthSolver(kmax=8, max_iters=30, dsmax=2.0, exact_fold_gradient=True)
    states = [np.zeros(prob.ns)]
    sol.kinematic_arc_length(prob, states[0], drivers, on_converged=lambda k, mu, x, ang: states.append(x.copy()))
    rng = np.random.default_rng(7)
    for x in (states[0], states[-1]):
        K, _ = prob.assemble(x)
        c_all, J_all = prob.constraints(x)
        J = sol.filter_rows(J_all)
        Kf = K + sp.triu(K, k=1).T
        Afull = sp.bmat([[Kf, J.T], [J, None]], format="csc")
        b = rng.standard_normal(Afull.shape[0])
        ref = spla.spsolve(Afull, b)
        got = S._KKT(K, J, "device_mixed").solve(b)
        err = float(np.abs(got - ref).max() / np.abs(ref).max())
        print("device_mixed KKT error", err, S._KKT.stats)
        assert err <= 1e-8
