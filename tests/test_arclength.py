"""Arc-length drivers (curvami_gb300/arclength.py) on the host, over the CPU oracle.

- StepController rules (ASLA, curvature controller, no-progress stall) against the
  reference's constants;
- ComputeFoldGradient: -sum w grad(theta) at the flat state (to round-off), drifting from it
  as the fold closes (the reference's formula), exact with exact=True (central differences);
- KinematicArcLength on a plate with four creases from the centre (the drivers' rest angle
  moved from 0 to 150 deg): every step converges, the stiff drivers follow their rest
  angle, the continuation ends past mu = 1;
- TargetDirectedArcLength on the same plate stops once both drivers are within tolerance.
"""
import math

import numpy as np
import pytest

from curvami_gb300 import arclength as A
from curvami_gb300 import solver as S
from oracle import Oracle

from arclength_helpers import four_crease_case, oracle_arc_problem


@pytest.fixture(scope="module")
def o():
    return Oracle(native=True)


def test_asla_and_curvature_controller_rules():
    s = A.ArcLengthSolver(ds=1.0, dsmin=1e-3, dsmax=10.0, max_iters=30)
    s.asla(0, 5, 1.0)                    # failed before max_iters: cut by half
    assert s.ds == pytest.approx(0.5)
    s.asla(0, 30, 1.0)                   # failed at max_iters: cut by a quarter
    assert s.ds == pytest.approx(0.375)
    s.ds = 1.0
    s.asla(1, 3, 0.5)                    # sqrt(6 / 3)
    assert s.ds == pytest.approx(math.sqrt(2.0))
    s.ds = 1.0
    s.asla(1, 3, 0.995)                  # target relaxed to 12 iterations on a straight path
    assert s.ds == pytest.approx(2.0)
    s.ds = 1.0
    s.asla(1, 1, 0.995)                  # sqrt(12 / 1)
    assert s.ds == pytest.approx(math.sqrt(12.0))
    s.ds, s.Id = 1.0, 20
    s.asla(1, 1, 0.5)                    # sqrt(20) capped at 4
    assert s.ds == pytest.approx(4.0)
    s.Id = 6
    s.ds = 1.0
    s.asla(1, 6, 0.5)                    # inside the 0.9 - 1.1 dead band
    assert s.ds == 1.0
    for cos_t, factor in ((0.995, 1.5), (0.95, 1.0), (0.8, 0.8), (0.3, 0.5)):
        s.ds = 1.0
        s.curvature_controller(2, cos_t)
        assert s.ds == pytest.approx(factor)
    s.ds = 1.0
    s.curvature_controller(1, 0.3)       # never on the first step
    assert s.ds == 1.0


def test_no_progress_stall_at_dsmin():
    s = A.ArcLengthSolver(ds=1e-3, dsmin=1e-3, no_progress_window=4)
    x = np.zeros(3)
    assert not s.stalled_at_dsmin(x, np.zeros(3))          # arms the reference state
    step = np.array([1.0, 0.0, 0.0])
    stalled = []
    for i in range(4):                                       # a period-2 cycle: no net motion
        x = x + (step if i % 2 == 0 else -step)
        stalled.append(s.stalled_at_dsmin(x, step))
    assert stalled == [False, False, False, True]
    s2 = A.ArcLengthSolver(ds=1e-3, dsmin=1e-3, no_progress_window=4)
    x = np.zeros(3)
    s2.stalled_at_dsmin(x, np.zeros(3))
    assert not any(s2.stalled_at_dsmin(x := x + step, step) for _ in range(8))   # steady progress
    s3 = A.ArcLengthSolver(ds=1.0, dsmin=1e-3)
    assert not s3.stalled_at_dsmin(np.zeros(3), np.zeros(3))                      # not at dsmin


def test_wrapped_distance():
    assert A.wrapped_distance_deg(-179.5, 180.0) == pytest.approx(0.5)
    assert A.wrapped_distance_deg(170.0, -170.0) == pytest.approx(-20.0)
    assert A.wrapped_distance_deg(10.0, 5.0) == pytest.approx(5.0)


def _fold_about_crease(p, amp):
    c = np.asarray(p.creases[0]["vertices"][0])
    d = np.asarray(p.creases[0]["vertices"][-1]) - c
    d /= np.linalg.norm(d)
    sd = (p.node_xy - c) @ np.array([-d[1], d[0]])
    x = np.zeros((len(p.node_xy), 3))
    x[:, 2] = amp * np.maximum(sd, 0.0)
    return x.ravel()


def test_fold_gradient_reference_and_exact(o):
    p, doms, _ = four_crease_case()
    prob = oracle_arc_problem(o, p, doms)
    f = prob.folds[0]
    x0 = np.zeros(prob.ns)
    g_ref, g_ex = A.fold_gradient(f, x0), A.fold_gradient(f, x0, exact=True)
    assert np.abs(g_ref - g_ex).max() <= 1e-12 * np.abs(g_ex).max()
    x = _fold_about_crease(p, 0.3)
    g_ref, g_ex = A.fold_gradient(f, x), A.fold_gradient(f, x, exact=True)
    cos = g_ref @ g_ex / (np.linalg.norm(g_ref) * np.linalg.norm(g_ex))
    assert 0.999 < cos < 1.0 - 1e-6              # the reference's formula drifts as the fold closes
    # exact: -sum w d theta / d x, checked by central differences of the weighted angle sum
    def wsum(xv):
        X = xv.reshape(-1, 3)
        Lt, Rt = f.left, f.right
        F12 = np.empty((Lt.n_gp, 12))
        F12[:, 0:3] = Lt.Dx @ X; F12[:, 3:6] = Lt.Dy @ X; F12[:, 6:9] = Rt.Dx @ X; F12[:, 9:12] = Rt.Dy @ X
        F12[:, 0] += 1.0; F12[:, 4] += 1.0; F12[:, 6] += 1.0; F12[:, 10] += 1.0
        th, _ = S.fold_angle_and_grad(F12, f.tangent[:, 0], f.tangent[:, 1])
        return float(f.weight @ th)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(prob.ns)
    h = 1e-6
    fd = (wsum(x + h * v) - wsum(x - h * v)) / (2 * h)
    assert abs(-(g_ex @ v) - fd) <= 1e-6 * abs(fd)


def test_fold_angle_matches_the_imposed_fold(o):
    p, doms, _ = four_crease_case()
    prob = oracle_arc_problem(o, p, doms)
    x = _fold_about_crease(p, 1.0)        # w = dist: a 45 deg fold about crease 0
    assert abs(abs(A.fold_angle_deg(prob.folds[0], x)) - 45.0) < 1e-6


@pytest.mark.parametrize("exact", [True, False])
def test_kinematic_arc_length_oracle(o, exact):
    # The reference's gradient (exact=False) is held to the first few degrees of fold, where
    # it is accurate; further on its corrector converges linearly and steps fail.
    p, doms, drivers = four_crease_case(target_deg=150.0)
    prob = oracle_arc_problem(o, p, doms)
    n = 6 if exact else 4
    sol = A.ArcLengthSolver(kmax=n, max_iters=30, dsmax=2.0 if exact else 0.5, exact_fold_gradient=exact)
    sol.kinematic_arc_length(prob, np.zeros(prob.ns), drivers)
    assert len(sol.steps) == n and sol.failed_steps == 0
    mus = [s.load for s in sol.steps]
    assert all(b > a for a, b in zip(mus, mus[1:]))
    for st in sol.steps:
        assert 2 <= st.iterations <= 30
        for d in drivers:      # stiff drivers (Kt 0.1) follow the rest angle mu * 150 deg
            assert abs(st.angles[d.fold] - 150.0 * st.load) < 0.05 * 150.0 * st.load + 0.05
    if exact:                  # consistent linearisation: a few corrector iterations per step
        assert max(st.iterations for st in sol.steps) <= 8


def test_kinematic_arc_length_reaches_the_target(o):
    p, doms, drivers = four_crease_case(target_deg=150.0)
    prob = oracle_arc_problem(o, p, doms)
    sol = A.ArcLengthSolver(kmax=60, max_iters=30, dsmax=2.0, exact_fold_gradient=True)
    sol.kinematic_arc_length(prob, np.zeros(prob.ns), drivers)
    last = sol.steps[-1]
    assert last.load >= 1.0 and sol.failed_steps == 0
    for d in drivers:
        assert abs(last.angles[d.fold] - 150.0 * last.load) < 0.5


def test_target_directed_arc_length_oracle(o):
    """The first TargetDirectedArcLength step: the follower load sum r_i ComputeFoldGradient_i
    is -sum r_i w grad(theta_i) (the gradient's sign at the flat state), so with positive
    travel the drivers' angle first moves negative; the reference's target check wraps at
    +-180 deg (FoldAngle::wrappedDistanceDeg), which is how its +-180 deg targets are met."""
    p, doms, drivers = four_crease_case(target_deg=20.0)
    prob = oracle_arc_problem(o, p, doms)
    sol = A.ArcLengthSolver(kmax=1, max_iters=30, ds=6.25e-3, dsmax=0.5, psi=0.0, exact_fold_gradient=True)
    sol.target_directed_arc_length(prob, 0.0, np.zeros(prob.ns), 500.0, drivers, target_tol_deg=1.0)
    assert len(sol.steps) == 1
    st = sol.steps[0]
    assert st.load > 0.0
    for d in drivers:
        assert st.angles[d.fold] < 0.0


def test_gmres_ir_on_an_ill_conditioned_indefinite_matrix():
    """gmres_ir (solver.py) with an FP32 LU preconditioner, on the CPU: a symmetric
    indefinite matrix of condition 1e8 (the KKT matrices of the arc-length runs reach
    1e7 - 1e9); plain refinement with the same LU stalls there."""
    import torch

    rng = np.random.default_rng(11)
    n = 300
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    sv = np.logspace(0, -8, n) * np.where(rng.random(n) < 0.3, -1.0, 1.0)
    A = torch.from_numpy((Q * sv) @ Q.T)
    b = torch.from_numpy(rng.standard_normal(n))
    lu, piv = torch.linalg.lu_factor(A.float())
    x, rel, steps = S.gmres_ir(A, lu.double(), piv, b)
    ref = torch.linalg.solve(A, b)
    assert rel <= 1e-8 and steps <= 60
    # forward error within the conditioning of the problem (1e8 x 1e-16)
    assert float((x - ref).norm() / ref.norm()) <= 1e-6
    xp = torch.linalg.lu_solve(lu, piv, b.float().unsqueeze(1)).squeeze(1).double()
    for _ in range(20):
        xp = xp + torch.linalg.lu_solve(lu, piv, (b - A @ xp).float().unsqueeze(1)).squeeze(1).double()
    assert float((b - A @ xp).norm() / b.norm()) > 1e-6


@pytest.mark.parametrize("mode", ["device", "device_mixed"])
def test_dense_kkt_formation_and_solve(mode):
    """The dense KKT modes (formed from K's stored upper triangle and J, on a torch device;
    the CPU here) against SciPy's sparse LU of the same [K J^T; J 0]."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    n, m = 80, 9
    A = sp.random(n, n, density=0.15, random_state=1)
    A = (A + A.T + 4.0 * sp.eye(n)).tocsc()
    cols = np.repeat(np.arange(n), np.diff(A.indptr))
    K_upper = sp.csc_matrix((np.where(A.indices <= cols, A.data, 0.0), A.indices, A.indptr), shape=(n, n))
    J = sp.random(m, n, density=0.3, random_state=2).tocsr()
    full = sp.bmat([[A, J.T], [J, None]], format="csc")
    b = np.random.default_rng(0).standard_normal(n + m)
    ref = spla.spsolve(full, b)
    got = S._KKT(K_upper, J, mode, device="cpu").solve(b)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_target_directed_restart(o, tmp_path):
    """TargetDirectedArcLength cut by kmax and restarted from its record (the reference's
    restart_check cuts tdal_arccrease by kmax) continues exactly as the uninterrupted run."""
    p, doms, drivers = four_crease_case(target_deg=20.0)

    def run(kmax, path=""):
        prob = oracle_arc_problem(o, p, doms)
        prob.backend.threads = 1      # the oracle's OpenMP merge is bitwise only on one thread
        sol = A.ArcLengthSolver(kmax=kmax, max_iters=30, ds=6.25e-3, dsmax=0.5, psi=0.0,
                                exact_fold_gradient=True, restart_file=path)
        out = []
        sol.target_directed_arc_length(prob, 0.0, np.zeros(prob.ns), 500.0, drivers, target_tol_deg=1.0,
                                       on_converged=lambda k, lam, x, ang: out.append((k, lam, x.copy())))
        return sol, out

    _, full = run(2)
    path = str(tmp_path / "t.res")
    _, a = run(1, path)
    s2, b = run(2, path)
    assert s2.restarted_from == 2
    assert [r[0] for r in a + b] == [r[0] for r in full] == [1, 2]
    for u, v in zip(a + b, full):
        assert u[1] == v[1] and np.array_equal(u[2], v[2])
