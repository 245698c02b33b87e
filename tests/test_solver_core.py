"""The host drivers on the reference's own consumer tests (tests/consumer/main.cpp:1-240 of
the reference): analytic problems for the generic solver core, restated with the same
problems, settings and bars.

- CubicSpring: x0 on a grounded spring k0, a cubic spring kc d + a d^3 (d = x1 - x0) to x1,
  load lambda on x1, constraint x0 = 0; equilibrium kc x1 + a x1^3 = lambda (x1 = 1 at
  lambda = 2 with kc = a = 1).
- FollowerSpring: one rotation theta, spring k theta under a follower torque
  lambda m sin(beta - theta); exact path lambda = k theta / (m sin(beta - theta)); the
  exact tangent needs the load stiffness -m cos(beta - theta).
"""
import math

import numpy as np
import scipy.sparse as sp

from curvami_gb300 import arclength as A
from curvami_gb300 import solver as S


class CubicSpring:
    k0, kc, a = 10.0, 1.0, 1.0

    def num_dofs(self):
        return 2

    def internal_force(self, x):
        d = x[1] - x[0]
        f = self.kc * d + self.a * d ** 3
        return np.array([self.k0 * x[0] - f, f])

    def external_force(self, x=None):
        return np.array([0.0, 1.0])

    def assemble(self, x):
        d = x[1] - x[0]
        kt = self.kc + 3.0 * self.a * d * d
        K = sp.csc_matrix(np.array([[self.k0 + kt, -kt], [0.0, kt]]))   # upper triangle only
        return K, self.internal_force(x)

    def constraints(self, x):
        return np.array([x[0]]), sp.csr_matrix(np.array([[1.0, 0.0]]))


class FollowerSpring:
    k, m, beta = 2.0, 1.0, 0.5 * math.pi

    def __init__(self, use_load_stiffness=True):
        self.use = use_load_stiffness
        self.assemblies = 0

    def num_dofs(self):
        return 1

    def internal_force(self, x):
        return np.array([self.k * x[0]])

    def external_force(self, x):
        return np.array([self.m * math.sin(self.beta - x[0])])

    def assemble(self, x):
        self.assemblies += 1
        return sp.csc_matrix(np.array([[self.k]])), self.internal_force(x)

    def load_stiffness(self, x):
        if not self.use:
            return None
        return sp.csc_matrix(np.array([[-self.m * math.cos(self.beta - x[0])]]))

    def constraints(self, x):
        return np.zeros(0), sp.csr_matrix((0, 1))

    def path_error(self, lam, theta):
        return abs(lam - self.k * theta / (self.m * math.sin(self.beta - theta)))


def test_line_search_cubic_spring():
    solver = S.ContinuationSolver()
    x = np.zeros(2)
    assert solver.line_search(CubicSpring(), 2.0, x)
    assert abs(x[1] - 1.0) <= 1e-8
    assert abs(x[0]) <= 1e-12


def test_arc_length_cubic_spring():
    solver = A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.5)
    seen = []
    solver.arc_length(CubicSpring(), 0.0, np.zeros(2), 5.0, on_converged=lambda k, lam, x, w: seen.append((lam, x.copy())))
    assert seen and seen[-1][0] > 5.0
    assert max(abs(x[1] + x[1] ** 3 - lam) for lam, x in seen) <= 1e-8
    assert max(abs(x[0]) for _, x in seen) <= 1e-12


def test_line_search_follower_torque():
    iters, theta = {}, {}
    for with_kl in (True, False):
        fs = FollowerSpring(with_kl)
        x = np.zeros(1)
        assert S.ContinuationSolver().line_search(fs, 1.0, x)
        iters[with_kl], theta[with_kl] = fs.assemblies, x[0]
        assert fs.path_error(1.0, x[0]) <= 1e-7
    assert iters[True] < iters[False]
    assert abs(theta[True] - theta[False]) <= 1e-8


def test_arc_length_follower_torque():
    per_step = {}
    for with_kl in (True, False):
        fs = FollowerSpring(with_kl)
        solver = A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.2)
        worst, steps = [0.0], [0]

        def cb(k, lam, x, w):
            steps[0] += 1
            worst[0] = max(worst[0], fs.path_error(lam, x[0]))

        solver.arc_length(fs, 0.0, np.zeros(1), 2.0, on_converged=cb)
        assert steps[0] > 0 and worst[0] <= 1e-7
        per_step[with_kl] = fs.assemblies / steps[0]
    assert per_step[True] < per_step[False]


def test_arc_length_follower_torque_passes_the_barrier_only_with_load_stiffness():
    """Without the load stiffness the corrector's contraction factor lambda m sin(theta) / k
    reaches 1 at theta tan(theta) = 1 (lambda* = 2.6245); with it the path passes lambda = 3."""
    reached = {}
    for with_kl in (True, False):
        fs = FollowerSpring(with_kl)
        solver = A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.2, kmax=200)
        last = [0.0]
        solver.arc_length(fs, 0.0, np.zeros(1), 3.0, on_converged=lambda k, lam, x, w: last.__setitem__(0, lam))
        reached[with_kl] = last[0]
    assert reached[True] > 3.0
    assert reached[False] < 2.6245 + 0.05


def test_kmax_is_a_pure_step_cap():
    """kmax caps the continuation's accepted steps and nothing else (the reference's
    tests/regression/kmax_check.py): a capped run is the uncapped run's prefix, and the
    LineSearch iteration cap (ls_max_iters) is a separate setting."""
    full, capped = [], []
    A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.5).arc_length(
        CubicSpring(), 0.0, np.zeros(2), 5.0, on_converged=lambda k, lam, x, w: full.append((lam, x.copy())))
    A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.5, kmax=3).arc_length(
        CubicSpring(), 0.0, np.zeros(2), 5.0, on_converged=lambda k, lam, x, w: capped.append((lam, x.copy())))
    assert len(capped) == 3 < len(full)
    for (l1, x1), (l2, x2) in zip(capped, full):
        assert l1 == l2 and np.array_equal(x1, x2)
    s = S.ContinuationSolver(ls_max_iters=7)
    assert s.ls_max_iters == 7 and not hasattr(s, "kmax")


def test_restart_continues_the_uninterrupted_run(tmp_path):
    """A run cut short (lambda_tot, as the reference's restart_check cuts al_arccrease by
    max_load) and restarted from its record to the end gives the uninterrupted run's steps,
    bitwise, including the external work."""
    from curvami_gb300 import restart as RM

    full = []
    A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.5).arc_length(
        CubicSpring(), 0.0, np.zeros(2), 5.0, on_converged=lambda k, lam, x, w: full.append((k, lam, x.copy(), w)))
    path = str(tmp_path / "run.res")
    first, second = [], []
    A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.5, restart_file=path).arc_length(
        CubicSpring(), 0.0, np.zeros(2), 2.5, on_converged=lambda k, lam, x, w: first.append((k, lam, x.copy(), w)))
    s2 = A.ArcLengthSolver(psi=1.0, ds=0.2, dsmax=0.5, restart_file=path)
    s2.arc_length(CubicSpring(), 0.0, np.zeros(2), 5.0,
                  on_converged=lambda k, lam, x, w: second.append((k, lam, x.copy(), w)))
    assert s2.restarted_from == len(first) + 1
    both = first + second
    assert len(both) == len(full)
    for a, b in zip(both, full):
        assert a[0] == b[0] and a[1] == b[1] and np.array_equal(a[2], b[2]) and a[3] == b[3]


def test_restart_record_layout_and_rejections(tmp_path):
    from curvami_gb300 import restart as RM

    p = str(tmp_path / "r.res")
    x = np.array([1.0, -2.0, 3.5])
    assert RM.save(p, 7, 0.25, 0.1, 0.01, 3.0, x, 2 * x)
    raw = open(p, "rb").read()
    assert raw[:8] == b"CURVRES\x00" and len(raw) == 8 + 4 + 4 + 32 + 4 + 48
    k, lam, ds, dl, W, xr, dU = RM.load(p, 3)
    assert (k, lam, ds, dl, W) == (7, 0.25, 0.1, 0.01, 3.0) and np.array_equal(xr, x) and np.array_equal(dU, 2 * x)
    assert RM.load(p, 4) is None                       # another problem's record
    open(p, "wb").write(raw[:-5])
    assert RM.load(p) is None                           # truncated
    open(p, "wb").write(b"XXXXXXXX" + raw[8:])
    assert RM.load(p) is None                           # not a record
    assert RM.load(str(tmp_path / "none.res")) is None
    assert not RM.save(p, 1, 0.0, 0.1, 0.0, 0.0, x, x[:2])
