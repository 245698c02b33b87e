"""Arc-length continuation of fold-driven plates over the GPU assembly.

The reference drives its fold mechanisms with two arc-length continuations in
(state x, load parameter), both on the host around the assembly and a KKT solve:

  * ``kinematic_arc_length`` = NonLinearSolver::KinematicArcLength
    (plate/NonLinearSolver.h:607-812): the rest angle of every driver crease moves from
    angle_start to angle_target as the deployment parameter mu goes from 0 to 1; the
    predictor load is the pseudo-force of that motion through the driver hinges,
    -sum Kt (d theta0 / d mu) grad(theta); no external force;
  * ``target_directed_arc_length`` = NonLinearSolver::TargetDirectedArcLength
    (plate/NonLinearSolver.h:156-410): a follower moment lambda * sum r_i grad(theta_i) on
    the driver creases (r_i their remaining travel, scaled to max |r_i| = 1) until every
    driver is within target_tol_deg of its target.

Both, and the generic ``arc_length`` (ContinuationSolver::ArcLength, core/include/curvami/
solver/ContinuationSolver.h:329-540, checked against the reference's own consumer tests),
share the step control of StepController (core/include/curvami/solver/
StepController.h:16-229), restated here with the same names and defaults: ASLA (Crisfield's
square-root rule with target relaxation), the curvature controller, reversal bookkeeping
and the no-progress stall test at dsmin. ``fold_gradient`` restates ComputeFoldGradient
(NonLinearSolver.h:417-493) and ``fold_angle_deg`` ComputeFoldAngleDeg (NonLinearSolver.h:
62-90, with the FoldAngle averages of plate/FoldAngleUtil.h).

Restart records (``restart_file``) follow RestartManager: loaded at the start of a run, written
after every accepted step, in the reference's binary layout (restart.py). As in the reference,
KinematicArcLength's first predictor after a restart takes the pseudo-load at the plate's
kinematics when the record was loaded (the initial state), so a restarted kinematic run leaves
the uninterrupted path; ArcLength and TargetDirectedArcLength evaluate their load at the loaded
state and continue it exactly. Not restated: the inertia count. The reference reads
the reduced Hessian's negative modes from MUMPS's factorisation (INFOG(12)) and uses them
only with the opt-in snap-back veto (off by default, StepController.h:41). The KKT here is
an LU, so a requested reversal is always taken, as the reference does with the veto off.

Any PlateProblem (solver.py) with fold data (FoldSides with Kt and weight) and a backend
that can set a fold's rest angle drives the same algorithm: the GPU library, or the oracle
in the tests.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

from . import restart as RM
from . import solver as S
from .creasing import weighted_mean_about_circular_mean_rad


@dataclass
class Driver:
    """Fold::is_driver with its angle_start / angle_target (radians) and fold_sign
    (plate/PlateData.h:78-86; main.cpp:105-127)."""
    fold: int
    angle_start: float = 0.0
    angle_target: float = 0.0
    fold_sign: float = 1.0


def sector_supports(plate, crease_a: int = 0, crease_b: int = 1, offset: float = 0.3, spacing: float = 0.08):
    """Three point supports inside the sector between creases a and b of a plate whose
    creases start at one vertex (synth.four_crease_plate): P1 on the sector's bisector at
    `offset` x the plate's width from the vertex with u = v = w = 0, P2 = P1 + s e_x with
    v = w = 0 and P3 = P1 + s e_y with w = 0 (s = `spacing` x the width). They remove the
    rigid-body motion the way the reference's point supports do (u v w / v w / w on three
    mesh points, examples/fourvertex/*.json). Returns LineDomains of one point each."""
    c = np.asarray(plate.creases[crease_a]["vertices"][0], np.float64)
    da = np.asarray(plate.creases[crease_a]["vertices"][-1], np.float64) - c
    db = np.asarray(plate.creases[crease_b]["vertices"][-1], np.float64) - c
    a0, a1 = math.atan2(da[1], da[0]), math.atan2(db[1], db[0])
    mid = a0 + 0.5 * ((a1 - a0) % (2.0 * math.pi))
    width = float(plate.node_xy[:, 0].max() - plate.node_xy[:, 0].min())
    P1 = c + offset * width * np.array([math.cos(mid), math.sin(mid)])
    s = spacing * width
    pts = [(P1, S.BoundaryCondition(True, True, True)),
           (P1 + np.array([s, 0.0]), S.BoundaryCondition(False, True, True)),
           (P1 + np.array([0.0, s]), S.BoundaryCondition(False, False, True))]
    return [S.LineDomain(np.asarray([q], np.float64), np.ones(1), np.array([[1.0, 0.0]]),
                         np.array([[0.0, 1.0]]), bc) for q, bc in pts]


# ---- fold kinematics ----------------------------------------------------------------------

def _frames(tab: S.ShapeTable, X: np.ndarray):
    """a1 = e1 + u_X, a2 = e2 + u_Y and the unit normal b at every point of a shape table
    (Kinematics::compute, plate/Kinematics.h:61-104)."""
    a1 = tab.Dx @ X
    a2 = tab.Dy @ X
    a1[:, 0] += 1.0
    a2[:, 1] += 1.0
    n = np.cross(a1, a2)
    b = n / np.linalg.norm(n, axis=1)[:, None]
    return a1, a2, b


def fold_gradient(fold: S.FoldSides, x, exact: bool = False) -> np.ndarray:
    """ComputeFoldGradient (plate/NonLinearSolver.h:417-493): sum over the crease points of
    weight * (s dc/du - c ds/du) / (c^2 + s^2) for the fold angle theta = atan2(-s, c), with
    c = bL.bR, s = (bL x bR).t and t the left side's deformed tangent; dc/du and ds/du as the
    reference forms them (the normal's derivative taken as -[W]x with W = dPsi_y a1 - dPsi_x
    a2, neither normalised nor projected). At the flat state this is -sum w grad(theta); as
    the fold closes it drifts from it (measured: direction off by 1.2 deg and norm by 3 % at
    17 deg of fold, 10 deg and 21 % at 45 deg), which leaves the arc-length corrector's
    linearisation inconsistent. Points with a degenerate tangent (|aT| < 1e-14) or collinear
    normals (c^2 + s^2 < 1e-14) are skipped.

    exact=True (an extension, off in the reference's algorithm) returns -sum w grad(theta)
    with the exact fold-angle gradient of the hinge (Constraints::foldAngleAndGrad), the same
    sign convention, so the corrector's linearisation is consistent."""
    Lt, Rt = fold.left, fold.right
    X = np.asarray(x, np.float64).reshape(-1, 3)
    ns = 3 * Lt.n_nodes
    out = np.zeros(ns)
    if Lt.n_gp == 0 or Rt.n_gp == 0:
        return out
    if exact:
        F12 = np.empty((Lt.n_gp, 12))
        F12[:, 0:3] = Lt.Dx @ X; F12[:, 3:6] = Lt.Dy @ X
        F12[:, 6:9] = Rt.Dx @ X; F12[:, 9:12] = Rt.Dy @ X
        F12[:, 0] += 1.0; F12[:, 4] += 1.0; F12[:, 6] += 1.0; F12[:, 10] += 1.0
        _, g = S.fold_angle_and_grad(F12, fold.tangent[:, 0], fold.tangent[:, 1])
        w = np.asarray(fold.weight, np.float64)
        for tab, off in ((Lt, 0), (Rt, 6)):
            e = tab.rows()
            for d in range(3):
                v = -w[e] * (g[e, off + d] * tab.dpsi[:, 0] + g[e, off + 3 + d] * tab.dpsi[:, 1])
                out[d::3] += np.bincount(tab.idx, weights=v, minlength=tab.n_nodes)
        return out
    a1L, a2L, bL = _frames(Lt, X)
    a1R, a2R, bR = _frames(Rt, X)
    tx, ty = fold.tangent[:, 0], fold.tangent[:, 1]
    aT = a1L * tx[:, None] + a2L * ty[:, None]
    naT = np.linalg.norm(aT, axis=1)
    ok = naT >= 1e-14
    t = aT / np.where(ok, naT, 1.0)[:, None]
    c = np.einsum("ij,ij->i", bL, bR)
    nLR = np.cross(bL, bR)
    s = np.einsum("ij,ij->i", nLR, t)
    denom = c * c + s * s
    ok &= denom >= 1e-14
    w = np.asarray(fold.weight, np.float64) * ok
    inv = np.where(ok, 1.0 / np.where(ok, denom, 1.0), 0.0)
    # Pt n_LR = (n_LR - t (t . n_LR)) / |aT|, per point.
    Pt_n = (nLR - t * s[:, None]) / np.where(ok, naT, 1.0)[:, None]

    # Left side: dc = W x bR, ds = W x (bR x t) + dPsi_t Pt n_LR.
    e = Lt.rows()
    dx, dy = Lt.dpsi[:, 0], Lt.dpsi[:, 1]
    W = dy[:, None] * a1L[e] - dx[:, None] * a2L[e]
    dc = np.cross(W, bR[e])
    dt = (dx * tx[e] + dy * ty[e])[:, None] * Pt_n[e]
    ds = np.cross(W, np.cross(bR, t)[e]) + dt
    g = (w * inv)[e][:, None] * (s[e][:, None] * dc - c[e][:, None] * ds)
    for d in range(3):
        out[d::3] += np.bincount(Lt.idx, weights=g[:, d], minlength=Lt.n_nodes)
    # Right side: dc = W x bL, ds = W x (t x bL).
    e = Rt.rows()
    dx, dy = Rt.dpsi[:, 0], Rt.dpsi[:, 1]
    W = dy[:, None] * a1R[e] - dx[:, None] * a2R[e]
    dc = np.cross(W, bL[e])
    ds = np.cross(W, np.cross(t, bL)[e])
    g = (w * inv)[e][:, None] * (s[e][:, None] * dc - c[e][:, None] * ds)
    for d in range(3):
        out[d::3] += np.bincount(Rt.idx, weights=g[:, d], minlength=Rt.n_nodes)
    return out


def fold_angle_deg(fold: S.FoldSides, x) -> float:
    """ComputeFoldAngleDeg (plate/NonLinearSolver.h:62-90): theta = atan2(-s, c) at every
    active crease point, averaged with the points' weights about their circular mean."""
    Lt, Rt = fold.left, fold.right
    if Lt.n_gp == 0 or Rt.n_gp == 0:
        return 0.0
    X = np.asarray(x, np.float64).reshape(-1, 3)
    a1L, a2L, bL = _frames(Lt, X)
    _, _, bR = _frames(Rt, X)
    aT = a1L * fold.tangent[:, 0][:, None] + a2L * fold.tangent[:, 1][:, None]
    t = aT / np.linalg.norm(aT, axis=1)[:, None]
    c = np.einsum("ij,ij->i", bL, bR)
    s = np.einsum("ij,ij->i", np.cross(bL, bR), t)
    theta = np.arctan2(-s, c)
    act = np.ones(Lt.n_gp, bool) if fold.active is None or len(fold.active) == 0 else np.asarray(fold.active) != 0
    if not act.any():
        return 0.0
    return weighted_mean_about_circular_mean_rad(theta[act], np.asarray(fold.weight)[act]) * 180.0 / math.pi


def wrapped_distance_deg(a_deg: float, b_deg: float) -> float:
    """FoldAngle::wrappedDistanceDeg: a - b the short way round (IEEE remainder by 360)."""
    return math.remainder(a_deg - b_deg, 360.0)


# ---- the step controller and the two continuations ---------------------------------------

@dataclass
class Step:
    """One accepted continuation step: its number, the load parameter, the corrector
    iterations that converged it, ds after the controllers, the fold angles (degrees)."""
    k: int
    load: float
    iterations: int
    ds: float
    angles: list


class ArcLengthSolver(S.ContinuationSolver):
    """ContinuationSolver + StepController with the reference's defaults (kmax 5000,
    max_iters 100, psi 1, ds 0.1 in [1e-6, 10], Id 6, the no-progress window of 24 accepted
    steps at efficiency 0.15)."""

    NO_REVERSAL_YET = 1 << 20

    def __init__(self, ds=0.1, dsmin=1e-6, dsmax=10.0, Id=6, max_iters=100, psi=1.0, kmax=5000,
                 asla_hold_after_reversal=False, no_progress_window=24, no_progress_efficiency=0.15,
                 no_progress_abort=True, exact_fold_gradient=False, restart_file="", **kw):
        """exact_fold_gradient: the drivers' load direction from the exact fold-angle gradient
        (fold_gradient(exact=True)), an extension; False is the reference's algorithm."""
        super().__init__(**kw)
        self.exact_fold_gradient = bool(exact_fold_gradient)
        self.restart_file = restart_file
        self.restarted_from = None   # step k the last run resumed at, when it did
        self.ds, self.dsmin, self.dsmax = float(ds), float(dsmin), float(dsmax)
        self.Id, self.max_iters, self.psi, self.kmax = int(Id), int(max_iters), float(psi), int(kmax)
        self.asla_hold_after_reversal = asla_hold_after_reversal
        self.no_progress_window = int(no_progress_window)
        self.no_progress_efficiency = float(no_progress_efficiency)
        self.no_progress_abort = no_progress_abort
        self.steps_since_reversal = self.NO_REVERSAL_YET
        self._np_ref = None
        self._np_count = 0
        self._np_path = 0.0
        self.steps: list[Step] = []
        self.failed_steps = 0
        self.log: list[str] = []
        self.timing = {"assemble_s": 0.0, "kkt_s": 0.0, "constraints_s": 0.0, "folds_s": 0.0}
        self.counts = {"assemblies": 0, "kkt_factorisations": 0, "kkt_solves": 0, "kkt_refine_steps": 0,
                       "kkt_fallbacks": 0}

    # -- StepController (StepController.h) --
    def note_reversal(self):
        self.steps_since_reversal = 0

    def note_accepted_step(self):
        if self.steps_since_reversal < self.NO_REVERSAL_YET:
            self.steps_since_reversal += 1

    def reset_no_progress(self):
        self._np_ref, self._np_count, self._np_path = None, 0, 0.0

    def reset_inertia_tracking(self):
        self.steps_since_reversal = self.NO_REVERSAL_YET
        self.reset_no_progress()

    def stalled_at_dsmin(self, x, dU) -> bool:
        if not self.no_progress_abort:
            return False
        if self.ds > self.dsmin * (1.0 + 1e-12):
            self.reset_no_progress()
            return False
        if self._np_ref is None or len(self._np_ref) != len(x):
            self.reset_no_progress()
            self._np_ref = np.array(x, copy=True)
            return False
        self._np_path += float(np.linalg.norm(dU))
        self._np_count += 1
        if self._np_count < self.no_progress_window:
            return False
        moved = float(np.linalg.norm(x - self._np_ref))
        path = self._np_path
        self._np_ref = np.array(x, copy=True)
        self._np_count, self._np_path = 0, 0.0
        return path > 0.0 and moved <= self.no_progress_efficiency * path

    def confirm_reversal(self, label: str) -> bool:
        # Without the opt-in inertia veto the reference takes every requested reversal.
        self.log.append(label)
        return True

    def asla(self, icorr_ok: int, k_corr: int, cos_theta: float):
        opt_iter = float(self.Id)
        if cos_theta >= 0.99:
            opt_iter = max(opt_iter, 12.0)
        elif cos_theta >= 0.90:
            opt_iter = max(opt_iter, 8.0)
        if icorr_ok == 0:
            self.ds *= 0.50 if k_corr < self.max_iters else 0.75
            return
        scale = min(math.sqrt(opt_iter / float(max(k_corr, 1))), 4.0)
        if 0.90 < scale < 1.10:
            scale = 1.0
        self.ds = min(max(self.ds * scale, self.dsmin), self.dsmax)

    def curvature_controller(self, step: int, cos_theta: float):
        """ApplyMatlabCurvatureController."""
        if step <= 1:
            return
        if cos_theta >= 0.99:
            if not (self.asla_hold_after_reversal and self.steps_since_reversal <= 1):
                self.ds = min(self.ds * 1.5, self.dsmax)
        elif cos_theta >= 0.90:
            pass
        elif cos_theta >= 0.75:
            self.ds = max(self.ds * 0.8, self.dsmin)
        else:
            self.ds = max(self.ds * 0.5, self.dsmin)

    # -- timed pieces --
    def _assemble(self, prob, x):
        t0 = time.perf_counter()
        K, F = prob.assemble(x)
        self.timing["assemble_s"] += time.perf_counter() - t0
        self.counts["assemblies"] += 1
        return K, F

    def _constraints(self, prob, x):
        t0 = time.perf_counter()
        c_all, J_all = prob.constraints(x)
        J = self.filter_rows(J_all)
        c = c_all[self.ind_rows] if len(self.ind_rows) else np.zeros(0)
        self.timing["constraints_s"] += time.perf_counter() - t0
        return c, J

    def _kkt(self, K, J, rhs_cols):
        t0 = time.perf_counter()
        before = dict(S._KKT.stats)
        kkt = S._KKT(K, J, self.kkt)
        self.counts["kkt_factorisations"] += 1
        out = []
        for r in rhs_cols:
            out.append(kkt.solve(r))
            self.counts["kkt_solves"] += 1
        self.counts["kkt_refine_steps"] += S._KKT.stats["refine_steps"] - before["refine_steps"]
        self.counts["kkt_fallbacks"] += S._KKT.stats["fallbacks"] - before["fallbacks"]
        self.timing["kkt_s"] += time.perf_counter() - t0
        return out

    def _fold_gradient(self, prob, f, x):
        t0 = time.perf_counter()
        g = fold_gradient(prob.folds[f], x, exact=self.exact_fold_gradient)
        self.timing["folds_s"] += time.perf_counter() - t0
        return g

    def _cos_theta(self, dU_old, dl_old, dU, dl):
        old_load, new_load = self.psi * dl_old, self.psi * dl
        on = math.sqrt(float(dU_old @ dU_old) + old_load * old_load)
        nn = math.sqrt(float(dU @ dU) + new_load * new_load)
        if on > 0.0 and nn > 0.0:
            return max(-1.0, min(1.0, (float(dU_old @ dU) + old_load * new_load) / (on * nn)))
        return 1.0

    @staticmethod
    def _sym_upper_times(K, v):
        return K @ v + sp.triu(K, k=1).T @ v          # selfadjointView<Upper> * v

    # -- ContinuationSolver::ArcLength (core/include/curvami/solver/ContinuationSolver.h:329-540) --
    def arc_length(self, prob, lambda_0, x0, lambda_tot, on_converged=None):
        """The generic arc-length continuation of F_int(x) - lambda F_ext(x) = 0 with c(x) = 0
        for any problem with num_dofs / assemble / internal_force / external_force /
        constraints (and optionally load_stiffness): predictor K d_T = F_ext, Crisfield's
        corrector with the sphere ||dU||^2 + psi^2 dl^2 ||F_ext||^2 = ds^2, the step control
        above. on_converged(k, lambda, x, W_ext) after every accepted step (W_ext by the
        trapezoidal rule on the initial load). Returns the final state."""
        jmax = self.max_iters
        x = np.array(x0, np.float64, copy=True)
        ns = x.size
        if ns != prob.num_dofs():
            raise ValueError(f"ArcLength: state vector has {ns} entries, problem has {prob.num_dofs()} DOFs")
        lam, k = float(lambda_0), 1
        dU_old, dl_old = np.zeros(ns), 0.0
        c_all, J_all = prob.constraints(x)
        self.initialize_topology(J_all)
        self.reset_inertia_tracking()
        nc = len(self.ind_rows)
        W_ext = 0.0
        F_ref = np.asarray(prob.external_force(x), np.float64)
        x_prev = x.copy()
        if self.restart_file:
            r = RM.load(self.restart_file, ns)
            if r is not None:
                k, lam, self.ds, dl_old, W_ext, x, dU_old = r
                x_prev = x.copy()
                self.restarted_from = k
        while k <= self.kmax and lam <= lambda_tot:
            Fext = np.asarray(prob.external_force(x), np.float64)
            K, _ = self._assemble(prob, x)
            K = self.with_load_stiffness(prob, K, x, lam)
            c_ind, J_ind = self._constraints(prob, x)
            xb_p = S._Projector(J_ind).corrector(c_ind, ns)
            rhs = np.zeros(ns + nc)
            rhs[:ns] = Fext
            (sol,) = self._kkt(K, J_ind, [rhs])
            if not np.all(np.isfinite(sol)):
                break
            d_T = sol[:ns]
            ff = float(Fext @ Fext)
            sgn = 1.0
            if k == 1:
                sgn = 1.0 if float(d_T @ Fext) >= 0.0 else -1.0
            elif float(dU_old @ d_T) < 0.0 and self.confirm_reversal(f"snap-back at step {k}"):
                sgn = -1.0
                self.note_reversal()
            dl = sgn * self.ds / math.sqrt(float(d_T @ d_T) + self.psi * self.psi * ff)
            dU = dl * d_T + xb_p
            icorr_ok, k_corr = 0, jmax
            for j in range(1, jmax + 1):
                curr_lam = lam + dl
                x_curr = x + dU
                c_ind_c, J_ind_c = self._constraints(prob, x_curr)
                Fext_c = np.asarray(prob.external_force(x_curr), np.float64)
                K_c, Fint_c = self._assemble(prob, x_curr)
                K_c = self.with_load_stiffness(prob, K_c, x_curr, curr_lam)
                R = Fint_c - curr_lam * Fext_c
                v_res = float(dU @ dU) + self.psi * self.psi * dl * dl * ff - self.ds * self.ds
                xb_c = S._Projector(J_ind_c).corrector(c_ind_c, ns)
                r0 = np.zeros(ns + nc)
                r1 = np.zeros(ns + nc)
                r0[:ns] = Fext_c
                r1[:ns] = -(R + self._sym_upper_times(K_c, xb_c))
                s0, s1 = self._kkt(K_c, J_ind_c, [r0, r1])
                if not (np.all(np.isfinite(s0)) and np.all(np.isfinite(s1))):
                    icorr_ok, k_corr = 0, j
                    break
                daP = s0[:ns]
                daPsi = s1[:ns] + xb_c
                mult = s1[ns:]
                denom = float(dU @ daP) + self.psi * self.psi * dl * ff
                dl_c = -(0.5 * v_res + float(dU @ daPsi)) / denom
                dl += dl_c
                dU = dU + daPsi + dl_c * daP
                Rm = R + (J_ind_c.T @ mult if nc else 0.0)
                max_force = float(np.abs(Rm).max())
                energy = abs(float(daPsi @ R))
                geom = float(np.abs(c_ind_c).max()) if nc else 0.0
                if j > 1 and max_force <= self.tol_force and energy <= self.tol_energy and \
                        geom <= self.tol_geom and abs(v_res) <= self.tol_geom:
                    icorr_ok, k_corr = 1, j
                    break
                if max_force >= self.div or math.isnan(max_force):
                    icorr_ok, k_corr = 0, j
                    break
            cos_t = self._cos_theta(dU_old, dl_old, dU, dl) if (k > 1 and icorr_ok == 1) else 1.0
            self.asla(icorr_ok, k_corr, cos_t)
            if icorr_ok == 1:
                self.curvature_controller(k, cos_t)
                self.note_accepted_step()
                dU_old, dl_old = dU, dl
                x = x + dU
                lam += dl
                W_ext += 0.5 * ((lam - dl) + lam) * float(F_ref @ (x - x_prev))
                x_prev = x.copy()
                self.steps.append(Step(k, lam, k_corr, self.ds, []))
                if on_converged is not None:
                    on_converged(k, lam, x, W_ext)
                k += 1
                if self.restart_file:
                    RM.save(self.restart_file, k, lam, self.ds, dl_old, W_ext, x, dU_old)
                if self.stalled_at_dsmin(x, dU):
                    break
            else:
                self.failed_steps += 1
                if self.ds <= self.dsmin:
                    break
        return x

    # -- NonLinearSolver::KinematicArcLength --
    def kinematic_arc_length(self, prob, x0, drivers, on_converged=None):
        """Returns the final state; the accepted steps are in ``self.steps``."""
        jmax = self.max_iters
        x = np.array(x0, np.float64, copy=True)
        ns = x.size
        mu, k = 0.0, 1
        dU_old, dmu_old = np.zeros(ns), 0.0
        c_all, J_all = prob.constraints(x)
        self.initialize_topology(J_all)
        self.reset_inertia_tracking()
        nc = len(self.ind_rows)
        state = x.copy()      # the plate's kinematics: the last state assembled or constrained
        if self.restart_file:
            r = RM.load(self.restart_file, ns)
            if r is not None:
                k, mu, self.ds, dmu_old, _, x, dU_old = r
                self.restarted_from = k

        def update_driver_angles(m):
            for d in drivers:
                prob.set_fold_theta0(d.fold, d.fold_sign * (d.angle_start + m * (d.angle_target - d.angle_start)))

        def f_pseudo(xe):
            F = np.zeros(ns)
            for d in drivers:
                dth = d.fold_sign * (d.angle_target - d.angle_start)
                F -= prob.folds[d.fold].Kt * dth * self._fold_gradient(prob, d.fold, xe)
            return F

        while k <= self.kmax and mu <= 1.05:
            update_driver_angles(mu)
            Fp = f_pseudo(state)
            K, _ = self._assemble(prob, x)
            c_ind, J_ind = self._constraints(prob, x)
            state = x
            xb_p = S._Projector(J_ind).corrector(c_ind, ns)
            rhs = np.zeros(ns + nc)
            rhs[:ns] = Fp
            (sol,) = self._kkt(K, J_ind, [rhs])
            if not np.all(np.isfinite(sol)):
                break
            d_T = sol[:ns]
            sgn = 1.0
            if k > 1 and float(dU_old @ d_T) + self.psi * self.psi * dmu_old < 0.0:
                if self.confirm_reversal(f"kinematic snap-back at step {k}"):
                    sgn = -1.0
                    self.note_reversal()
            dmu = sgn * self.ds / math.sqrt(float(d_T @ d_T) + self.psi * self.psi)
            dU = dmu * d_T + xb_p
            dU_pred, dmu_pred = dU.copy(), dmu
            icorr_ok, k_corr = 0, jmax
            for j in range(1, jmax + 1):
                curr_mu = mu + dmu
                x_curr = x + dU
                c_ind_c, J_ind_c = self._constraints(prob, x_curr)
                update_driver_angles(curr_mu)
                Fp_c = f_pseudo(x_curr)
                K_c, Fint_c = self._assemble(prob, x_curr)
                state = x_curr
                R = Fint_c
                xb_c = S._Projector(J_ind_c).corrector(c_ind_c, ns)
                r0 = np.zeros(ns + nc)
                r1 = np.zeros(ns + nc)
                r0[:ns] = Fp_c
                r1[:ns] = -(R + self._sym_upper_times(K_c, xb_c))
                s0, s1 = self._kkt(K_c, J_ind_c, [r0, r1])
                if not (np.all(np.isfinite(s0)) and np.all(np.isfinite(s1))):
                    icorr_ok, k_corr = 0, j
                    break
                daP = s0[:ns]
                daPsi = s1[:ns] + xb_c
                mult = s1[ns:]
                denom = float(dU_pred @ daP) + self.psi * self.psi * dmu_pred
                dm_c = -float(dU_pred @ daPsi) / denom
                dmu += dm_c
                dU = dU + daPsi + dm_c * daP
                Rm = R + (J_ind_c.T @ mult if nc else 0.0)
                max_force = float(np.abs(Rm).max())
                energy = abs(float(daPsi @ R))
                geom = float(np.abs(c_ind_c).max()) if nc else 0.0
                if j > 1 and max_force <= self.tol_force and energy <= self.tol_energy and geom <= self.tol_geom:
                    icorr_ok, k_corr = 1, j
                    break
                if max_force >= self.div or math.isnan(max_force):
                    icorr_ok, k_corr = 0, j
                    break
            cos_t = self._cos_theta(dU_old, dmu_old, dU, dmu) if (k > 1 and icorr_ok == 1) else 1.0
            self.asla(icorr_ok, k_corr, cos_t)
            if icorr_ok == 1:
                self.curvature_controller(k, cos_t)
                self.note_accepted_step()
                dU_old, dmu_old = dU, dmu
                x = x + dU
                mu += dmu
                state = x
                angles = [fold_angle_deg(f, x) for f in prob.folds]
                self.steps.append(Step(k, mu, k_corr, self.ds, angles))
                if on_converged is not None:
                    on_converged(k, mu, x, angles)
                k += 1
                if self.restart_file:
                    RM.save(self.restart_file, k, mu, self.ds, dmu_old, 0.0, x, dU_old)
                if mu >= 1.0:
                    break
            else:
                self.failed_steps += 1
                if self.ds <= self.dsmin:
                    break
        return x

    # -- NonLinearSolver::TargetDirectedArcLength --
    def target_directed_arc_length(self, prob, lambda_0, x0, lambda_tot, drivers, target_tol_deg=2.0,
                                   on_converged=None):
        """Returns the final state; the accepted steps are in ``self.steps``."""
        jmax = self.max_iters
        x = np.array(x0, np.float64, copy=True)
        ns = x.size
        ang0 = [d.angle_start * d.fold_sign for d in drivers]   # Fold::Ang0 = initial angle
        ratios = np.array([d.angle_target - a for d, a in zip(drivers, ang0)], np.float64)
        if len(ratios) == 0:
            raise ValueError("target_directed_arc_length: no driver folds")
        if np.abs(ratios).max() > 1e-12:
            ratios /= np.abs(ratios).max()
        lam, k = float(lambda_0), 1
        dU_old, dl_old = np.zeros(ns), 0.0
        c_all, J_all = prob.constraints(x)
        self.initialize_topology(J_all)
        self.reset_inertia_tracking()
        nc = len(self.ind_rows)

        def follower(xe):
            F = np.zeros(ns)
            for r, d in zip(ratios, drivers):
                F += r * self._fold_gradient(prob, d.fold, xe)
            return F

        W_ext = 0.0
        x_prev = x.copy()
        if self.restart_file:
            rr = RM.load(self.restart_file, ns)
            if rr is not None:
                k, lam, self.ds, dl_old, W_ext, x, dU_old = rr
                x_prev = x.copy()
                self.restarted_from = k

        while k <= self.kmax and lam <= lambda_tot:
            F_ref = follower(x)
            Fext = F_ref
            K, _ = self._assemble(prob, x)
            c_ind, J_ind = self._constraints(prob, x)
            xb_p = S._Projector(J_ind).corrector(c_ind, ns)
            rhs = np.zeros(ns + nc)
            rhs[:ns] = Fext
            (sol,) = self._kkt(K, J_ind, [rhs])
            if not np.all(np.isfinite(sol)):
                break
            d_T = sol[:ns]
            ff = float(Fext @ Fext)
            sgn = 1.0
            if k == 1:
                sgn = 1.0 if float(d_T @ Fext) >= 0.0 else -1.0
            elif float(dU_old @ d_T) < 0.0 and self.confirm_reversal(f"snap-back at step {k}"):
                sgn = -1.0
                self.note_reversal()
            dl = sgn * self.ds / math.sqrt(float(d_T @ d_T) + self.psi * self.psi * ff)
            dU = dl * d_T + xb_p
            icorr_ok, k_corr = 0, jmax
            for j in range(1, jmax + 1):
                curr_lam = lam + dl
                x_curr = x + dU
                c_ind_c, J_ind_c = self._constraints(prob, x_curr)
                Fext_c = follower(x_curr)
                K_c, Fint_c = self._assemble(prob, x_curr)
                R = Fint_c - curr_lam * Fext_c
                v_res = float(dU @ dU) + self.psi * self.psi * dl * dl * ff - self.ds * self.ds
                xb_c = S._Projector(J_ind_c).corrector(c_ind_c, ns)
                r0 = np.zeros(ns + nc)
                r1 = np.zeros(ns + nc)
                r0[:ns] = Fext_c
                r1[:ns] = -(R + self._sym_upper_times(K_c, xb_c))
                s0, s1 = self._kkt(K_c, J_ind_c, [r0, r1])
                if not (np.all(np.isfinite(s0)) and np.all(np.isfinite(s1))):
                    icorr_ok, k_corr = 0, j
                    break
                daP = s0[:ns]
                daPsi = s1[:ns] + xb_c
                mult = s1[ns:]
                denom = float(dU @ daP) + self.psi * self.psi * dl * ff
                dl_c = -(0.5 * v_res + float(dU @ daPsi)) / denom
                dl += dl_c
                dU = dU + daPsi + dl_c * daP
                Rm = R + (J_ind_c.T @ mult if nc else 0.0)
                max_force = float(np.abs(Rm).max())
                energy = abs(float(daPsi @ R))
                geom = float(np.abs(c_ind_c).max()) if nc else 0.0
                if j > 1 and max_force <= self.tol_force and energy <= self.tol_energy and \
                        geom <= self.tol_geom and abs(v_res) <= self.tol_geom:
                    icorr_ok, k_corr = 1, j
                    break
                if max_force >= self.div or math.isnan(max_force):
                    icorr_ok, k_corr = 0, j
                    break
            cos_t = self._cos_theta(dU_old, dl_old, dU, dl) if (k > 1 and icorr_ok == 1) else 1.0
            self.asla(icorr_ok, k_corr, cos_t)
            if icorr_ok == 1:
                self.curvature_controller(k, cos_t)
                self.note_accepted_step()
                dU_old, dl_old = dU, dl
                x = x + dU
                lam += dl
                W_ext += 0.5 * ((lam - dl) + lam) * float(F_ref @ (x - x_prev))
                x_prev = x.copy()
                angles = [fold_angle_deg(f, x) for f in prob.folds]
                self.steps.append(Step(k, lam, k_corr, self.ds, angles))
                if on_converged is not None:
                    on_converged(k, lam, x, angles)
                k += 1
                if self.restart_file:
                    RM.save(self.restart_file, k, lam, self.ds, dl_old, W_ext, x, dU_old)
                reached = all(abs(wrapped_distance_deg(angles[d.fold], d.angle_target * 180.0 / math.pi))
                              <= target_tol_deg for d in drivers)
                if reached:
                    break
                if self.stalled_at_dsmin(x, dU):
                    break
            else:
                self.failed_steps += 1
                if self.ds <= self.dsmin:
                    break
        return x
