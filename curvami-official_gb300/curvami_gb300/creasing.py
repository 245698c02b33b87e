"""Progressive creasing over the GPU path (plate/ProgressiveCreasing.h:33-873).

A crease is written along a fixed polyline and exists only between its tips. At every step
the tips move to the next polyline vertices; every RKPM shape function is rebuilt for the
cut truncated at the tips (``cgb_shape_rebuild``: the neighbour lists and the K pattern
stay, stage A becomes per-step work); the hinge and the continuity constraint are on at the
crease points strictly between the tips, with the rest angle theta0* (``cgb_assembler_set_
fold_state``); one LineSearch Newton solve finds the new equilibrium. When it fails, or the
guard refuses what it converged to, theta0 on the newest crease points is raised from 0 to
theta0* over a few sub-steps from the same start; when that fails too the run stops.

Restated from the reference, with the same names:
  * ``schedule`` / ``truncate`` / ``cumulative_arc_length`` / ``project_arc_length``
    (ProgressiveCreasing.h:82-125, 390-443): the tip positions of the five modes and the cut
    between two path vertices (a tip inside the sheet gets the indicator's end cap);
  * ``circular_mean_rad`` / ``unwrap_about_rad`` / ``weighted_mean_about_circular_mean_rad``
    (plate/FoldAngleUtil.h): the fold-angle averages the step report uses;
  * ``Refitter`` (ProgressiveCreasing.h:219-337): the optional l2 / h1 least-squares re-fit of
    the coefficients after a rebuild;
  * ``run`` = Progressive::run (ProgressiveCreasing.h:450-871): the stages of every line, the
    rebuild with the reported jump, the crease state, the guard, the fallback, the per-step
    CSV log with the reference's columns.
Not restated: the single-step diagnosis mode (``diagnose_step``, printing only) and the
negative-mode count of the reduced Hessian, which the reference reads from MUMPS's
factorisation (INFOG(12)); the KKT here is an LU, so ``neg_modes`` is reported as -1.

The plate is an object with the methods ``run`` needs (``GpuCreasingPlate`` over the GPU
library; any other implementation of the same methods drives the same algorithm).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import solver as S


# ---- configuration and lines (ProgressiveCreasing.h:50-80, 372-381) -----------------------

@dataclass
class Config:
    num_steps: int = 40                # all_at_once only: theta0 ramp steps
    fallback_substeps: int = 4         # newest-piece theta0 sub-steps after a failed solve
    L_ref: float = 1.0                 # facet width L, for the normalised diagnostics
    refit: str = "none"                # none | l2 | h1
    guard_max_theta_deg: float = 180.0
    guard_energy_factor: float = 3.0
    guard_max_motion: float = 0.5
    guard_max_motion_topology: float = 1.0
    log_file: str | None = None        # per-step CSV


@dataclass
class Line:
    """One cut that carries one or more folds (indices into the plate's folds)."""
    folds: list
    full: dict                         # vertices (m, 2), extend_start, extend_end, is_closed
    mode: str = "one_end"
    tip_step: int = 1
    skip: tuple = ()                   # path vertices where a tip must not stop


@dataclass
class Stage:
    a: int
    b: int
    frac: float
    outside: bool = False


def cumulative_arc_length(vertices) -> np.ndarray:
    v = np.asarray(vertices, np.float64)
    S_ = np.zeros(len(v))
    for i in range(1, len(v)):
        S_[i] = S_[i - 1] + math.hypot(*(v[i] - v[i - 1]))
    return S_


def project_arc_length(P, vertices, S_) -> float:
    """Arc length of the closest point of the path to P (first segment wins ties)."""
    v = np.asarray(vertices, np.float64)
    P = np.asarray(P, np.float64)
    best_d, best_s = math.inf, 0.0
    for i in range(len(v) - 1):
        A, d = v[i], v[i + 1] - v[i]
        v2 = float(d @ d)
        if v2 == 0.0:
            continue
        t = max(0.0, min(1.0, float((P - A) @ d) / v2))
        dist = math.hypot(*(P - (A + t * d)))
        if dist < best_d:
            best_d, best_s = dist, S_[i] + t * math.sqrt(v2)
    return best_s


def truncate(full: dict, a: int, b: int) -> dict:
    """The cut between path vertices a and b: an end that is an end of the full path keeps
    its extension flag, a tip inside the sheet gets the end cap."""
    N = len(full["vertices"]) - 1
    return {"vertices": np.asarray(full["vertices"], np.float64)[a:b + 1].copy(),
            "extend_start": bool(full.get("extend_start", False)) if a == 0 else False,
            "extend_end": bool(full.get("extend_end", False)) if b == N else False,
            "is_closed": bool(full.get("is_closed", False)) and a == 0 and b == N}


def schedule(mode: str, tip_step: int, num_steps: int, N: int, skip=()) -> list:
    """Tip positions per step for one line (ProgressiveCreasing.h:390-443)."""
    st = []
    m = max(1, int(tip_step))
    skip = set(int(v) for v in skip)
    if mode == "all_at_once":
        for k in range(num_steps + 1):
            st.append(Stage(0, N, k / num_steps))
    elif mode == "one_end":
        k = 0
        while True:
            b = min(k * m, N)
            if b == N or b not in skip:
                st.append(Stage(0, b, 1.0))
            if b == N:
                break
            k += 1
    elif mode == "one_end_reverse":
        k = 0
        while True:
            a = max(N - k * m, 0)
            if a == 0 or a not in skip:
                st.append(Stage(a, N, 1.0))
            if a == 0:
                break
            k += 1
    elif mode == "middle_out":
        c = N // 2
        k = 0
        while True:
            a, b = max(c - k * m, 0), min(c + k * m, N)
            st.append(Stage(a, b, 1.0))
            if a == 0 and b == N:
                break
            k += 1
    elif mode == "ends_in":
        c = N // 2
        k = 0
        while True:
            a, b = min(k * m, c), max(N - k * m, c)
            last = a == c and b == c
            if last or (a not in skip and b not in skip):
                st.append(Stage(a, b, 1.0, True))
            if last:
                break
            k += 1
    else:
        raise ValueError(f"Progressive creasing: unknown mode '{mode}'")
    return st


# ---- fold-angle averages (plate/FoldAngleUtil.h) ------------------------------------------

def circular_mean_rad(theta, weight) -> float:
    theta = np.asarray(theta, np.float64)
    w = np.asarray(weight, np.float64)
    return math.atan2(float(np.sum(np.sin(theta) * w)), float(np.sum(np.cos(theta) * w)))


def unwrap_about_rad(theta: float, ref: float) -> float:
    d = theta - ref
    while d > math.pi:
        d -= 2.0 * math.pi
    while d < -math.pi:
        d += 2.0 * math.pi
    return ref + d


def weighted_mean_about_circular_mean_rad(theta, weight) -> float:
    if len(theta) == 0:
        return 0.0
    ref = circular_mean_rad(theta, weight)
    acc = sum(unwrap_about_rad(float(t), ref) * float(w) for t, w in zip(theta, weight))
    wsum = float(np.sum(weight))
    return acc / wsum if wsum > 1e-14 else 0.0


def active_fold_angles(theta, weight, active):
    """(mean, largest |theta|) in degrees over the active crease points of one fold
    (Progressive::activeFoldAngles, ProgressiveCreasing.h:157-178)."""
    th = np.asarray(theta, np.float64)[active]
    w = np.asarray(weight, np.float64)[active]
    if len(th) == 0:
        return 0.0, 0.0
    ref = circular_mean_rad(th, w)
    mean = weighted_mean_about_circular_mean_rad(th, w) * 180.0 / math.pi
    mx = max(abs(unwrap_about_rad(float(t), ref)) * 180.0 / math.pi for t in th)
    return mean, mx


# ---- the plate over the GPU library -----------------------------------------------------

@dataclass
class FoldSpec:
    """What a fold of the run carries besides its points: its signed rest-angle target
    theta0* = fold_sign * angle_target (radians) and its crease tag."""
    theta_star: float
    crease_tag: int = 0


class GpuCreasingPlate:
    """A PlateModel (api.py) made ready for ``run``: the LineSearch problem over the GPU
    assembly (with the exact hinge tangent when asked, as fold_exact_tangent), Dirichlet
    rows at the point domains, and the host copies of the shape tables that the constraint
    rows and the step report read, refreshed after every rebuild."""

    def __init__(self, model, point_bcs: dict, folds: list, exact_tangent: bool = True, mixed: bool = False,
                 kkt: str = "host"):
        self.model = model
        self.plate = model.plate
        self.n = len(self.plate.node_xy)
        self.specs = list(folds)
        self.point_bcs = dict(point_bcs)
        backend = S.GpuAssembly(model.asm, mixed=mixed, exact_hinge=exact_tangent)
        sides = []
        for (Ls, Rs), fd in zip(model.fold_sets, self.plate.folds):
            sides.append(S.FoldSides(S.ShapeTable.from_shape_set(Ls, self.n), S.ShapeTable.from_shape_set(Rs, self.n),
                                     np.asarray(fd.left.tangent, np.float64), fd.theta0, fd.rigid))
        points = []
        for tag, bc in self.point_bcs.items():
            ps = self.plate.points[tag]
            z = np.zeros((len(ps.xy), 2))
            dom = S.LineDomain(np.asarray(ps.xy, np.float64), np.asarray(ps.weight, np.float64), z, z, bc)
            points.append((dom, S.ShapeTable.from_shape_set(model.point_sets[tag], self.n)))
        self.problem = S.PlateProblem(self.n, backend, S.ShapeTable.from_shape_set(model.faces, self.n),
                                      self.plate.faces.weight, points=points, folds=sides)
        self.kkt = kkt

    # -- what run() needs --
    @property
    def n_folds(self) -> int:
        return len(self.plate.folds)

    @property
    def rho(self) -> float:
        return float(self.plate.rho)

    def node_xy(self):
        return self.plate.node_xy

    def face_xy(self):
        return self.plate.faces.xy

    def face_weight(self):
        return self.plate.faces.weight

    def fold_points(self, f):
        L_ = self.plate.folds[f].left
        return np.asarray(L_.xy), np.asarray(L_.weight), np.asarray(L_.tangent)

    def theta_star(self, f) -> float:
        return self.specs[f].theta_star

    def crease_tag(self, f) -> int:
        return self.specs[f].crease_tag

    def set_fold_state(self, f, theta0_gp, active):
        self.model.asm.set_fold_state(f, 0.0, theta0_gp, active)
        side = self.problem.folds[f]
        side.theta0_gp = np.array(theta0_gp, np.float64)
        side.active = np.array(active, np.int8)

    def rebuild(self, cuts):
        self.model.rebuild(cuts)
        m, prob = self.model, self.problem
        prob.faces = S.ShapeTable.from_shape_set(m.faces, self.n)
        for side, (Ls, Rs) in zip(prob.folds, m.fold_sets):
            side.left = S.ShapeTable.from_shape_set(Ls, self.n)
            side.right = S.ShapeTable.from_shape_set(Rs, self.n)
        prob.points = [(dom, S.ShapeTable.from_shape_set(m.point_sets[tag], self.n))
                       for (dom, _), tag in zip(prob.points, self.point_bcs)]
        prob._f_ext = None

    def tables(self):
        """(faces, [(left, right)]) host shape tables of the current cut."""
        return self.problem.faces, [(s.left, s.right) for s in self.problem.folds]

    def energies(self, x):
        return self.model.asm.energies(x)


# ---- sampling with the current shape functions --------------------------------------------

def _field(tab, X):
    return tab.P @ X, tab.Dx @ X, tab.Dy @ X


def face_displacements(plate, x):
    faces, _ = plate.tables()
    return faces.P @ np.asarray(x, np.float64).reshape(-1, 3)


def max_distance(u1, u2, xy):
    d = np.linalg.norm(u1 - u2, axis=1)
    if len(d) == 0:
        return 0.0, np.zeros(2)
    i = int(np.argmax(d))
    if d[i] <= 0.0:
        return 0.0, np.zeros(2)
    return float(d[i]), np.asarray(xy[i], np.float64)


def fold_angles_all(plate, f, x):
    """Local fold angle (radians) at every crease point of fold f."""
    _, sides = plate.tables()
    Lt, Rt = sides[f]
    X = np.asarray(x, np.float64).reshape(-1, 3)
    F12 = np.empty((Lt.n_gp, 12))
    F12[:, 0:3] = Lt.Dx @ X; F12[:, 3:6] = Lt.Dy @ X
    F12[:, 6:9] = Rt.Dx @ X; F12[:, 9:12] = Rt.Dy @ X
    F12[:, 0] += 1.0; F12[:, 4] += 1.0; F12[:, 6] += 1.0; F12[:, 10] += 1.0
    _, _, t = plate.fold_points(f)
    theta, _ = S.fold_angle_and_grad(F12, t[:, 0], t[:, 1])
    return theta


def crease_gaps(plate, f, x, L):
    _, sides = plate.tables()
    Lt, Rt = sides[f]
    X = np.asarray(x, np.float64).reshape(-1, 3)
    return np.linalg.norm(Lt.P @ X - Rt.P @ X, axis=1) / L


# ---- re-fit (ProgressiveCreasing.h:219-337) ------------------------------------------------

class Refitter:
    """Least-squares re-fit of the coefficients after the shape functions change, the three
    displacement components at once: l2 minimises sum_g w_g |u(a)_g - u_g|^2 over the face
    points; h1 adds l^2 |G(a)_g - G_g|^2 (G the displacement gradient) and the crease points
    of both sides with weight w_g rho. Targets are the previous state sampled with the
    previous shape functions."""

    def __init__(self, mode: str, l: float):
        if mode not in ("l2", "h1"):
            raise ValueError("creasing.refit must be none, l2 or h1")
        self.h1 = mode == "h1"
        self.l2len = l * l

    @staticmethod
    def sample(plate, x):
        X = np.asarray(x, np.float64).reshape(-1, 3)
        faces, sides = plate.tables()
        return {"face": _field(faces, X), "sides": [(_field(Lt, X), _field(Rt, X)) for Lt, Rt in sides]}

    def fit(self, plate, target, x):
        """Fitted coefficients, or None when the normal equations cannot be solved."""
        faces, sides = plate.tables()
        l2 = self.l2len if self.h1 else 0.0
        w = sp.diags(np.asarray(plate.face_weight(), np.float64))
        M = faces.P.T @ w @ faces.P
        u, gx, gy = target["face"]
        rhs = faces.P.T @ (w @ u)
        if self.h1:
            M = M + l2 * (faces.Dx.T @ w @ faces.Dx + faces.Dy.T @ w @ faces.Dy)
            rhs = rhs + l2 * (faces.Dx.T @ (w @ gx) + faces.Dy.T @ (w @ gy))
            for f, ((Lt, Rt), (tl, tr)) in enumerate(zip(sides, target["sides"])):
                _, wf, _ = plate.fold_points(f)
                wc = sp.diags(np.asarray(wf, np.float64) * plate.rho)
                for tab, (uu, ggx, ggy) in ((Lt, tl), (Rt, tr)):
                    M = M + tab.P.T @ wc @ tab.P + l2 * (tab.Dx.T @ wc @ tab.Dx + tab.Dy.T @ wc @ tab.Dy)
                    rhs = rhs + tab.P.T @ (wc @ uu) + l2 * (tab.Dx.T @ (wc @ ggx) + tab.Dy.T @ (wc @ ggy))
        try:
            lu = spla.splu(sp.csc_matrix(M))
            a = lu.solve(np.asarray(rhs, np.float64))
        except RuntimeError:
            return None
        if not np.all(np.isfinite(a)):
            return None
        return a.reshape(-1)


# ---- the run (ProgressiveCreasing.h:450-871) ---------------------------------------------

CSV_COLUMNS = ("step,a,b,ell,ell_over_Lc,theta0_frac,newton_iters,substeps,E_mem,E_ben,E_hin,"
               "theta_mean_deg,theta_max_deg,neg_modes,jump_over_L,jump_X,jump_Y,change_over_L,"
               "jump_refit_over_L,refit_seconds,start_gap_newest_over_L,start_theta_newest_min_deg,"
               "start_theta_newest_max_deg,guard_retry,line")


@dataclass
class RunResult:
    steps: list = field(default_factory=list)     # one dict per accepted step (the CSV columns)
    stopped: str = ""                             # empty when every stage was made


def run(solver: S.ContinuationSolver, plate, x: np.ndarray, lines, static_creases=(), cfg: Config | None = None,
        on_converged=None, verbose: bool = False) -> RunResult:
    """Progressive::run: make the lines in order, one LineSearch solve per tip move.

    x is updated in place (the last accepted state). On entry the shape functions must be
    those of every cut in full, as the reference's set-up leaves them. on_converged(k, x,
    record) is called after each accepted step."""
    cfg = cfg or Config()
    lines = list(lines)
    if not lines:
        raise RuntimeError("Progressive creasing: no line to make")
    nlines = len(lines)
    prob = plate.problem
    L = cfg.L_ref
    say = print if verbose else (lambda *a, **k: None)

    Sl, Nl, all_folds = [], [], []
    Lc, ngp = 0.0, 0
    gp_s, active, theta0 = {}, {}, {}
    worst_tip = 0.0
    nodes = np.asarray(plate.node_xy(), np.float64)
    for ln in lines:
        N = len(ln.full["vertices"]) - 1
        if N < 1:
            raise RuntimeError("Progressive creasing: crease path has no segments")
        Sv = cumulative_arc_length(ln.full["vertices"])
        Sl.append(Sv); Nl.append(N)
        Lc += Sv[-1]
        for f in ln.folds:
            xy, _, _ = plate.fold_points(f)
            gp_s[f] = np.array([project_arc_length(p, ln.full["vertices"], Sv) for p in xy])
            active[f] = np.zeros(len(xy), np.int8)
            theta0[f] = np.zeros(len(xy))
            all_folds.append(f)
            ngp += len(xy)
        for V in np.asarray(ln.full["vertices"], np.float64):
            worst_tip = max(worst_tip, float(np.min(np.hypot(*(nodes - V).T))))
    multi = len(all_folds) > 1

    def sync(f):
        plate.set_fold_state(f, theta0[f], active[f])

    for f in all_folds:
        sync(f)

    st = []
    for li, ln in enumerate(lines):
        for s in schedule(ln.mode, ln.tip_step, cfg.num_steps, Nl[li], ln.skip):
            empty = (s.a == 0 and s.b == Nl[li]) if s.outside else (s.b == s.a)
            if li > 0 and empty:
                continue
            st.append((li, s))
    say(f" >>> PROGRESSIVE CREASING: {nlines} line(s), {len(all_folds)} fold(s), total crease length "
        f"{Lc:.6g}, {ngp} crease GPs, {len(st)} steps; largest tip-to-node distance {worst_tip:.3e}")

    log = open(cfg.log_file, "w") if cfg.log_file else None
    if log:
        t_star = plate.theta_star(all_folds[0]) * 180.0 / math.pi
        log.write(f"# progressive creasing, mode={lines[0].mode}, L_ref={cfg.L_ref:.10g}, L_c={Lc:.10g}, "
                  f"N={Nl[0]}, tip_step={lines[0].tip_step}, theta0_star_deg={t_star:.10g}, "
                  f"refit={cfg.refit}, ls_on_fail={'fail' if solver.ls_fail_on_no_descent else 'accept'}, "
                  f"guard_max_theta_deg={cfg.guard_max_theta_deg:g}, guard_energy_factor={cfg.guard_energy_factor:g}, "
                  f"guard_max_motion={cfg.guard_max_motion:g}, "
                  f"guard_max_motion_topology={cfg.guard_max_motion_topology:g}, lines={nlines}\n")
        cols = CSV_COLUMNS
        if multi:
            cols += "".join(f",theta_mean_tag{plate.crease_tag(f)},theta_max_tag{plate.crease_tag(f)}"
                            for f in all_folds)
        log.write(cols + "\n")

    refitter = None
    if cfg.refit in ("l2", "h1"):
        refitter = Refitter(cfg.refit, cfg.L_ref)
    elif cfg.refit != "none":
        raise ValueError("creasing.refit must be none, l2 or h1")

    result = RunResult()
    face_xy = np.asarray(plate.face_xy(), np.float64)
    prev_E_tot = 0.0
    prev_edge_ends = 0
    prev_edge_line = 0
    prev = (nlines - 1, 0, Nl[nlines - 1], False)
    prev_active = {f: np.zeros_like(active[f]) for f in all_folds}

    for k, (li, s) in enumerate(st):
        ln = lines[li]
        full, Sv, N = ln.full, Sl[li], Nl[li]
        whole = s.outside and s.a >= s.b
        ell = (Sv[N] if whole else Sv[s.a] + (Sv[N] - Sv[s.b])) if s.outside else Sv[s.b] - Sv[s.a]
        ell += sum(Sl[l_][-1] for l_ in range(li))

        # --- 1. move the tips: rebuild the shape functions, report the jump ---
        jump = jump_refit = refit_s = 0.0
        jump_at = np.zeros(2)
        if (li, s.a, s.b, s.outside) != prev:
            u_old = face_displacements(plate, x)
            target = refitter.sample(plate, x) if refitter else None
            cuts = list(static_creases) + [lines[l_].full for l_ in range(li)]
            if not s.outside:
                if s.b > s.a:
                    cuts.append(truncate(full, s.a, s.b))
            elif whole:
                cuts.append(full)
            else:
                if s.a > 0:
                    cuts.append(truncate(full, 0, s.a))
                if s.b < N:
                    cuts.append(truncate(full, s.b, N))
            plate.rebuild(cuts)
            d, jump_at = max_distance(u_old, face_displacements(plate, x), face_xy)
            jump = jump_refit = d / L
            if refitter:
                t0 = time.perf_counter()
                a_fit = refitter.fit(plate, target, x)
                if a_fit is not None:
                    x[:] = a_fit
                    jump_refit = max_distance(u_old, face_displacements(plate, x), face_xy)[0] / L
                else:
                    say("!!! WARNING: re-fit failed; coefficients carried over.")
                refit_s = time.perf_counter() - t0
            prev = (li, s.a, s.b, s.outside)

        # --- 2. creases on: completed lines in full, this line between its tips ---
        newest = []
        for l_, ln2 in enumerate(lines):
            for f in ln2.folds:
                for i in range(len(gp_s[f])):
                    frac = 1.0
                    if l_ < li:
                        on = True
                    elif l_ > li:
                        on = False
                    elif not s.outside:
                        on = s.b > s.a and Sv[s.a] < gp_s[f][i] < Sv[s.b]
                        frac = s.frac
                    else:
                        on = whole or gp_s[f][i] < Sv[s.a] or gp_s[f][i] > Sv[s.b]
                        frac = s.frac
                    active[f][i] = 1 if on else 0
                    theta0[f][i] = frac * plate.theta_star(f) if on else 0.0
                    if on and not prev_active[f][i]:
                        newest.append((f, i))
        for f in all_folds:
            sync(f)
        say(f"--- Progressive step {k}/{len(st) - 1} | line {li} | vertices "
            f"{'outside ' if s.outside else ''}[{s.a}, {s.b}] | ell/L_c = {ell / Lc:.4f} | "
            f"theta0 frac = {s.frac:.4f} | jump = {jump:.3e} L ---")

        if s.outside:
            edge_ends = (int((s.a > 0 or whole) and bool(full.get("extend_start"))) +
                         int((s.b < N or whole) and bool(full.get("extend_end"))))
        else:
            edge_ends = (int(s.a == 0 and bool(full.get("extend_start"))) +
                         int(s.b == N and bool(full.get("extend_end")))) if s.b > s.a else 0
        topology_step = edge_ends != prev_edge_ends or li != prev_edge_line
        motion_limit = cfg.guard_max_motion_topology if topology_step else cfg.guard_max_motion

        def evaluate(xs, u0):
            r = {}
            r["change"] = max_distance(u0, face_displacements(plate, xs), face_xy)[0] / L
            r["neg"] = -1
            r["E_mem"], r["E_ben"], r["E_hin"] = plate.energies(xs)
            r["f_mean"], r["f_max"] = [], []
            if not multi:
                f = all_folds[0]
                _, w, _ = plate.fold_points(f)
                r["th_mean"], r["th_max"] = active_fold_angles(fold_angles_all(plate, f, xs), w, active[f] != 0)
            else:
                wsum = acc = mx = 0.0
                for f in all_folds:
                    _, w, _ = plate.fold_points(f)
                    m_, x_ = active_fold_angles(fold_angles_all(plate, f, xs), w, active[f] != 0)
                    r["f_mean"].append(m_); r["f_max"].append(x_)
                    wf = float(np.sum(np.asarray(w)[active[f] != 0]))
                    acc += wf * abs(m_); wsum += wf
                    mx = max(mx, x_)
                r["th_mean"] = acc / wsum if wsum > 0.0 else 0.0
                r["th_max"] = mx
            return r

        def guard_why(r):
            why = ""
            E_tot = r["E_mem"] + r["E_ben"] + r["E_hin"]
            if r["th_max"] > cfg.guard_max_theta_deg:
                why += f" max fold angle {r['th_max']:.2f} deg > {cfg.guard_max_theta_deg:.1f};"
            if prev_E_tot > 1e-10 and E_tot > cfg.guard_energy_factor * prev_E_tot:
                why += (f" total energy {prev_E_tot:.3e} -> {E_tot:.3e} (x{E_tot / prev_E_tot:.1f} > "
                        f"x{cfg.guard_energy_factor:.1f});")
            if r["change"] > motion_limit:
                why += (f" step motion {r['change']:.3f} L > {motion_limit:.3f} L"
                        f"{' (topology-change step)' if topology_step else ''};")
            return why

        def set_newest(fac):
            for f, i in newest:
                theta0[f][i] = fac * s.frac * plate.theta_star(f)
            for f in {f for f, _ in newest}:
                sync(f)

        def ramp_newest(xs):
            iters, ok = 0, True
            for j in range(1, cfg.fallback_substeps + 1):
                if not ok:
                    break
                set_newest(j / cfg.fallback_substeps)
                say(f">> fallback sub-step {j}/{cfg.fallback_substeps}")
                ok = solver.line_search(prob, 0.0, xs)
                iters += solver.last_ls_attempts
            return ok, iters

        def full_step(xs):
            set_newest(1.0)
            x0 = xs.copy()
            u0 = face_displacements(plate, xs)
            substeps = retry = 0
            ok = solver.line_search(prob, 0.0, xs)
            iters = solver.last_ls_attempts
            r, why = None, ""
            if ok:
                r = evaluate(xs, u0)
                why = guard_why(r)
                if not why:
                    return True, iters, substeps, retry, r, why
                say(f"!!! GUARD: step {k} converged to a refused state:{why} - discarded.")
                if log:
                    log.write(f"# GUARD REFUSED at step {k}, ell_over_Lc={ell / Lc:.10g}:{why} "
                              f"theta_max={r['th_max']:.6g}, change_over_L={r['change']:.6g}, iters={iters}\n")
                retry = 1
            else:
                say(">> Newton failed.")
            if not newest or cfg.fallback_substeps <= 0:
                return False, iters, substeps, retry, r, why
            xs[:] = x0
            ok, more = ramp_newest(xs)
            iters += more
            substeps = cfg.fallback_substeps
            if not ok:
                return False, iters, substeps, retry, r, ""
            r = evaluate(xs, u0)
            why = guard_why(r)
            if why:
                say(f"!!! GUARD: the fallback's state is refused too:{why}")
                return False, iters, substeps, retry, r, why
            return True, iters, substeps, retry, r, why

        # --- 3. solve ---
        sg = st_lo = st_hi = 0.0
        if newest:
            st_lo, st_hi = 1e9, -1e9
            for f, i in newest:
                g = crease_gaps(plate, f, x, L)[i]
                t = fold_angles_all(plate, f, x)[i] * 180.0 / math.pi
                sg, st_lo, st_hi = max(sg, g), min(st_lo, t), max(st_hi, t)
        x_start = x.copy()
        ok, iters, substeps, guard_retry, r, why = full_step(x)
        if not ok:
            if not why:
                result.stopped = (f"no equilibrium at ell = {ell:.6g} (ell/L_c = {ell / Lc:.4f}), step {k}, "
                                  f"line {li}, vertices [{s.a}, {s.b}]")
                if log:
                    log.write(f"# STOPPED at step {k}, ell={ell:.10g}, ell_over_Lc={ell / Lc:.10g}, line={li}, "
                              f"a={s.a}, b={s.b}\n")
            else:
                result.stopped = f"guard at step {k} (ell/L_c = {ell / Lc:.4f}):{why}"
                if log:
                    log.write(f"# GUARD STOP at step {k}, ell_over_Lc={ell / Lc:.10g}:{why} "
                              f"theta_max={r['th_max']:.6g}, change_over_L={r['change']:.6g}\n")
            say("!!! PROGRESSIVE CREASING STOPPED: " + result.stopped)
            x[:] = x_start
            break
        for f in all_folds:
            prev_active[f] = active[f].copy()
        prev_edge_ends = edge_ends
        prev_edge_line = li

        # --- 4. report ---
        rec = {"step": k, "a": s.a, "b": s.b, "ell": ell, "ell_over_Lc": ell / Lc, "theta0_frac": s.frac,
               "newton_iters": iters, "substeps": substeps, "E_mem": r["E_mem"], "E_ben": r["E_ben"],
               "E_hin": r["E_hin"], "theta_mean_deg": r["th_mean"], "theta_max_deg": r["th_max"],
               "neg_modes": r["neg"], "jump_over_L": jump, "jump_X": float(jump_at[0]),
               "jump_Y": float(jump_at[1]), "change_over_L": r["change"], "jump_refit_over_L": jump_refit,
               "refit_seconds": refit_s, "start_gap_newest_over_L": sg, "start_theta_newest_min_deg": st_lo,
               "start_theta_newest_max_deg": st_hi, "guard_retry": guard_retry, "line": li}
        if multi:
            for f, m_, x_ in zip(all_folds, r["f_mean"], r["f_max"]):
                rec[f"theta_mean_tag{plate.crease_tag(f)}"] = m_
                rec[f"theta_max_tag{plate.crease_tag(f)}"] = x_
        result.steps.append(rec)
        say(f" >> step {k}: iters {iters} (guard retry {guard_retry}, sub-steps {substeps}) | E_mem {r['E_mem']:.4e} "
            f"E_ben {r['E_ben']:.4e} E_hin {r['E_hin']:.4e} | theta mean {r['th_mean']:.3f} max {r['th_max']:.3f} deg"
            f" | jump {jump:.3e} L | step change {r['change']:.3e} L")
        if log:
            log.write(f"{k},{s.a},{s.b},{ell:.10g},{ell / Lc:.10g},{s.frac:.10g},{iters},{substeps},"
                      f"{r['E_mem']:.10e},{r['E_ben']:.10e},{r['E_hin']:.10e},{r['th_mean']:.10g},"
                      f"{r['th_max']:.10g},{r['neg']},{jump:.10e},{jump_at[0]:.10g},{jump_at[1]:.10g},"
                      f"{r['change']:.10e},{jump_refit:.10e},{refit_s:.6g},{sg:.10e},{st_lo:.10g},{st_hi:.10g},"
                      f"{guard_retry},{li}")
            if multi:
                for m_, x_ in zip(r["f_mean"], r["f_max"]):
                    log.write(f",{m_:.10g},{x_:.10g}")
            log.write("\n")
            log.flush()
        prev_E_tot = r["E_mem"] + r["E_ben"] + r["E_hin"]
        if on_converged:
            on_converged(k, x, rec)
    if log:
        log.close()
    return result


# ---- set-up of a run from a mesh (main.cpp:78-250, 536-616) -------------------------------

def plate_for_mesh(path, crease_tag: int, E: float, nu: float, h: float, stiffness: float, angle_target_deg: float,
                   fold_sign: float = 1.0, order: int = 3):
    """synth.Plate of a msh 4.1 file as the reference's set-up builds it for one elastic,
    progressively made fold: the mesh's Gauss points (1-point lines, 3x3 quadrangles),
    rho = (3 + 3) x the median third-neighbour spacing, the reproducibility order of the
    app (Meshless plate(3)), one isotropic ply; theta0* = fold_sign x angle_target."""
    from . import mesh

    p = mesh.plate_from_mesh(path, crease_tags=[crease_tag], Kt=stiffness, order=order, kernel=0, E=E, nu=nu,
                             thickness=h, theta0=0.0)
    spec = FoldSpec(fold_sign * angle_target_deg * math.pi / 180.0, crease_tag)
    return p, spec


# ---- the reference's centre-crease example (examples/smoke_centre_crease, paperA_centre_crease) --

CENTRE_CREASE = {"E": 96000000.0, "nu": 0.3, "h": 0.005, "crease_tag": 5, "stiffness": 1.098901098901099,
                 "angle_target": 0.5, "mode": "middle_out", "tip_step": 1, "num_steps": 40,
                 "fallback_substeps": 4, "L_ref": 1.0,
                 "guard": {"max_theta_deg": 180.0, "energy_factor": 1e30, "max_motion": 1e30,
                           "max_motion_topology": 1e30},
                 "point_bcs": {1: (0.0, 0.0, 0.0), 2: (None, 0.0, 0.0), 4: (None, None, 0.0)},
                 "ls_max_iters": 500, "tol_force": 1e-10, "tol_energy": 1e-12, "fold_exact_tangent": True}


@dataclass
class CentreCreaseCase:
    plate: object
    spec: FoldSpec
    point_bcs: dict
    line: Line
    config: Config
    solver_args: dict


def centre_crease_case(path, n_cells=20, node_xy=None, log_file=None) -> CentreCreaseCase:
    """The reference's centre-crease run (smoke.json / CB_n80_t0.5_xi1.json): a [-1, 1]^2 sheet
    of n_cells^2 quadrangles, a crease (-0.5, 0) -> (0.5, 0) of n_cells / 2 segments grown from
    the centre one segment per step at each end (middle_out), theta0* = 0.5 deg, Kt = D = 1.0989,
    three corner supports that remove the rigid-body motions, Newton tolerances 1e-10 / 1e-12.
    The mesh is written to `path`; node_xy replaces the ideal node coordinates (the gmsh
    coordinates of the reference's own mesh, whose last bits decide on which side of the cut
    the nodes of the crease line fall)."""
    from . import mesh

    c = CENTRE_CREASE
    xy, els = mesh.centre_crease_sheet(n_cells=n_cells, half=1.0, crease_half=0.5, crease_segments=n_cells // 2,
                                       crease_tag=c["crease_tag"])
    if node_xy is not None:
        xy = np.asarray(node_xy, np.float64)
    mesh.write_msh41(path, xy, els)
    p, spec = plate_for_mesh(path, c["crease_tag"], c["E"], c["nu"], c["h"], c["stiffness"], c["angle_target"])
    bcs = {tag: S.BoundaryCondition(u is not None, v is not None, w is not None, u or 0.0, v or 0.0, w or 0.0)
           for tag, (u, v, w) in c["point_bcs"].items()}
    g = c["guard"]
    cfg = Config(num_steps=c["num_steps"], fallback_substeps=c["fallback_substeps"], L_ref=c["L_ref"],
                 guard_max_theta_deg=g["max_theta_deg"], guard_energy_factor=g["energy_factor"],
                 guard_max_motion=g["max_motion"], guard_max_motion_topology=g["max_motion_topology"],
                 log_file=log_file)
    line = Line(folds=[0], full=p.creases[0], mode=c["mode"], tip_step=c["tip_step"])
    return CentreCreaseCase(p, spec, bcs, line, cfg,
                            {"tol_force": c["tol_force"], "tol_energy": c["tol_energy"],
                             "ls_max_iters": c["ls_max_iters"]})
