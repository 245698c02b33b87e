"""Post-processing over the GPU path: the per-step field table of the exporter and the
stress sampler along rays from a crease tip.

  * ``point_state`` = cgb_point_state: Kinematics::compute + Constitutive::evaluate and the
    displacement at every point of a shape set, on the GPU (one FP64 thread per point);
  * ``step_table`` / ``planarity`` / ``crease_table`` = the three parts of
    Exporter::writeBinaryStep (plate/Exporter.h:27-207): the face Gauss-point rows
    [X, Y, u, v, w, rotX_deg, rotY_deg, fields...], the PCA flatness of the deformed
    point cloud, and the per-crease-point dihedral chained along each crease;
  * ``StepWriter`` stores what writeBinaryStep stores (dataset step_NNNNN, its
    step_NNNNN_creases companion and the attributes angles, is_driver, disp, W_ext,
    E_mem, E_ben, E_hin, planar_rms, planar_max, ref_diag) as one .npz per step: HDF5 (the
    reference's container) is not available in this environment;
  * ``StressSettings`` / ``stress_rays`` = StressSampler::report (plate/StressSampler.h:
    60-170): points every dr along rays from a tip, their shape functions built on the GPU
    (stage A's second caller), and the membrane / bending / surface stresses per point,
    written as the reference's per-ray CSV files.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

POINT_STATE_COLUMNS = ("u", "v", "w", "rX_x", "rX_y", "rX_z", "rY_x", "rY_y", "rY_z",
                       "rXX_x", "rXX_y", "rXX_z", "rYY_x", "rYY_y", "rYY_z", "rXY_x", "rXY_y", "rXY_z",
                       "b_x", "b_y", "b_z", "E0_xx", "E0_yy", "E0_xy", "E1_xx", "E1_yy", "E1_xy",
                       "N_xx", "N_yy", "N_xy", "M_xx", "M_yy", "M_xy")
assert len(POINT_STATE_COLUMNS) == L.POINT_STATE_COLS
_COL = {n: i for i, n in enumerate(POINT_STATE_COLUMNS)}

# Exporter's optional columns (Exporter.h:66-78): membrane strain and curvature, tensor form.
FIELDS = {"E_XX": "E0_xx", "E_YY": "E0_yy", "E_XY": "E0_xy", "K_XX": "E1_xx", "K_YY": "E1_yy", "K_XY": "E1_xy"}


def point_state(ctx, shapes, x, A, B, D) -> np.ndarray:
    """(n_points, 33) kinematic state rows of a shape set at x (cgb_point_state)."""
    x = np.ascontiguousarray(x, np.float64)
    A, B, D = (np.ascontiguousarray(M, np.float64).reshape(9) for M in (A, B, D))
    out = np.zeros((max(shapes.n_gp, 1), L.POINT_STATE_COLS))
    ctx.check(ctx.lib.cgb_point_state(ctx.h, shapes.h, x.ctypes.data, A.ctypes.data, B.ctypes.data,
                                      D.ctypes.data, out.ctypes.data))
    return out[: shapes.n_gp]


_warned = set()


def step_table(face_xy, state: np.ndarray, fields=()) -> np.ndarray:
    """Exporter rows of the face Gauss points: [X, Y, u, v, w, rotX_deg, rotY_deg] and one
    column per requested field; an unknown field name gives a column of zeros and one
    warning (Exporter.h:80-89)."""
    xy = np.asarray(face_xy, np.float64)
    n = len(xy)
    out = np.empty((n, 7 + len(fields)))
    out[:, 0:2] = xy
    out[:, 2:5] = state[:, 0:3]
    bx, by, bz = state[:, _COL["b_x"]], state[:, _COL["b_y"]], state[:, _COL["b_z"]]
    out[:, 5] = np.degrees(np.arctan2(-by, bz))
    out[:, 6] = np.degrees(np.arctan2(bx, bz))
    for k, f in enumerate(fields):
        if f in FIELDS:
            out[:, 7 + k] = state[:, _COL[FIELDS[f]]]
        else:
            if f not in _warned:
                _warned.add(f)
                print(f'!!! WARNING: unknown output field "{f}" - writing zeros. Valid names: E_XX, E_YY, E_XY,'
                      f' K_XX, K_YY, K_XY.', file=sys.stderr)
            out[:, 7 + k] = 0.0
    return out


def planarity(table: np.ndarray):
    """(planar_rms, planar_max, ref_diag): the RMS and largest distance of the deformed
    points (X+u, Y+v, w) from their best-fit plane (smallest-eigenvalue direction of the
    covariance), and the diagonal of the reference bounding box (Exporter.h:101-131)."""
    if len(table) <= 2:
        return 0.0, 0.0, 0.0
    P = np.stack([table[:, 0] + table[:, 2], table[:, 1] + table[:, 3], table[:, 4]], axis=1)
    mean = P.mean(axis=0)
    d = P - mean
    Cv = d.T @ d / len(P)
    w, V = np.linalg.eigh(Cv)
    n = V[:, 0]
    rms = math.sqrt(max(0.0, float(w[0])))
    mx = float(np.abs(d @ n).max())
    diag = math.hypot(float(table[:, 0].max() - table[:, 0].min()), float(table[:, 1].max() - table[:, 1].min()))
    return rms, mx, diag


def chain_order(xy) -> list:
    """Crease points chained nearest-neighbour from one end of the farthest pair
    (Exporter.h:167-188; first index wins ties)."""
    P = np.asarray(xy, np.float64)
    n = len(P)
    if n == 0:
        return []
    best, start = -1.0, 0
    for i in range(n):
        d = ((P[i + 1:] - P[i]) ** 2).sum(axis=1)
        if len(d) and d.max() > best:
            j = int(np.argmax(d))
            best, start = float(d[j]), i
    used = np.zeros(n, bool)
    order = [start]
    used[start] = True
    cur = start
    for _ in range(1, n):
        d = ((P - P[cur]) ** 2).sum(axis=1)
        d[used] = np.inf
        nxt = int(np.argmin(d))
        if not np.isfinite(d[nxt]):
            break
        used[nxt] = True
        order.append(nxt)
        cur = nxt
    return order


def crease_table(folds) -> np.ndarray:
    """Rows [fold_index, crease_tag, X_ref, Y_ref, s_arc, theta_deg, weight] per crease point,
    chained along each crease; s_arc is the midpoint of each point's weight along the chain
    (Exporter.h:143-207). folds: (fold_index, crease_tag, left xy, weight, theta_deg) per fold."""
    rows = []
    for fi, tag, xy, w, th in folds:
        s_acc = 0.0
        for i in chain_order(xy):
            rows.append((fi, tag, xy[i][0], xy[i][1], s_acc + 0.5 * w[i], th[i], w[i]))
            s_acc += w[i]
    return np.asarray(rows, np.float64).reshape(-1, 7)


class StepWriter:
    """writeBinaryStep's content, one .npz per step: <stem>_step_NNNNN.npz holding `data`
    (the face rows), `columns`, `creases` (+ `crease_columns`) and the attributes."""

    def __init__(self, stem: str):
        self.stem = stem
        self.failed_writes = 0

    def path(self, step: int) -> str:
        return f"{self.stem}_step_{step:05d}.npz"

    def write(self, step: int, table: np.ndarray, fields, creases: np.ndarray, angles=(), is_driver=(),
              disp=0.0, W_ext=0.0, E_mem=0.0, E_ben=0.0, E_hin=0.0) -> bool:
        rms, mx, diag = planarity(table)
        cols = ["X", "Y", "u", "v", "w", "rotX_deg", "rotY_deg"] + list(fields)
        try:
            np.savez(self.path(step), data=table, columns=np.array(cols), creases=creases,
                     crease_columns=np.array("fold_index,crease_tag,X_ref,Y_ref,s_arc,theta_deg,weight".split(",")),
                     angles=np.asarray(list(angles) or [0.0], np.float64),
                     is_driver=np.asarray(list(is_driver) or [0], np.int32), disp=disp, W_ext=W_ext, E_mem=E_mem,
                     E_ben=E_ben, E_hin=E_hin, planar_rms=rms, planar_max=mx, ref_diag=diag)
        except OSError as e:
            print(f"!!! step {step} write FAILED -> {self.path(step)}: {e}", file=sys.stderr)
            self.failed_writes += 1
            return False
        return True


def export_step(model, x, step, fields=(), fold_tags=None, writer: StepWriter | None = None, **attrs):
    """Exporter::writeBinaryStep over a PlateModel (api.py): the face rows and the
    crease-point dihedrals from the GPU's shape functions at x. Returns (table, creases);
    writes them when a writer is given."""
    from . import solver as S

    p = model.plate
    A, B, D = model.asm.A, model.asm.B, model.asm.D
    st = point_state(model.ctx, model.faces, x, A, B, D)
    table = step_table(p.faces.xy, st, fields)
    folds = []
    for fi, ((Ls, Rs), fd) in enumerate(zip(model.fold_sets, p.folds)):
        sL = point_state(model.ctx, Ls, x, A, B, D)
        sR = point_state(model.ctx, Rs, x, A, B, D)
        F12 = np.concatenate([sL[:, 3:9], sR[:, 3:9]], axis=1)
        th, _ = S.fold_angle_and_grad(F12, fd.left.tangent[:, 0], fd.left.tangent[:, 1])
        tag = fold_tags[fi] if fold_tags else fi
        folds.append((fi, tag, np.asarray(fd.left.xy), np.asarray(fd.left.weight), np.degrees(th)))
    cr = crease_table(folds)
    if writer is not None:
        writer.write(step, table, fields, cr, **attrs)
    return table, cr


# ---- the stress sampler (plate/StressSampler.h) ----------------------------------------------

@dataclass
class StressSettings:
    tip: tuple = (0.0, 0.0)
    dir: tuple = (1.0, 0.0)
    r_max: float = 0.0
    dr: float = 0.0
    angles_deg: list = field(default_factory=list)   # empty: -170 .. 170 every 10
    steps: list = field(default_factory=list)        # empty: every step
    stem: str = "stress"


STRESS_COLUMNS = ("r,X,Y,sig_nn_top,sig_nn_bot,tau_nt_top,tau_nt_bot,sig_nn_max,Nnn_over_h,Nnt_over_h,Mnn,"
                  "S_nn_top,S_nn_bot,J_top,J_bot,n_neighbours")


def surface_stress(state: np.ndarray, Q: np.ndarray, z: float, N2: np.ndarray, T2: np.ndarray):
    """(sig_nn, tau_nt, S_nn, J) at height z of every point (StressSampler::atSurface,
    StressSampler.h:32-48): E = E0 + z E1, S = Q E (second Piola-Kirchhoff), F = F0 + z F0 C0^-1 E1,
    sigma = F S F^T / J, n the deformed image of the normal N, t of the tangent T."""
    c = _COL
    E0 = np.stack([[state[:, c["E0_xx"]], state[:, c["E0_xy"]]], [state[:, c["E0_xy"]], state[:, c["E0_yy"]]]])
    E1 = np.stack([[state[:, c["E1_xx"]], state[:, c["E1_xy"]]], [state[:, c["E1_xy"]], state[:, c["E1_yy"]]]])
    E0 = np.moveaxis(E0, -1, 0)
    E1 = np.moveaxis(E1, -1, 0)
    E = E0 + z * E1
    s = np.einsum("ij,nj->ni", Q, np.stack([E[:, 0, 0], E[:, 1, 1], 2.0 * E[:, 0, 1]], axis=1))
    Sm = np.stack([np.stack([s[:, 0], s[:, 2]], 1), np.stack([s[:, 2], s[:, 1]], 1)], 1)
    F0 = np.stack([state[:, 3:6], state[:, 6:9]], axis=2)                     # (n, 3, 2)
    C0 = np.einsum("nki,nkj->nij", F0, F0)
    C0i = np.linalg.inv(C0)
    F = F0 + z * np.einsum("nij,njk,nkl->nil", F0, C0i, E1)
    Cm = np.einsum("nki,nkj->nij", F, F)
    J = np.sqrt(np.linalg.det(Cm))
    sigma = np.einsum("nij,njk,nlk->nil", F, Sm, F) / J[:, None, None]
    n = np.einsum("nij,njk,k->ni", F, np.linalg.inv(Cm), N2)
    n /= np.linalg.norm(n, axis=1)[:, None]
    t = np.einsum("nij,j->ni", F, T2)
    t /= np.linalg.norm(t, axis=1)[:, None]
    return (np.einsum("ni,nij,nj->n", n, sigma, n), np.einsum("ni,nij,nj->n", t, sigma, n),
            np.einsum("i,nij,j->n", N2, Sm, N2), J)


def distance_to_cut(X, cut) -> float:
    V = np.asarray(cut["vertices"], np.float64)
    n = len(V)
    closed = bool(cut.get("is_closed", False))
    best = math.inf
    i = 0
    while i + 1 < n or (closed and i < n):
        A, v = V[i], V[(i + 1) % n] - V[i]
        v2 = float(v @ v)
        t = max(0.0, min(1.0, float((X - A) @ v) / v2)) if v2 > 0.0 else 0.0
        best = min(best, float(np.hypot(*(X - (A + t * v)))))
        i += 1
    return best


def stress_rays(model, x, step: int, settings: StressSettings, creases, h: float, write: bool = True):
    """StressSampler::report: per ray, the sample points' shape functions on the GPU (a ray
    whose support is rank-deficient is skipped with a warning, as the reference does), their
    kinematic state at x, resultants and surface stresses (Q = A / h). Returns
    {angle: (n, 16) rows in STRESS_COLUMNS order}; writes <stem>_s<step>_p<angle>.csv."""
    from .api import shape_functions

    s = settings
    if s.r_max <= 0.0 or s.dr <= 0.0:
        return {}
    if s.steps and step not in s.steps:
        return {}
    p = model.plate
    A, B, D = model.asm.A, model.asm.B, model.asm.D
    Q = np.asarray(A, np.float64).reshape(3, 3) / h
    lo, hi = p.node_xy.min(axis=0), p.node_xy.max(axis=0)
    angles = list(s.angles_deg) or list(range(-170, 171, 10))
    phi0 = math.atan2(s.dir[1], s.dir[0])
    nr = int(math.floor(s.r_max / s.dr + 1e-9))
    tip = np.asarray(s.tip, np.float64)
    out = {}
    kw = dict(rho=p.rho, order=p.order, creases=creases, rho_node=p.rho_node, kernel=p.kernel)
    for a in angles:
        phi = phi0 + math.radians(a)
        T = np.array([math.cos(phi), math.sin(phi)])
        N = np.array([-T[1], T[0]])
        pts, rr = [], []
        for i in range(1, nr + 1):
            X = tip + (i * s.dr) * T
            if X[0] < lo[0] or X[0] > hi[0] or X[1] < lo[1] or X[1] > hi[1]:
                break
            if any(distance_to_cut(X, c) < 1e-9 * p.rho for c in creases):
                continue
            pts.append(X)
            rr.append(i * s.dr)
        if not pts:
            continue
        try:
            sh = shape_functions(model.ctx, np.asarray(pts), **kw)
        except L.CGBError as e:
            print(f"!!! WARNING: stress sampler: ray at {a:g} deg skipped ({e})", file=sys.stderr)
            continue
        st = point_state(model.ctx, sh, x, A, B, D)
        nn = np.diff(sh.download()["ptr"])
        top = surface_stress(st, Q, 0.5 * h, N, T)
        bot = surface_stress(st, Q, -0.5 * h, N, T)
        Nr = np.stack([np.stack([st[:, 27], st[:, 29]], 1), np.stack([st[:, 29], st[:, 28]], 1)], 1)
        Mr = np.stack([np.stack([st[:, 30], st[:, 32]], 1), np.stack([st[:, 32], st[:, 31]], 1)], 1)
        P = np.asarray(pts)
        rows = np.column_stack([rr, P[:, 0], P[:, 1], top[0], bot[0], top[1], bot[1], np.maximum(top[0], bot[0]),
                                np.einsum("i,nij,j->n", N, Nr, N) / h, np.einsum("i,nij,j->n", T, Nr, N) / h,
                                np.einsum("i,nij,j->n", N, Mr, N), top[2], bot[2], top[3], bot[3], nn])
        out[a] = rows
        if write:
            path = f"{s.stem}_s{step}_p{int(round(a)):+04d}.csv"
            with open(path, "w") as f:
                f.write(f"# stress along a ray from the tip, step={step}, tip_x={tip[0]:.12g}, tip_y={tip[1]:.12g}, "
                        f"dir_x={s.dir[0]:.12g}, dir_y={s.dir[1]:.12g}, phi_deg={a:.6g}, h={h:.12g}, "
                        f"rho={p.rho:.12g}, order={p.order}\n")
                f.write(STRESS_COLUMNS + "\n")
                for r in rows:
                    f.write(",".join([f"{r[0]:.10g}", f"{r[1]:.10g}", f"{r[2]:.10g}"] +
                                     [f"{v:.10e}" for v in r[3:13]] + [f"{r[13]:.12g}", f"{r[14]:.12g}",
                                                                        str(int(r[15]))]) + "\n")
    return out
