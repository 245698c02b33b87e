"""Domain-integral energy release rate of a crease tip (plate/JIntegral.h) over the GPU state.

For a ring rho1 < |X - tip| < rho2 around the tip,

    G_vec = (1/h) sum_g w_g B_g grad q(X_g),    B = C0 N + 2 E1 M - W_h I,

with C0 = F0^T F0, N and M the resultants as 2x2 tensors, E1 the bending strain and
W_h = 1/2 (N . e0 + M . e1) (JIntegral.h:17-44). The per-point inputs are one call of
cgb_point_state on the face Gauss points (Kinematics::compute + Constitutive::evaluate on
the GPU, 33 values per point); the ring sums are vectorised on the host.

Restated from ``JIntegral::compute`` (JIntegral.h:420-535), with its names: G (analytic q),
G_c (B less its ring mean, the quadrature leak removed), G_h (q interpolated from its nodal
values by the shape functions, the first-order term cancelled by nodal equilibrium), G_d
(displacement-gradient form), G_m / G_mc (mixed form), G_s (first-order part subtracted
through the virtual work vw), vw1_h (the same virtual work with the interpolated q, equal to
the nodal residual sum_I q_I d . F_int,I), abs_sum, grad_q_sum, and the main CSV of
``JIntegral::report`` (JIntegral.h:751-916) with its columns.

Not restated: the fold terms of a ring that a crease crosses (the one-sided B, f_n, f_T,
G_fold, G_tip, the band, tie-work and line terms of JIntegral.h:535-750 and their _fold.csv /
_crease.csv files), and the natural-curvature band term (the assembly here has no natural
curvature, so Gband is zero and G1b_h = G1_h, as in the reference without one). Rings that
a fold crosses get the plate part only.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Ring:
    rho1: float
    rho2: float


@dataclass
class Settings:
    """JIntegral::Settings (JIntegral.h:171-182): tip, direction of advance d, rings, q shape."""
    tip: tuple = (0.0, 0.0)
    dir: tuple = (1.0, 0.0)
    rings: list = field(default_factory=list)
    linear_q: bool = False


def q_value(rho, r: Ring, linear_q: bool):
    """qValue (JIntegral.h:264-270), vectorised over rho."""
    rho = np.asarray(rho, np.float64)
    t = np.clip((rho - r.rho1) / (r.rho2 - r.rho1), 0.0, 1.0)
    q = 1.0 - t if linear_q else 1.0 - 3.0 * t * t + 2.0 * t * t * t
    return np.where(rho <= r.rho1, 1.0, np.where(rho >= r.rho2, 0.0, q))


def _tensors(state: np.ndarray):
    """Per-point F0 (n,3,2), C0, N, M, E1 (n,2,2), W_h, b, r_XX, r_YY, r_XY from cgb_point_state
    rows: u, r_X, r_Y, r_XX, r_YY, r_XY, b, E0 (xx yy xy), E1 (xx yy xy), N, M (Voigt)."""
    st = np.asarray(state, np.float64)
    a1, a2 = st[:, 3:6], st[:, 6:9]
    F0 = np.stack([a1, a2], axis=2)
    C0 = np.einsum("nki,nkj->nij", F0, F0)

    def sym(v):
        return np.stack([np.stack([v[:, 0], v[:, 2]], 1), np.stack([v[:, 2], v[:, 1]], 1)], 1)

    N, M = sym(st[:, 27:30]), sym(st[:, 30:33])
    E1 = sym(st[:, 24:27])
    e0 = st[:, 21:24] * np.array([1.0, 1.0, 2.0])
    e1 = st[:, 24:27] * np.array([1.0, 1.0, 2.0])
    W = 0.5 * (np.einsum("ni,ni->n", st[:, 27:30], e0) + np.einsum("ni,ni->n", st[:, 30:33], e1))
    return dict(F0=F0, C0=C0, N=N, M=M, E1=E1, W=W, Nv=st[:, 27:30], Mv=st[:, 30:33], b=st[:, 18:21],
                rXX=st[:, 9:12], rYY=st[:, 12:15], rXY=st[:, 15:18])


def eshelby(T):
    """eshelbyB (JIntegral.h:272-302): B, B_d and C0 N per point."""
    I2 = np.eye(2)[None]
    FN = np.einsum("nij,njk->nik", T["F0"], T["N"])
    CN = np.einsum("nij,njk->nik", T["C0"], T["N"])
    EM2 = 2.0 * np.einsum("nij,njk->nik", T["E1"], T["M"])
    WI = T["W"][:, None, None] * I2
    H = T["F0"].copy()
    H[:, 0, 0] -= 1.0
    H[:, 1, 1] -= 1.0
    Bd = np.einsum("nki,nkj->nij", H, FN) + EM2 - WI
    return CN + EM2 - WI, Bd, CN


def virtual_work(T, e, g, Hs):
    """virtualWork (JIntegral.h:225-234): N . de0 + M . de1 for the displacement variation
    f(X) e with grad f = g (n,2), grad grad f = Hs (n,2,2); vectorised over points."""
    F0 = T["F0"]
    a1, a2 = F0[:, :, 0], F0[:, :, 1]
    p1, p2 = a1 @ e, a2 @ e
    be = T["b"] @ e
    Cinv = np.linalg.inv(T["C0"])
    gI = np.einsum("nij,nj->ni", F0, np.einsum("nij,nj->ni", Cinv, g))
    de0 = np.stack([p1 * g[:, 0], p2 * g[:, 1], p1 * g[:, 1] + p2 * g[:, 0]], 1)
    de1 = np.stack([(-Hs[:, 0, 0] + np.einsum("ni,ni->n", T["rXX"], gI)) * be,
                    (-Hs[:, 1, 1] + np.einsum("ni,ni->n", T["rYY"], gI)) * be,
                    2.0 * (-Hs[:, 0, 1] + np.einsum("ni,ni->n", T["rXY"], gI)) * be], 1)
    return np.einsum("ni,ni->n", T["Nv"], de0) + np.einsum("ni,ni->n", T["Mv"], de1)


def compute_from_state(state, face_xy, face_weight, node_xy, ptr, idx, dpsi, ddpsi, h: float, s: Settings):
    """JIntegral::compute's plate part from a point state (n, 33) and the faces' shape
    functions. Returns one dict per ring with the reference's RingResult names."""
    X = np.asarray(face_xy, np.float64)
    w = np.asarray(face_weight, np.float64)
    node_xy = np.asarray(node_xy, np.float64)
    ptr = np.asarray(ptr, np.int64)
    idx = np.asarray(idx, np.int64)
    dpsi = np.asarray(dpsi, np.float64).reshape(-1, 2)
    ddpsi = np.asarray(ddpsi, np.float64).reshape(-1, 3)
    n = len(X)
    rows = np.repeat(np.arange(n), np.diff(ptr))
    tip = np.asarray(s.tip, np.float64)
    d = np.asarray(s.dir, np.float64)
    d = d / np.linalg.norm(d)
    dperp = np.array([-d[1], d[0]])
    d3, dperp3 = np.array([d[0], d[1], 0.0]), np.array([dperp[0], dperp[1], 0.0])
    T = _tensors(state)
    B, Bd, CN = eshelby(T)
    rvec = X - tip
    rho = np.linalg.norm(rvec, axis=1)
    rnode = np.linalg.norm(node_xy - tip, axis=1)
    out = []
    for r in s.rings:
        R = dict(rho1=r.rho1, rho2=r.rho2)
        # interpolated q (every point whose support sees q vary)
        qI = q_value(rnode, r, s.linear_q)[idx]
        gh = np.zeros((n, 2))
        Hh = np.zeros((n, 2, 2))
        for c in range(2):
            gh[:, c] = np.bincount(rows, weights=qI * dpsi[:, c], minlength=n)
        Hh[:, 0, 0] = np.bincount(rows, weights=qI * ddpsi[:, 0], minlength=n)
        Hh[:, 1, 1] = np.bincount(rows, weights=qI * ddpsi[:, 1], minlength=n)
        Hh[:, 0, 1] = Hh[:, 1, 0] = np.bincount(rows, weights=qI * ddpsi[:, 2], minlength=n)
        qmin = np.full(n, 2.0)
        qmax = np.full(n, -1.0)
        np.minimum.at(qmin, rows, qI)
        np.maximum.at(qmax, rows, qI)
        mh = qmax > qmin
        Bg = np.einsum("nij,nj->ni", B, gh)
        Gh = (w[mh, None] * Bg[mh]).sum(0)
        Gm = (w[mh, None] * np.einsum("nij,nj->ni", CN, gh)[mh]).sum(0)
        vw1_h = float((w[mh] * virtual_work({k: v[mh] for k, v in T.items()}, d3, gh[mh], Hh[mh])).sum())
        abs_sum_h = float((w[mh] * np.abs(Bg[mh] @ d)).sum())
        # analytic q on the ring
        ma = (rho > r.rho1) & (rho < r.rho2)
        width = r.rho2 - r.rho1
        t = (rho[ma] - r.rho1) / width
        dq = (np.full_like(t, -1.0) if s.linear_q else (-6.0 * t + 6.0 * t * t)) / width
        d2q = (np.zeros_like(t) if s.linear_q else (-6.0 + 12.0 * t)) / (width * width)
        er = rvec[ma] / rho[ma][:, None]
        gq = dq[:, None] * er
        eer = np.einsum("ni,nj->nij", er, er)
        Ha = d2q[:, None, None] * eer + (dq / rho[ma])[:, None, None] * (np.eye(2)[None] - eer)
        wa = w[ma]
        Ta = {k: v[ma] for k, v in T.items()}
        c = wa[:, None] * np.einsum("nij,nj->ni", B[ma], gq)
        G = c.sum(0)
        Gd = (wa[:, None] * np.einsum("nij,nj->ni", Bd[ma], gq)).sum(0)
        Bsum = (wa[:, None, None] * B[ma]).sum(0)
        B2sum = (wa[:, None, None] * (B[ma] - CN[ma])).sum(0)
        Gm = Gm + (wa[:, None] * np.einsum("nij,nj->ni", B[ma] - CN[ma], gq)).sum(0)
        gsum = (wa[:, None] * gq).sum(0)
        wsum = float(wa.sum())
        vw1 = float((wa * virtual_work(Ta, d3, gq, Ha)).sum())
        vw2 = float((wa * virtual_work(Ta, dperp3, gq, Ha)).sum())
        abs_sum = float(np.linalg.norm(c, axis=1).sum())
        Gc = (G - (Bsum / wsum) @ gsum) / h if wsum > 0.0 else np.zeros(2)
        Gmc = Gm - (B2sum / wsum) @ gsum if wsum > 0.0 else Gm.copy()
        G, Gd, Gh, Gm, Gmc = G / h, Gd / h, Gh / h, Gm / h, Gmc / h
        R.update(G_x=float(G[0]), G_y=float(G[1]), G1=float(d @ G), G2=float(dperp @ G),
                 G_abs=float(np.linalg.norm(G)), n_gp=int(ma.sum()), abs_sum=abs_sum / h,
                 G1_c=float(d @ Gc), G2_c=float(dperp @ Gc), G_abs_c=float(np.linalg.norm(Gc)),
                 grad_q_sum=float(np.linalg.norm(gsum)), G1_h=float(d @ Gh), G2_h=float(dperp @ Gh),
                 n_gp_h=int(mh.sum()), G1_d=float(d @ Gd), G2_d=float(dperp @ Gd), G1_m=float(d @ Gm),
                 G2_m=float(dperp @ Gm), G1_mc=float(d @ Gmc), G2_mc=float(dperp @ Gmc),
                 vw1_s=vw1 / h, vw2_s=vw2 / h, vw1_h=vw1_h / h, abs_sum_h=abs_sum_h / h)
        R["angle_deg"] = math.degrees(math.atan2(R["G2"], R["G1"]))
        R["G1_s"], R["G2_s"] = R["G1"] - R["vw1_s"], R["G2"] - R["vw2_s"]
        R["Gband_h"] = R["Gband_a"] = R["Gband2_h"] = 0.0
        R["G1b_h"], R["G2b_h"] = R["G1_h"], R["G2_h"]
        out.append(R)
    return out


def compute(model, x, s: Settings, h: float | None = None):
    """compute_from_state with the point state of the model's faces from the GPU
    (cgb_point_state) at x; h defaults to the plate's thickness."""
    from .export import point_state

    p = model.plate
    st = point_state(model.ctx, model.faces, x, model.asm.A, model.asm.B, model.asm.D)
    dn = model.faces.download()
    return compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, dn["ptr"], dn["idx"], dn["dpsi"],
                              dn["ddpsi"], p.thickness if h is None else h, s)


CSV_COLUMNS = ["step", "ring", "rho1", "rho2", "G_x", "G_y", "G1", "G2", "G_abs", "angle_deg", "n_gp", "abs_sum",
               "G1_c", "G2_c", "G_abs_c", "grad_q_sum", "G1_h", "G2_h", "n_gp_h", "G1_d", "G2_d", "G1_m", "G2_m",
               "G1_mc", "G2_mc", "G1_s", "G2_s", "vw1_s", "vw1_h", "Gband_h", "Gband_a", "G1b_h", "Gband2_h", "G2b_h"]


def write_csv(path: str, step: int, s: Settings, results, h: float, first: bool, commit: str = "none"):
    """The main CSV of JIntegral::report (JIntegral.h:855-870): a comment line with the
    settings on the first write, then one row per ring."""
    with open(path, "w" if first else "a") as f:
        if first:
            f.write(f"# energy release rate, domain integral, git_commit={commit}, tip_x={s.tip[0]:.12g}, "
                    f"tip_y={s.tip[1]:.12g}, d_x={s.dir[0]:.12g}, d_y={s.dir[1]:.12g}, "
                    f"q={'linear' if s.linear_q else 'cubic'}, h={h:.12g}\n")
            f.write(",".join(CSV_COLUMNS) + "\n")
        for k, r in enumerate(results):
            vals = [step, k] + [r[c] for c in CSV_COLUMNS[2:]]
            f.write(",".join(f"{v:.12e}" if isinstance(v, float) else str(v) for v in vals) + "\n")
