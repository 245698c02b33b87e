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

The fold terms of a ring that a crease crosses (JIntegral.h:303-418, 551-746) are restated
over the point states of both sides of every fold (the one-sided kinematics the hinge uses):
the crease points (one-sided B, f_n, f_T, psi and d(psi)/ds), the line term, G_D, G_fold and
G_tip with the interpolated and the analytic q, the hinge virtual work, the forms with the
tie work removed (_r), the mixed and subtracted forms at a fold, and the band form
(fold_band > 0), with the _fold.csv and _crease.csv files of ``JIntegral::report``.

With a natural curvature (Kinematics::NaturalCurvature, the context's
cgb_set_natural_curvature), N, M and W_h come from the elastic bending strain E1_el = E1 +
kappa_bar while the 2 E1 M term keeps the geometric E1, and the band term (JIntegral.h:
145-166, 492-520) is added: Gband_h = -(1/h) sum_g w_g q_h M : d(kappa_bar)/dX . d, Gband2_h
the same along d_perp, Gband_a with the analytic q; G1b_h = G1_h + Gband_h, G2b_h = G2_h +
Gband2_h. Without one these are zero and G1b_h = G1_h, as in the reference.

Not restated: the console summary and the HDF5 datasets (no HDF5 library here).
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
    fold_band: float = 0.0           # half-width of the band form of G_fold; 0: not computed
    fold_band_plateau: float = 0.0   # half-width of the part of the band where chi = 1


def q_value(rho, r: Ring, linear_q: bool):
    """qValue (JIntegral.h:264-270), vectorised over rho."""
    rho = np.asarray(rho, np.float64)
    t = np.clip((rho - r.rho1) / (r.rho2 - r.rho1), 0.0, 1.0)
    q = 1.0 - t if linear_q else 1.0 - 3.0 * t * t + 2.0 * t * t * t
    return np.where(rho <= r.rho1, 1.0, np.where(rho >= r.rho2, 0.0, q))


def natural_kappa(X, nc):
    """kappa_bar_XX(X) of a natural-curvature band (Kinematics.h:25-34; nc as the config's
    "natural_curvature" object) and its X-derivative; zeros without one."""
    X = np.asarray(X, np.float64)
    if nc is None:
        return np.zeros_like(X), np.zeros_like(X)
    sign = -1.0 if nc.get("sense", "mountain") == "mountain" else 1.0
    w = float(nc["width"])
    t = (X - float(nc["x0"])) / w
    k = sign * math.radians(float(nc["angle_deg"])) * np.exp(-t * t) / (math.sqrt(math.pi) * w)
    return k, k * (-2.0 * (X - float(nc["x0"])) / (w * w))


def _tensors(state: np.ndarray, kbar=None):
    """Per-point F0 (n,3,2), C0, N, M, E1 (n,2,2), W_h, b, r_XX, r_YY, r_XY from cgb_point_state
    rows: u, r_X, r_Y, r_XX, r_YY, r_XY, b, E0 (xx yy xy), E1 (xx yy xy), N, M (Voigt). kbar:
    the natural curvature kappa_bar_XX per point (W_h from E1_el = E1 + kappa_bar; E1 stays
    the geometric curvature)."""
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
    if kbar is not None:
        e1 = e1.copy()
        e1[:, 0] += kbar
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


def q_analytic(rvec, r: Ring, linear_q: bool):
    """qAnalytic (JIntegral.h:235-249), vectorised: q, grad q (n,2), grad grad q (n,2,2)."""
    rvec = np.asarray(rvec, np.float64).reshape(-1, 2)
    rho = np.linalg.norm(rvec, axis=1)
    q = q_value(rho, r, linear_q)
    grad = np.zeros((len(rho), 2))
    hess = np.zeros((len(rho), 2, 2))
    m = (rho > r.rho1) & (rho < r.rho2)
    if m.any():
        width = r.rho2 - r.rho1
        t = (rho[m] - r.rho1) / width
        dq = (np.full_like(t, -1.0) if linear_q else (-6.0 * t + 6.0 * t * t)) / width
        d2q = (np.zeros_like(t) if linear_q else (-6.0 + 12.0 * t)) / (width * width)
        er = rvec[m] / rho[m][:, None]
        eer = np.einsum("ni,nj->nij", er, er)
        grad[m] = dq[:, None] * er
        hess[m] = d2q[:, None, None] * eer + (dq / rho[m])[:, None, None] * (np.eye(2)[None] - eer)
    return q, grad, hess


# ---- fold terms (JIntegral.h:303-418, 551-746) -------------------------------------------

@dataclass
class FoldState:
    """One fold for the fold terms: the crease data of a Fold (Meshless.h:30-46: left point
    X + 1e-7 n, right point X - 1e-7 n, n the tangent turned by +90 degrees, the left
    point's weight), both sides' point states (cgb_point_state rows) and their shape
    functions (dicts with ptr, idx, psi, dpsi), the hinge stiffness and rest angle, and the
    per-point crease state (Fold::gp_theta0 / gp_active; None = the scalar rest angle /
    every point active)."""
    left_xy: np.ndarray
    right_xy: np.ndarray
    weight: np.ndarray
    tangent: np.ndarray
    state_left: np.ndarray
    state_right: np.ndarray
    left: dict
    right: dict
    Kt: float
    theta0: float = 0.0
    rigid: bool = False
    theta0_gp: np.ndarray | None = None
    active: np.ndarray | None = None

    def __post_init__(self):
        self._angles = None

    def active_mask(self):
        """Constraints::gpActive (Constraints.h:17-19)."""
        if self.active is None or len(self.active) == 0:
            return np.ones(len(self.weight), bool)
        return np.asarray(self.active) != 0

    def theta0_at(self):
        """Constraints::gpTheta0 (Constraints.h:20-22) at every crease point."""
        if self.theta0_gp is None or len(self.theta0_gp) == 0:
            return np.full(len(self.weight), float(self.theta0))
        return np.asarray(self.theta0_gp, np.float64)

    def normal(self):
        t = np.asarray(self.tangent, np.float64).reshape(-1, 2)
        return np.stack([-t[:, 1], t[:, 0]], 1)

    def angles(self):
        """Fold angle and d theta / dF (12) at every crease point, from both sides' deformed
        tangent vectors (Constraints::foldAngleAndGrad, as the hinge computes them)."""
        if self._angles is None:
            from .solver import fold_angle_and_grad

            F12 = np.concatenate([np.asarray(self.state_left, np.float64)[:, 3:9],
                                  np.asarray(self.state_right, np.float64)[:, 3:9]], 1)
            t = np.asarray(self.tangent, np.float64).reshape(-1, 2)
            with np.errstate(divide="ignore", invalid="ignore"):
                self._angles = fold_angle_and_grad(F12, t[:, 0], t[:, 1])
        return self._angles


def _side_sums(sh: dict, g):
    """Per point of one side: sum_I g_I Psi_I, sum_I g_I grad Psi_I (n,2), sum_I g_I."""
    ptr = np.asarray(sh["ptr"], np.int64)
    idx = np.asarray(sh["idx"], np.int64)
    n = len(ptr) - 1
    rows = np.repeat(np.arange(n), np.diff(ptr))
    gi = np.asarray(g, np.float64)[idx]
    dp = np.asarray(sh["dpsi"], np.float64).reshape(-1, 2)
    val = np.bincount(rows, weights=gi * np.asarray(sh["psi"], np.float64), minlength=n)
    grad = np.stack([np.bincount(rows, weights=gi * dp[:, 0], minlength=n),
                     np.bincount(rows, weights=gi * dp[:, 1], minlength=n)], 1)
    return val, grad, np.bincount(rows, weights=gi, minlength=n)


def _hinge_work(f: FoldState, keep, ggL, ggR, dirv) -> float:
    """sum_k w_k Kt (theta - theta0) dtheta_k over the kept points, for the in-plane shift
    whose gradient is ggL on the left side and ggR on the right."""
    if not keep.any():
        return 0.0
    theta, grad = f.angles()
    e = np.array([dirv[0], dirv[1], 0.0])
    dth = ((grad[:, 0:3] @ e) * ggL[:, 0] + (grad[:, 3:6] @ e) * ggL[:, 1]
           + (grad[:, 6:9] @ e) * ggR[:, 0] + (grad[:, 9:12] @ e) * ggR[:, 1])
    m = f.Kt * (theta - f.theta0_at())
    return float((np.asarray(f.weight, np.float64) * m * dth)[keep].sum())


def hinge_virtual_work(folds, g, dirv) -> float:
    """hingeVirtualWork (JIntegral.h:361-389): the hinges' virtual work for the in-plane
    virtual displacement with nodal values g_I dir, over the active points of the elastic
    folds."""
    work = 0.0
    for f in folds:
        if f.rigid or len(f.weight) == 0:
            continue
        _, ggL, _ = _side_sums(f.left, g)
        _, ggR, _ = _side_sums(f.right, g)
        keep = f.active_mask() & (((ggL ** 2).sum(1) > 0.0) | ((ggR ** 2).sum(1) > 0.0))
        work += _hinge_work(f, keep, ggL, ggR, dirv)
    return work


def hinge_virtual_work_analytic(folds, dirv, grad_at) -> float:
    """hingeVirtualWorkAnalytic (JIntegral.h:391-418): the same for an analytic shift
    f(X) dir, grad f = grad_at(X) (vectorised, (n,2) -> (n,2)) taken at the crease point
    and used on both sides."""
    work = 0.0
    for f in folds:
        if f.rigid or len(f.weight) == 0:
            continue
        X = 0.5 * (np.asarray(f.left_xy, np.float64) + np.asarray(f.right_xy, np.float64))
        gg = np.asarray(grad_at(X), np.float64).reshape(-1, 2)
        keep = f.active_mask() & ((gg ** 2).sum(1) > 0.0)
        work += _hinge_work(f, keep, gg, gg, dirv)
    return work


def dpsi_ds(s, psi, T, T0):
    """d(psi)/ds along each point's own tangent (JIntegral.h:343-356): points ordered by
    s = T0 . X, central differences between the neighbours in that order, one-sided at the
    two ends, 0 where the two neighbours share s."""
    s = np.asarray(s, np.float64)
    psi = np.asarray(psi, np.float64)
    K = len(s)
    out = np.zeros(K)
    if K == 0:
        return out
    order = np.argsort(s, kind="stable")
    m = np.arange(K)
    a = order[np.maximum(m - 1, 0)]
    b = order[np.minimum(m + 1, K - 1)]
    ds = s[b] - s[a]
    d = np.where(ds > 0.0, (psi[b] - psi[a]) / np.where(ds > 0.0, ds, 1.0), 0.0)
    sign = np.where(np.asarray(T, np.float64)[order] @ np.asarray(T0, np.float64) < 0.0, -1.0, 1.0)
    out[order] = d * sign
    return out


def crease_points(folds) -> list:
    """creasePoints (JIntegral.h:303-359): per fold, the arrays of its active crease points
    (fold, i, X, T, n, s, w, theta, theta0, psi, dpsi_ds, Bp, Bm, fn, fT, the one-sided
    resultants N_nn, N_Tn, M_nn and the hinge moment), in point order; folds without
    active points are left out."""
    out = []
    for fi, f in enumerate(folds):
        i = np.nonzero(f.active_mask())[0]
        if len(i) == 0:
            continue
        T = np.asarray(f.tangent, np.float64).reshape(-1, 2)[i]
        n = f.normal()[i]
        X = 0.5 * (np.asarray(f.left_xy, np.float64)[i] + np.asarray(f.right_xy, np.float64)[i])
        theta = f.angles()[0][i]
        th0 = f.theta0_at()[i]
        psi = np.zeros(len(i)) if f.rigid else 0.5 * f.Kt * (theta - th0) ** 2
        TL = _tensors(np.asarray(f.state_left, np.float64)[i])
        TR = _tensors(np.asarray(f.state_right, np.float64)[i])
        Bp, Bm = eshelby(TL)[0], eshelby(TR)[0]
        s = X @ T[0]
        dps = dpsi_ds(s, psi, T, T[0])
        Bpn, Bmn = np.einsum("nij,nj->ni", Bp, n), np.einsum("nij,nj->ni", Bm, n)
        jump = Bpn - Bmn

        def nt(A, a, b):
            return np.einsum("ni,nij,nj->n", a, A, b)

        out.append(dict(fold=fi, i=i, X=X, T=T, n=n, s=s, w=np.asarray(f.weight, np.float64)[i],
                        theta=theta, theta0=th0, psi=psi, dpsi_ds=dps, Bp=Bp, Bm=Bm,
                        fn=-(n * jump).sum(1), fT=-(T * jump).sum(1) + dps,
                        nBn_p=(n * Bpn).sum(1), nBn_m=(n * Bmn).sum(1), TBn_p=(T * Bpn).sum(1),
                        TBn_m=(T * Bmn).sum(1), Nnn_p=nt(TL["N"], n, n), Nnn_m=nt(TR["N"], n, n),
                        NTn_p=nt(TL["N"], T, n), NTn_m=nt(TR["N"], T, n), Mnn_p=nt(TL["M"], n, n),
                        Mnn_m=nt(TR["M"], n, n),
                        m_hinge=np.zeros(len(i)) if f.rigid else f.Kt * (theta - th0)))
    return out


def compute_from_state(state, face_xy, face_weight, node_xy, ptr, idx, dpsi, ddpsi, h: float, s: Settings,
                       folds=(), F_int=None, crease_out: list | None = None, natural_curvature=None, psi=None):
    """JIntegral::compute from a point state (n, 33) and the faces' shape functions. Returns
    one dict per ring with the reference's RingResult names (the fold columns under their
    _fold.csv names). With folds (FoldState list), the fold terms are added; they need F_int,
    the plate's own nodal internal force at the same state (the face assembly without the
    hinge), and fill crease_out, when given, with the crease points of crease_points().
    natural_curvature: the band the state was computed with (its N and M already include
    it), for W_h and the band term; the band term's interpolated q needs psi."""
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
    kbar, dkbar = natural_kappa(X[:, 0], natural_curvature)
    T = _tensors(state, kbar if natural_curvature is not None else None)
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
        if natural_curvature is not None:
            # JIntegral.h:492-520: -(1/h) sum_g w_g q M_ab d_c d(kappa_bar_ab)/dX_c over the points
            # where kappa_bar varies; only kappa_bar_XX is nonzero, so M : dk = M_XX dk_XX d_X.
            thr = 1e-14 * math.radians(float(natural_curvature["angle_deg"])) / float(natural_curvature["width"]) ** 2
            m1 = T["M"][:, 0, 0] * dkbar * d[0]
            m2 = T["M"][:, 0, 0] * dkbar * dperp[0]
            live = np.abs(dkbar * d[0]) + np.abs(dkbar * dperp[0]) >= thr
            if psi is None:
                raise ValueError("the natural-curvature band term needs the faces' Psi")
            qh = np.bincount(rows, weights=qI * np.asarray(psi, np.float64), minlength=n)
            qa = q_value(rho, r, s.linear_q)
            R["Gband_h"] = float(-(w * qh * m1)[live].sum() / h)
            R["Gband2_h"] = float(-(w * qh * m2)[live].sum() / h)
            R["Gband_a"] = float(-(w * qa * m1)[live].sum() / h)
        R["G1b_h"], R["G2b_h"] = R["G1_h"] + R["Gband_h"], R["G2_h"] + R["Gband2_h"]
        for k in FOLD_COLUMNS[4:]:
            R.setdefault(k, 0.0)
        R["plate_h"], R["plate_a"], R["abs_plate_h"] = R["G1_h"], R["G1"], R["abs_sum_h"]
        R["n_crease"] = 0
        R["GD_m"], R["GD_mc"], R["GD_s"] = R["G1_m"], R["G1_mc"], R["G1_s"]
        out.append(R)
    if len(folds):
        if F_int is None:
            raise ValueError("the fold terms need F_int, the plate's nodal internal force")
        _fold_terms(out, s, list(folds), np.asarray(F_int, np.float64), h, d, dperp, node_xy, rnode, tip, X, w,
                    T, B, CN, rows, idx, dpsi, crease_out)
    return out


def _fold_terms(out, s, folds, F_int, h, d, dperp, node_xy, rnode, tip, X, w, T, B, CN, rows, idx, dpsi,
                crease_out):
    """The fold part of JIntegral::compute (JIntegral.h:551-746), added to the rings' dicts."""
    cps = crease_points(folds)
    if crease_out is not None:
        crease_out.extend(cps)
    fn_max = max((float(np.abs(c["fn"]).max()) for c in cps), default=0.0)
    fT_max = max((float(np.abs(c["fT"]).max()) for c in cps), default=0.0)
    Fx, Fy = F_int[0::3], F_int[1::3]
    qns = [q_value(rnode, r, s.linear_q) for r in s.rings]
    for R, r, qn in zip(out, s.rings, qns):
        R["fn_max"], R["fT_max"] = fn_max, fT_max
        line_h = Gfold_h = abs_fold_h = GfoldT_h = line_a = Gfold_a = dq_max = dq_a_max = 0.0
        n_crease = 0
        for c in cps:
            f = folds[c["fold"]]
            i = c["i"]
            qp, gqp, sp = (a[i] for a in _side_sums(f.left, qn))
            qm, gqm, sm = (a[i] for a in _side_sums(f.right, qn))
            dn, dT = c["n"] @ d, c["T"] @ d
            has = (sp + sm) > 0.0
            fold_n = c["w"] * dn * (-(qp * c["nBn_p"] - qm * c["nBn_m"]))
            line_h += float((c["w"] * c["psi"] * dT * 0.5 * ((c["T"] * (gqp + gqm)).sum(1)))[has].sum())
            Gfold_h += float(fold_n[has].sum())
            abs_fold_h += float(np.abs(fold_n[has]).sum())
            GfoldT_h += float((c["w"] * dT * (-(qp * c["TBn_p"] - qm * c["TBn_m"])
                                              + 0.5 * (qp + qm) * c["dpsi_ds"]))[has].sum())
            n_crease += int(has.sum())
            if has.any():
                dq_max = max(dq_max, float(np.abs(qp - qm)[has].max()))
            # analytic q
            rv = c["X"] - tip
            rh = np.linalg.norm(rv, axis=1)
            Gfold_a += float((c["w"] * q_value(rh, r, s.linear_q) * dn * c["fn"]).sum())
            inr = (rh > r.rho1) & (rh < r.rho2)
            if inr.any():
                width = r.rho2 - r.rho1
                t = (rh[inr] - r.rho1) / width
                dq = (np.full_like(t, -1.0) if s.linear_q else (-6.0 * t + 6.0 * t * t)) / width
                line_a += float((c["w"][inr] * c["psi"][inr] * dT[inr] * dq * (c["T"][inr] * rv[inr]).sum(1)
                                 / rh[inr]).sum())
            qL = q_value(np.linalg.norm(np.asarray(f.left_xy, np.float64)[i] - tip, axis=1), r, s.linear_q)
            qR = q_value(np.linalg.norm(np.asarray(f.right_xy, np.float64)[i] - tip, axis=1), r, s.linear_q)
            dq_a_max = max(dq_a_max, float(np.abs(qL - qR).max()))
        R.update(line_h=line_h / h, Gfold_h=Gfold_h / h, abs_fold_h=abs_fold_h / h, GfoldT_h=GfoldT_h / h,
                 line_a=line_a / h, Gfold_a=Gfold_a / h, n_crease=n_crease, dq_max=dq_max, dq_a_max=dq_a_max)
        R["GD_h"] = R["G1_h"] - R["line_h"]
        R["Gtip_h"] = R["GD_h"] - R["Gfold_h"]
        R["GD_a"] = R["G1"] - R["line_a"]
        R["Gtip_a"] = R["GD_a"] - R["Gfold_a"]
        # the plate's own nodal force and the hinges' virtual work: the "_r" forms
        nz = qn != 0.0
        R["resid_h"] = float((qn[nz] * (d[0] * Fx[nz] + d[1] * Fy[nz])).sum()) / h
        R["hinge_h"] = hinge_virtual_work(folds, qn, d) / h
        tie = R["resid_h"] + R["hinge_h"] + R["line_h"]
        R["GD_r"] = R["G1_h"] - tie
        R["GD_m"] = R["G1_m"] - tie
        R["GD_mc"] = R["G1_mc"] - tie

        def grad_q(Xc, r=r):
            return q_analytic(Xc - tip, r, s.linear_q)[1]

        R["hw1_s"] = hinge_virtual_work_analytic(folds, d, grad_q) / h
        R["hw2_s"] = hinge_virtual_work_analytic(folds, dperp, grad_q) / h
        R["G1_s"] = R["G1"] - R["vw1_s"] - R["hw1_s"]
        R["G2_s"] = R["G2"] - R["vw2_s"] - R["hw2_s"]
        R["GD_s"] = R["G1_s"] - R["line_a"]
    if s.fold_band > 0.0:
        _band_terms(out, s, folds, qns, Fx, Fy, h, d, node_xy, tip, X, w, T, B, CN, rows, idx, dpsi)


def _band_terms(out, s, folds, qns, Fx, Fy, h, d, node_xy, tip, X, w, T, B, CN, rows, idx, dpsi):
    """Band form of the fold's share (JIntegral.h:636-740): the release rate of the sideways
    shift g n, g = chi(eta) q (d . n), each fold taken as the straight line through its first
    crease point. Every face point is visited (the reference skips those farther than
    band + rho from the line, whose terms are all zero)."""
    band, eta0 = s.fold_band, s.fold_band_plateau
    n_pts = len(X)
    rvec = X - tip
    rho = np.linalg.norm(rvec, axis=1)
    for f in folds:
        if len(f.weight) == 0:
            continue
        nv = f.normal()[0]
        X0 = np.asarray(f.left_xy, np.float64)[0] - 1e-7 * nv
        dn = float(d @ nv)
        n3 = np.array([nv[0], nv[1], 0.0])

        def t_of(eta):
            return np.maximum(0.0, (np.abs(eta) - eta0) / (band - eta0))

        def chi(eta):
            t = t_of(eta)
            return np.where(t >= 1.0, 0.0, 1.0 - 3.0 * t * t + 2.0 * t * t * t)

        cn = chi((node_xy - X0) @ nv)
        gnodes = [np.where(cn > 0.0, cn * qn * dn, 0.0) for qn in qns]
        eta = (X - X0) @ nv
        t = t_of(eta)
        c = chi(eta)
        dc = np.where(t >= 1.0, 0.0, (-6.0 * t + 6.0 * t * t) / (band - eta0) * np.where(eta < 0.0, -1.0, 1.0))
        d2c = np.where((t >= 1.0) | (t <= 0.0), 0.0, (-6.0 + 12.0 * t) / ((band - eta0) * (band - eta0)))
        Btn = np.einsum("nji,nj->ni", B, np.broadcast_to(nv, (n_pts, 2)))
        CNtn = np.einsum("nji,nj->ni", CN, np.broadcast_to(nv, (n_pts, 2)))
        B2tn = Btn - CNtn
        for R, r, qn, g in zip(out, s.rings, qns, gnodes):
            nz = g != 0.0
            R["resid_band"] += float((g[nz] * (nv[0] * Fx[nz] + nv[1] * Fy[nz])).sum()) / h
            R["hinge_band"] += hinge_virtual_work(folds, g, nv) / h
            gi = g[idx]
            gh = np.stack([np.bincount(rows, weights=gi * dpsi[:, 0], minlength=n_pts),
                           np.bincount(rows, weights=gi * dpsi[:, 1], minlength=n_pts)], 1)
            gabs = np.bincount(rows, weights=np.abs(gi), minlength=n_pts)
            qa, gq, Hq = q_analytic(rvec, r, s.linear_q)
            ga = (dn * dc * qa)[:, None] * nv[None, :]
            inr = (c > 0.0) & (rho > r.rho1) & (rho < r.rho2)
            if inr.any():
                width = r.rho2 - r.rho1
                tq = (rho[inr] - r.rho1) / width
                dq = (np.full_like(tq, -1.0) if s.linear_q else (-6.0 * tq + 6.0 * tq * tq)) / width
                ga[inr] += (dn * c[inr] * dq / rho[inr])[:, None] * rvec[inr]
            ga2 = (ga ** 2).sum(1)
            keep = ~((gabs <= 0.0) & (ga2 <= 0.0))
            vsel = keep & ((ga2 > 0.0) | inr)
            if vsel.any():
                nn = np.outer(nv, nv)
                ngT = np.einsum("i,nj->nij", nv, gq[vsel])
                Ha = dn * (d2c[vsel, None, None] * qa[vsel, None, None] * nn[None]
                           + dc[vsel, None, None] * (ngT + ngT.transpose(0, 2, 1)) + c[vsel, None, None] * Hq[vsel])
                Tv = {k: v[vsel] for k, v in T.items()}
                R["vw_band_s"] += float((w[vsel] * virtual_work(Tv, n3, ga[vsel], Ha)).sum()) / h
            R["Gfold_band_h"] += float((w * (Btn * gh).sum(1))[keep].sum()) / h
            R["Gfold_band_a"] += float((w * (Btn * ga).sum(1))[keep].sum()) / h
            mixed = float((w * ((CNtn * gh).sum(1) + (B2tn * ga).sum(1)))[keep].sum()) / h
            gs = keep & (ga2 > 0.0)
            wasum = float(w[gs].sum())
            nB2sum = (w[gs, None] * B2tn[gs]).sum(0)
            gasum = (w[gs, None] * ga[gs]).sum(0)

            def grad_g(Xc, r=r):
                return dn * q_analytic(Xc - tip, r, s.linear_q)[1]

            R["hw_band_s"] += hinge_virtual_work_analytic(folds, nv, grad_g) / h
            R["Gfold_band_m"] += mixed
            R["Gfold_band_mc"] += mixed - (float((nB2sum / wasum) @ gasum) / h if wasum > 0.0 else 0.0)
    for R in out:
        R["Gtip_band_h"] = R["GD_h"] - R["Gfold_band_h"]
        R["Gtip_band_a"] = R["GD_a"] - R["Gfold_band_a"]
        R["Gfold_band_r"] = R["Gfold_band_h"] - R["resid_band"] - R["hinge_band"]
        R["Gtip_band_r"] = R["GD_r"] - R["Gfold_band_r"]
        R["Gfold_band_m"] -= R["resid_band"] + R["hinge_band"]
        R["Gfold_band_mc"] -= R["resid_band"] + R["hinge_band"]
        R["Gtip_band_m"] = R["GD_m"] - R["Gfold_band_m"]
        R["Gtip_band_mc"] = R["GD_mc"] - R["Gfold_band_mc"]
        R["Gfold_band_s"] = R["Gfold_band_a"] - R["vw_band_s"] - R["hw_band_s"]
        R["Gtip_band_s"] = R["GD_s"] - R["Gfold_band_s"]


def compute(model, x, s: Settings, h: float | None = None, fold_state=None, crease_out: list | None = None):
    """compute_from_state with the point states of the model's faces and fold sides from the
    GPU (cgb_point_state) at x and, with folds, the faces' nodal internal force from the GPU
    assembly (residual only, no hinge); h defaults to the plate's thickness. fold_state: per
    fold (theta0_gp, active) as set on the assembler, or None for the folds' own rest angle
    at every point, all points active."""
    from .export import point_state

    p = model.plate
    A, B_, D = model.asm.A, model.asm.B, model.asm.D
    st = point_state(model.ctx, model.faces, x, A, B_, D)
    dn = model.faces.download()
    folds, F_int = [], None
    for k, (f, (Ls, Rs)) in enumerate(zip(p.folds, model.fold_sets)):
        t0, act = (None, None) if fold_state is None or fold_state[k] is None else fold_state[k]
        ld, rd = Ls.download(), Rs.download()
        folds.append(FoldState(f.left.xy, f.right.xy, f.left.weight, f.left.tangent,
                               point_state(model.ctx, Ls, x, A, B_, D), point_state(model.ctx, Rs, x, A, B_, D),
                               ld, rd, f.Kt, f.theta0, f.rigid, t0, act))
    if folds:
        F_int = model.asm.assemble(x, 0)[1]
    return compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, dn["ptr"], dn["idx"], dn["dpsi"],
                              dn["ddpsi"], p.thickness if h is None else h, s, folds, F_int, crease_out,
                              natural_curvature=getattr(model.ctx, "natural_curvature", None), psi=dn["psi"])


CSV_COLUMNS = ["step", "ring", "rho1", "rho2", "G_x", "G_y", "G1", "G2", "G_abs", "angle_deg", "n_gp", "abs_sum",
               "G1_c", "G2_c", "G_abs_c", "grad_q_sum", "G1_h", "G2_h", "n_gp_h", "G1_d", "G2_d", "G1_m", "G2_m",
               "G1_mc", "G2_mc", "G1_s", "G2_s", "vw1_s", "vw1_h", "Gband_h", "Gband_a", "G1b_h", "Gband2_h", "G2b_h"]


FOLD_COLUMNS = ["step", "ring", "rho1", "rho2", "plate_h", "line_h", "GD_h", "Gfold_h", "Gtip_h", "GfoldT_h",
                "abs_plate_h", "abs_fold_h", "n_crease", "plate_a", "line_a", "GD_a", "Gfold_a", "Gtip_a", "fn_max",
                "fT_max", "dq_max", "Gfold_band_h", "Gtip_band_h", "Gfold_band_a", "Gtip_band_a", "resid_h",
                "hinge_h", "GD_r", "resid_band", "hinge_band", "Gfold_band_r", "Gtip_band_r", "GD_m",
                "Gfold_band_m", "Gtip_band_m", "GD_mc", "Gfold_band_mc", "Gtip_band_mc", "GD_s", "Gfold_band_s",
                "Gtip_band_s", "hw1_s", "vw_band_s", "hw_band_s", "dq_a_max"]

CREASE_COLUMNS = ["step", "fold", "i", "X", "Y", "s", "T_x", "T_y", "n_x", "n_y", "w", "theta", "theta0", "psi",
                  "dpsi_ds", "f_n", "f_T", "nBn_plus", "nBn_minus", "TBn_plus", "TBn_minus", "Nnn_plus",
                  "Nnn_minus", "NTn_plus", "NTn_minus", "Mnn_plus", "Mnn_minus", "m_hinge"]

_G_FORMAT = {"rho1": ".10g", "rho2": ".10g", "angle_deg": ".8g"}


def _row(vals, names, fmt):
    return ",".join(str(v) if isinstance(v, (int, np.integer)) else format(float(v), fmt.get(k, ".12e"))
                    for k, v in zip(names, vals)) + "\n"


def write_csv(path: str, step: int, s: Settings, results, h: float, first: bool, commit: str = "none",
              crease=None):
    """The CSV files of JIntegral::report (JIntegral.h:787-870): the main file (a comment line
    with the settings on the first write, then one row per ring) and, when crease points are
    given (the crease_out list of compute), <stem>_fold.csv (one row per ring) and
    <stem>_crease.csv (one row per crease point), stem = path less its last four characters."""
    q = "linear" if s.linear_q else "cubic"
    if crease and len(path) > 4:
        stem = path[:-4]
        with open(stem + "_fold.csv", "w" if first else "a") as f:
            if first:
                f.write(f"# fold terms of the energy release rate (along d), git_commit={commit}, "
                        f"tip_x={s.tip[0]:.12g}, tip_y={s.tip[1]:.12g}, d_x={s.dir[0]:.12g}, d_y={s.dir[1]:.12g}, "
                        f"q={q}, h={h:.12g}, fold_band={s.fold_band:.12g}, "
                        f"fold_band_plateau={s.fold_band_plateau:.12g}\n")
                f.write(",".join(FOLD_COLUMNS) + "\n")
            for k, r in enumerate(results):
                f.write(_row([step, k] + [r[c] for c in FOLD_COLUMNS[2:]], FOLD_COLUMNS, _G_FORMAT))
        cfmt = {c: ".12g" for c in ("X", "Y", "s")}
        cfmt.update({c: ".9g" for c in ("T_x", "T_y", "n_x", "n_y")})
        with open(stem + "_crease.csv", "w" if first else "a") as f:
            if first:
                f.write(f"# crease points: fold angle, hinge energy and configurational force, "
                        f"git_commit={commit}\n")
                f.write(",".join(CREASE_COLUMNS) + "\n")
            for c in crease:
                for j in range(len(c["i"])):
                    vals = [step, int(c["fold"]), int(c["i"][j]), c["X"][j, 0], c["X"][j, 1], c["s"][j],
                            c["T"][j, 0], c["T"][j, 1], c["n"][j, 0], c["n"][j, 1]]
                    vals += [c[k][j] for k in ("w", "theta", "theta0", "psi", "dpsi_ds", "fn", "fT", "nBn_p",
                                               "nBn_m", "TBn_p", "TBn_m", "Nnn_p", "Nnn_m", "NTn_p", "NTn_m",
                                               "Mnn_p", "Mnn_m", "m_hinge")]
                    f.write(_row(vals, CREASE_COLUMNS, cfmt))
    with open(path, "w" if first else "a") as f:
        if first:
            f.write(f"# energy release rate, domain integral, git_commit={commit}, tip_x={s.tip[0]:.12g}, "
                    f"tip_y={s.tip[1]:.12g}, d_x={s.dir[0]:.12g}, d_y={s.dir[1]:.12g}, "
                    f"q={q}, h={h:.12g}\n")
            f.write(",".join(CSV_COLUMNS) + "\n")
        for k, r in enumerate(results):
            f.write(_row([step, k] + [r[c] for c in CSV_COLUMNS[2:]], CSV_COLUMNS, _G_FORMAT))
