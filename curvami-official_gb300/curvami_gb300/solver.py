"""Host Newton driver around the GPU assembly.

The reference keeps its Newton / arc-length drivers and the KKT factorisation on the host;
this module restates the parts a static load-stepping run needs, so that the GPU assembly
can be driven exactly as the reference drives its own:

  * ``ContinuationSolver.line_search`` = ContinuationSolver::LineSearch
    (core/include/curvami/solver/ContinuationSolver.h:185-322): projected-residual merit,
    backtracking by halving (6 trials, accept when <= 1.05 x the current merit), the
    geometric corrector, convergence on max force / energy change / geometry error;
  * ``initialize_topology`` / ``filter_rows`` = InitializeTopology / filterRows
    (ContinuationSolver.h:101-161): independent constraint rows by column-pivoted QR of J^T;
  * ``_Projector`` = ConstraintProjector (core/include/curvami/solver/ConstraintProjector.h):
    minimum-norm corrector and null-space projection through (J J^T);
  * ``PlateProblem`` = PlateProblem (plate/PlateProblem.h:50-90) over Meshless:
    assemble / internal force through the GPU assembler (Meshless::assembleSystem*,
    plate/Meshless.h:102-127), external force (Meshless::computeExternalForce,
    Meshless.h:60-100, plus a face pressure: the reference loads points, edges and folds
    only), constraints (Meshless::evaluateConstraints, Meshless.h:129-195, with
    Constraints::evaluateDirichlet, plate/Constraints.h:24-54, and the pointwise
    Constraints::evaluateFold, Constraints.h:243-306);
  * the KKT system [K J^T; J 0] is solved by a sparse direct LU (SciPy SuperLU) standing in
    for the reference's symmetric MUMPS (MumpsSymmetricSolver.h:116-146 takes the upper
    triangle of K and J^T); MUMPS is not available here.

The assembly is a backend object with ``pattern()`` and ``assemble(x, want_K)``, so the
same driver runs over the GPU library or over any other implementation of the same call.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import _lib as L


# ---- domains and boundary conditions ----------------------------------------------------

@dataclass
class BoundaryCondition:
    """BoundaryCondition (plate/PlateData.h:35-50)."""
    active_u: bool = False
    active_v: bool = False
    active_w: bool = False
    val_u: float = 0.0
    val_v: float = 0.0
    val_w: float = 0.0
    active_rot: bool = False
    val_rot: float = 0.0
    force: tuple = (0.0, 0.0, 0.0)


@dataclass
class LineDomain:
    """Gauss points of an edge (or point) domain: one per segment at its midpoint with the
    segment length as weight, the normal the tangent turned by +90 degrees
    (core/include/curvami/Quadrature.h:99-128)."""
    xy: np.ndarray
    weight: np.ndarray
    tangent: np.ndarray
    normal: np.ndarray
    bc: BoundaryCondition = field(default_factory=BoundaryCondition)


def line_domain(vertices, bc: BoundaryCondition) -> LineDomain:
    v = np.asarray(vertices, np.float64)
    p1, p2 = v[:-1], v[1:]
    t = p2 - p1
    length = np.linalg.norm(t, axis=1)
    keep = length > 0
    p1, p2, t, length = p1[keep], p2[keep], t[keep], length[keep]
    t = t / length[:, None]
    n = np.stack([-t[:, 1], t[:, 0]], axis=1)
    return LineDomain(0.5 * p1 + 0.5 * p2, length.copy(), t, n, bc)


def clamped_edge(p0, p1, n_segments: int) -> LineDomain:
    """u = v = w = 0 and zero normal slope on every edge Gauss point (the reference's
    clamped support, main.cpp:228-247)."""
    v = np.linspace(np.asarray(p0, np.float64), np.asarray(p1, np.float64), n_segments + 1)
    return line_domain(v, BoundaryCondition(True, True, True, 0.0, 0.0, 0.0, True, 0.0))


class ShapeTable:
    """Psi and its gradient of one domain's Gauss points as sparse (n_gp x n_nodes)
    operators: P @ X gives the displacement at the points, Dx @ X, Dy @ X its gradient."""

    def __init__(self, ptr, idx, psi, dpsi, n_nodes: int):
        ptr = np.asarray(ptr, np.int64)
        idx = np.asarray(idx, np.int64)
        dpsi = np.asarray(dpsi, np.float64).reshape(-1, 2)
        n = len(ptr) - 1
        self.n_gp, self.n_nodes = n, n_nodes
        self.ptr, self.idx = ptr, idx
        self.psi = np.asarray(psi, np.float64)
        self.dpsi = dpsi
        shape = (n, n_nodes)
        self.P = sp.csr_matrix((self.psi, idx, ptr), shape=shape)
        self.Dx = sp.csr_matrix((dpsi[:, 0].copy(), idx, ptr), shape=shape)
        self.Dy = sp.csr_matrix((dpsi[:, 1].copy(), idx, ptr), shape=shape)

    @classmethod
    def from_shape_set(cls, shapes, n_nodes: int):
        d = shapes.download()
        return cls(d["ptr"], d["idx"], d["psi"], d["dpsi"], n_nodes)

    def rows(self):
        """Gauss point of every entry."""
        return np.repeat(np.arange(self.n_gp), np.diff(self.ptr))


# ---- fold angle (plate/Constraints.h:71-119), vectorised over crease points ---------------

def fold_angle_and_grad(F12: np.ndarray, tx: np.ndarray, ty: np.ndarray):
    """theta = atan2(-s, c) of every crease point and d theta / d F (12) for F packed as
    (a1L, a2L, a1R, a2R); Constraints::foldAngleAndGrad."""
    a1L, a2L, a1R, a2R = F12[:, 0:3], F12[:, 3:6], F12[:, 6:9], F12[:, 9:12]
    nL, nR = np.cross(a1L, a2L), np.cross(a1R, a2R)
    normL = np.linalg.norm(nL, axis=1)
    normR = np.linalg.norm(nR, axis=1)
    bL, bR = nL / normL[:, None], nR / normR[:, None]
    aT = a1L * tx[:, None] + a2L * ty[:, None]
    norm_aT = np.linalg.norm(aT, axis=1)
    t = aT / norm_aT[:, None]
    c = np.einsum("ij,ij->i", bL, bR)
    s = np.einsum("ij,ij->i", np.cross(bL, bR), t)
    theta = np.arctan2(-s, c)

    def db_dF(a1, a2, b, norm_n):
        # (I - b b^T) / |n| * dn/dF, dn/dF(:, i) = e_i x a2, dn/dF(:, 3+i) = a1 x e_i
        eye = np.eye(3)
        dn = np.empty((len(a1), 3, 6))
        for i in range(3):
            dn[:, :, i] = np.cross(np.broadcast_to(eye[i], a2.shape), a2)
            dn[:, :, 3 + i] = np.cross(a1, np.broadcast_to(eye[i], a1.shape))
        proj = eye[None] - b[:, :, None] * b[:, None, :]
        return np.einsum("nij,njk->nik", proj, dn) / norm_n[:, None, None]

    dbL = db_dF(a1L, a2L, bL, normL)
    dbR = db_dF(a1R, a2R, bR, normR)
    daT = np.zeros((len(tx), 3, 6))
    for r in range(3):
        daT[:, r, r] = tx
        daT[:, r, 3 + r] = ty
    proj_t = np.eye(3)[None] - t[:, :, None] * t[:, None, :]
    dt = np.einsum("nij,njk->nik", proj_t, daT) / norm_aT[:, None, None]
    dc_dFL = np.einsum("ni,nij->nj", bR, dbL)
    dc_dFR = np.einsum("ni,nij->nj", bL, dbR)
    ds_dFL = np.einsum("ni,nij->nj", np.cross(bR, t), dbL) + np.einsum("ni,nij->nj", np.cross(bL, bR), dt)
    ds_dFR = np.einsum("ni,nij->nj", np.cross(t, bL), dbR)
    denom = c * c + s * s
    inv = np.where(denom > 1e-14, 1.0 / np.where(denom > 1e-14, denom, 1.0), 0.0)
    grad = np.empty((len(tx), 12))
    grad[:, :6] = -(c[:, None] * ds_dFL - s[:, None] * dc_dFL) * inv[:, None]
    grad[:, 6:] = -(c[:, None] * ds_dFR - s[:, None] * dc_dFR) * inv[:, None]
    return theta, grad


# ---- the problem --------------------------------------------------------------------------

@dataclass
class FoldSides:
    """One Fold for the constraint rows: both sides' shape tables and the crease data.
    active / theta0_gp: Fold::gp_active / gp_theta0 (None = every point active / the
    scalar theta0), as progressive creasing sets them (plate/ProgressiveCreasing.h:621-639)."""
    left: ShapeTable
    right: ShapeTable
    tangent: np.ndarray
    theta0: float = 0.0
    rigid: bool = False
    active: np.ndarray | None = None
    theta0_gp: np.ndarray | None = None
    Kt: float = 0.0                      # hinge stiffness (the arc-length drivers' pseudo-load)
    weight: np.ndarray | None = None     # the left points' weights (fold angle and gradient)


class GpuAssembly:
    """Backend over the GPU assembler (NonLinearAssembler of api.py)."""

    def __init__(self, assembler, mixed: bool = False, deterministic: bool = False, exact_hinge: bool = False):
        """exact_hinge: the hinge tangent with the dihedral Hessian (Meshless::fold_exact_tangent)."""
        self.asm = assembler
        self.extra = ((L.MIXED if mixed else 0) | (L.DETERMINISTIC if deterministic else 0) |
                      (L.HINGE_EXACT if exact_hinge else 0))

    def pattern(self):
        return self.asm.pattern()

    def set_fold_theta0(self, fold: int, theta0: float):
        """Fold::Ang0 of one fold: its hinge's rest angle at every crease point."""
        self.asm.set_fold_state(fold, theta0)

    def assemble(self, x, want_K: bool, hinge: bool = True):
        flags = self.extra | (L.HINGE if hinge else 0)
        if want_K:
            return self.asm.assemble(x, flags | L.TANGENT)
        # residual only: the FP64 residual is the same in both precisions
        return None, self.asm.assemble(x, flags & ~L.TANGENT)[1]


class PlateProblem:
    """PlateProblem (plate/PlateProblem.h:50-90) of a plate whose assembly is ``backend``.

    flag_rig: folds are rigid constraints (no hinge force, a fold-angle row per crease
    point) instead of elastic hinges, as Meshless::assembleSystem / evaluateConstraints do
    for flagRig (plate/Meshless.h:113-127, Constraints.h:280-304)."""

    def __init__(self, n_nodes: int, backend, faces: ShapeTable, face_weight, face_load=None,
                 edges=(), folds=(), flag_rig: bool = False, points=()):
        self.n_nodes = n_nodes
        self.ns = 3 * n_nodes
        self.backend = backend
        self.faces = faces
        self.face_weight = np.asarray(face_weight, np.float64)
        self.face_load = None if face_load is None else np.asarray(face_load, np.float64)
        self.points = list(points)        # (LineDomain of point Gauss points, ShapeTable)
        self.edges = list(edges)          # (LineDomain, ShapeTable)
        self.folds = list(folds)          # FoldSides
        self.flag_rig = flag_rig
        outer, inner = backend.pattern()
        self.outer = np.asarray(outer, np.int64)
        self.inner = np.asarray(inner, np.int64)
        cols = np.repeat(np.arange(self.ns), np.diff(self.outer))
        self._upper = self.inner <= cols  # MUMPS reads the upper triangle (row <= col)
        self._f_ext = None
        self.n_assemble = 0
        self.n_residual = 0

    def num_dofs(self) -> int:
        return self.ns

    def set_fold_theta0(self, f: int, theta0: float):
        """Fold::Ang0 of fold f (the rest angle of its hinge and the target of its rigid
        row), as the arc-length drivers move it (NonLinearSolver.h:636-641)."""
        self.folds[f].theta0 = float(theta0)
        self.folds[f].theta0_gp = None
        self.backend.set_fold_theta0(f, float(theta0))

    # Meshless::assembleSystem: K (stored upper, symmetric) and F_int.
    def assemble(self, x):
        vals, F = self.backend.assemble(x, True, hinge=not self.flag_rig)
        self.n_assemble += 1
        vals = np.where(self._upper, vals, 0.0)
        K = sp.csc_matrix((vals, self.inner, self.outer), shape=(self.ns, self.ns))
        return K, F

    def internal_force(self, x):
        self.n_residual += 1
        return self.backend.assemble(x, False, hinge=not self.flag_rig)[1]

    # Meshless::computeExternalForce: dead loads, independent of x.
    def external_force(self, x=None):
        if self._f_ext is None:
            F = np.zeros(self.ns)
            if self.face_load is not None and np.any(self.face_load != 0.0):
                w = self.faces.P.T @ self.face_weight       # sum_g w_g Psi_I(x_g)
                for d in range(3):
                    F[d::3] += w * self.face_load[d]
            for dom, tab in self.points + self.edges:
                f = np.asarray(dom.bc.force, np.float64)
                if np.any(f != 0.0):
                    w = tab.P.T @ dom.weight
                    for d in range(3):
                        F[d::3] += w * f[d]
            self._f_ext = F
        return self._f_ext

    # Meshless::evaluateConstraints: c(x) and J(x), rows in the reference's order.
    def constraints(self, x):
        X = np.asarray(x, np.float64).reshape(-1, 3)
        c_parts, rows, cols, vals = [], [], [], []
        row = 0

        def add_rows(r_of_entry, col_nodes, comp, v):
            rows.append(row + r_of_entry)
            cols.append(3 * col_nodes + comp)
            vals.append(v)

        for dom, tab in self.points + self.edges:      # points first (Meshless.h:166-172)
            bc = dom.bc
            U = tab.P @ X
            UX, UY = tab.Dx @ X, tab.Dy @ X
            e_gp = tab.rows()
            per_gp = []   # (value, entries) per active row kind, in u v w rot order
            if bc.active_u: per_gp.append(("u", U[:, 0] - bc.val_u))
            if bc.active_v: per_gp.append(("v", U[:, 1] - bc.val_v))
            if bc.active_w: per_gp.append(("w", U[:, 2] - bc.val_w))
            if bc.active_rot:
                nx, ny = dom.normal[:, 0], dom.normal[:, 1]
                per_gp.append(("rot", (UX[:, 2] * nx + UY[:, 2] * ny) - bc.val_rot))
            k = len(per_gp)
            if k == 0:
                continue
            cvals = np.stack([v for _, v in per_gp], axis=1).reshape(-1)   # gp-major
            c_parts.append(cvals)
            for slot, (kind, _) in enumerate(per_gp):
                r = e_gp * k + slot
                if kind == "rot":
                    nx, ny = dom.normal[e_gp, 0], dom.normal[e_gp, 1]
                    add_rows(r, tab.idx, 2, tab.dpsi[:, 0] * nx + tab.dpsi[:, 1] * ny)
                else:
                    comp = {"u": 0, "v": 1, "w": 2}[kind]
                    add_rows(r, tab.idx, comp, tab.psi)
            row += k * tab.n_gp

        for f in self.folds:
            # Rows of the active crease points only, in point order (Constraints.h:263-266).
            Lt, Rt = f.left, f.right
            n_all = Lt.n_gp
            act = np.ones(n_all, bool) if f.active is None or len(f.active) == 0 else np.asarray(f.active) != 0
            slot = np.cumsum(act) - 1                     # row group of each active point
            n = int(act.sum())
            jump = (Lt.P @ X - Rt.P @ X)[act]
            k = 4 if self.flag_rig else 3
            cv = np.zeros((n, k))
            cv[:, :3] = jump
            eL, eR = Lt.rows(), Rt.rows()
            mL, mR = act[eL], act[eR]
            for d in range(3):
                add_rows(slot[eL[mL]] * k + d, Lt.idx[mL], d, Lt.psi[mL])
                add_rows(slot[eR[mR]] * k + d, Rt.idx[mR], d, -Rt.psi[mR])
            if self.flag_rig and n:
                F12 = np.empty((n_all, 12))
                F12[:, 0:3] = Lt.Dx @ X; F12[:, 3:6] = Lt.Dy @ X
                F12[:, 6:9] = Rt.Dx @ X; F12[:, 9:12] = Rt.Dy @ X
                F12[:, 0] += 1.0; F12[:, 4] += 1.0; F12[:, 6] += 1.0; F12[:, 10] += 1.0
                theta, g = fold_angle_and_grad(F12, f.tangent[:, 0], f.tangent[:, 1])
                th0 = f.theta0 if f.theta0_gp is None or len(f.theta0_gp) == 0 else np.asarray(f.theta0_gp)
                cv[:, 3] = (theta - th0)[act] if np.ndim(th0) else theta[act] - th0
                for side, tab, e, m in ((0, Lt, eL, mL), (6, Rt, eR, mR)):
                    em = e[m]
                    for d in range(3):
                        v = g[em, side + d] * tab.dpsi[m, 0] + g[em, side + 3 + d] * tab.dpsi[m, 1]
                        add_rows(slot[em] * k + 3, tab.idx[m], d, v)
            c_parts.append(cv.reshape(-1))
            row += k * n

        c = np.concatenate(c_parts) if c_parts else np.zeros(0)
        if rows:
            J = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                              shape=(row, self.ns))
        else:
            J = sp.csr_matrix((0, self.ns))
        return c, J


# ---- constraint handling (ContinuationSolver.h, ConstraintProjector.h) -------------------

class _Projector:
    """ConstraintProjector: (J J^T) factorised once, used for the corrector and the
    projection; a least-squares fallback when the Gram matrix is not positive definite.
    J stays sparse (a few nonzeros per row), so the Gram matrix costs the sparse product,
    not a dense one over every dof."""

    def __init__(self, J):
        self.J = sp.csr_matrix(J) if sp.issparse(J) else np.asarray(J)
        self.chol = None
        self.gram = None
        if self.J.shape[0]:
            G = self.J @ self.J.T
            self.gram = G.toarray() if sp.issparse(G) else np.asarray(G)
            try:
                self.chol = sla.cho_factor(self.gram)
            except np.linalg.LinAlgError:
                self.chol = None

    def _solve(self, rhs):
        if self.chol is not None:
            out = sla.cho_solve(self.chol, rhs)
            if np.all(np.isfinite(out)):
                return out
        return np.linalg.lstsq(self.gram, rhs, rcond=None)[0]

    def corrector(self, c, ns):
        if len(c) == 0:
            return np.zeros(ns)
        return self.J.T @ self._solve(-c)

    def project(self, R):
        if self.J.shape[0] == 0:
            return R
        return R - self.J.T @ self._solve(self.J @ R)


def gmres_ir(A, lu, piv, b, tol=1e-12, restart=30, max_cycles=4):
    """Solve A x = b (torch FP64, any device) with GMRES in FP64, right-preconditioned by an
    LU factorisation made in lower precision (lu, piv: torch.linalg.lu_factor of A in FP32,
    the factors then held in FP64 so that the preconditioner is applied in FP64 and stays
    linear): GMRES-based iterative refinement (Carson and Higham, SIAM J. Sci. Comput. 40
    (2018) A817-A847), which converges for condition numbers far beyond the reach of plain
    refinement with the same LU. Arnoldi with classical Gram-Schmidt applied twice; the
    small least-squares problem is solved every step to read the residual. Returns (x,
    relative residual ||b - A x|| / ||b||, GMRES steps)."""
    import torch

    def M(v):
        return torch.linalg.lu_solve(lu, piv, v.unsqueeze(1)).squeeze(1)

    bn = float(torch.linalg.vector_norm(b))
    if bn == 0.0:
        return torch.zeros_like(b), 0.0, 0
    x = M(b)
    steps = 0
    rel = float("inf")
    n = b.numel()
    for _ in range(max_cycles):
        r = b - A @ x
        rn = float(torch.linalg.vector_norm(r))
        prev, rel = rel, rn / bn
        if rel <= tol or rel > 0.5 * prev:     # converged, or at the attainable floor
            break
        m = min(restart, n)
        V = torch.zeros((n, m + 1), dtype=b.dtype, device=b.device)
        H = torch.zeros((m + 1, m), dtype=b.dtype, device=b.device)
        V[:, 0] = r / rn
        e1 = torch.zeros(m + 1, dtype=b.dtype, device=b.device)
        e1[0] = rn
        y = None
        k = 0
        for j in range(m):
            w = A @ M(V[:, j])
            for _ in range(2):
                h = V[:, : j + 1].T @ w
                w = w - V[:, : j + 1] @ h
                H[: j + 1, j] += h
            H[j + 1, j] = torch.linalg.vector_norm(w)
            k = j + 1
            steps += 1
            y = torch.linalg.lstsq(H[: j + 2, : j + 1], e1[: j + 2].unsqueeze(1)).solution.squeeze(1)
            res = float(torch.linalg.vector_norm(e1[: j + 2] - H[: j + 2, : j + 1] @ y))
            if res <= tol * bn or float(H[j + 1, j]) <= 1e-300:
                break
            V[:, j + 1] = w / H[j + 1, j]
        x = x + M(V[:, :k] @ y)
    r = b - A @ x
    return x, float(torch.linalg.vector_norm(r)) / bn, steps


class _KKT:
    """One factorisation of [K J^T; J 0] (K given by its upper triangle), reusable for
    several right-hand sides:
      "host":         sparse LU on the host (SciPy SuperLU);
      "device":       dense FP64 LU on the GPU;
      "device_mixed": dense LU in FP32 on the GPU (GB300 runs FP32 at 62x its FP64 rate) of
                      the symmetrically equilibrated matrix, then GMRES in FP64 preconditioned
                      by that LU (gmres_ir) to a residual <= 1e-12 of the right-hand side or
                      its attainable floor; a solve that ends above 1e-9 falls back to an FP64
                      LU (made on first need). Plain refinement with the FP32 LU stalls on the larger plates'
                      KKT matrices (condition beyond 1e8), GMRES does not.
    The two device modes stand in for the reference's symmetric MUMPS as direct solvers."""

    stats = {"solves": 0, "refine_steps": 0, "fallbacks": 0}   # refine_steps: GMRES steps
    _last_rows = None   # size of the last device factorisation

    def __init__(self, K_upper, J, kkt="host", device="cuda"):
        """device: where the two dense modes run (a torch device; "cuda" for the GPU)."""
        if kkt not in ("host", "device", "device_mixed"):
            raise ValueError("kkt must be 'host', 'device' or 'device_mixed'")
        self.ns = K_upper.shape[0]
        self.nc = J.shape[0]
        self.mode = kkt
        self.device = kkt != "host"
        if self.device:
            import torch

            # A KKT of another size (the constraint rows change as a crease grows) cannot reuse
            # the blocks torch's allocator cached for the last one; give those back, or the cache
            # grows with every size until it holds the whole device.
            if _KKT._last_rows is not None and _KKT._last_rows != self.ns + self.nc:
                torch.cuda.empty_cache()
            _KKT._last_rows = self.ns + self.nc
            # Only the nonzeros cross to the GPU and the dense symmetric matrix is formed
            # there: K's stored upper triangle into both triangles, J into its two blocks
            # (no sparse symmetrisation or block assembly on the host).
            Kc = K_upper.tocsc()
            kr = Kc.indices.astype(np.int64)
            kc = np.repeat(np.arange(self.ns, dtype=np.int64), np.diff(Kc.indptr))
            keep = kr <= kc
            kr, kc, kv = kr[keep], kc[keep], Kc.data[keep]
            Jo = J.tocoo()
            n = self.ns + self.nc
            dev = device
            self.dev = dev
            dense = torch.zeros((n, n), dtype=torch.float64, device=dev)
            r = torch.from_numpy(kr).to(dev)
            c = torch.from_numpy(kc).to(dev)
            v = torch.from_numpy(kv).to(dev)
            dense.index_put_((r, c), v, accumulate=True)
            off = r != c
            dense.index_put_((c[off], r[off]), v[off], accumulate=True)
            if self.nc:
                jr = torch.from_numpy(Jo.row.astype(np.int64) + self.ns).to(dev)
                jc = torch.from_numpy(Jo.col.astype(np.int64)).to(dev)
                jv = torch.from_numpy(Jo.data).to(dev)
                dense.index_put_((jr, jc), jv, accumulate=True)
                dense.index_put_((jc, jr), jv, accumulate=True)
            if kkt == "device":
                self.lu, self.piv = torch.linalg.lu_factor(dense)
            else:
                # D A D with D = |diag|^-1/2 (the constraint rows, zero on the diagonal,
                # by their largest entry), then FP32 LU of the scaled matrix.
                d = dense.diagonal().abs()
                big = dense.abs().amax(dim=1)
                self.scale = torch.where(d > 0, d, big).clamp_min(1e-300).rsqrt()
                self.As = self.scale[:, None] * dense * self.scale[None, :]
                lu32, self.piv = torch.linalg.lu_factor(self.As.float())
                self.lu = lu32.double()      # the FP32 factors, applied in FP64
                self.lu64 = None
        else:
            K = K_upper + sp.triu(K_upper, k=1).T
            A = sp.bmat([[K, J.T], [J, None]], format="csc") if self.nc else K.tocsc()
            self.lu = spla.splu(A)

    def _refined(self, b):
        import torch

        bs = b * self.scale
        x, rel, steps = gmres_ir(self.As, self.lu, self.piv, bs)
        _KKT.stats["refine_steps"] += steps
        if not rel <= 1e-9:
            _KKT.stats["fallbacks"] += 1
            if self.lu64 is None:
                self.lu64 = torch.linalg.lu_factor(self.As)
            x = torch.linalg.lu_solve(self.lu64[0], self.lu64[1], bs.unsqueeze(1)).squeeze(1)
        return x * self.scale

    def solve(self, rhs):
        b = np.ascontiguousarray(rhs[: self.ns + self.nc], dtype=np.float64)
        _KKT.stats["solves"] += 1
        if self.device:
            import torch

            bd = torch.from_numpy(b).to(self.dev)
            if self.mode == "device_mixed":
                return self._refined(bd).cpu().numpy()
            return torch.linalg.lu_solve(self.lu, self.piv, bd.unsqueeze(1)).squeeze(1).cpu().numpy()
        return self.lu.solve(b)


class ContinuationSolver:
    """LineSearch of ContinuationSolver (ContinuationSolver.h:185-322) with its defaults."""

    def __init__(self, tol_force=1e-8, tol_energy=1e-8, tol_geom=1e-12, ls_max_iters=500, div=1e7,
                 ls_fail_on_no_descent=False, verbose=False, kkt="host", refine_steps=0):
        """kkt: "host" solves the KKT system with a sparse LU on the host (SciPy SuperLU);
        "device" with a dense FP64 LU on the GPU (torch.linalg.lu_factor), for runs whose
        host factorisations would dominate; "device_mixed" with a dense FP32 LU on the GPU
        refined against the FP64 residual (see _KKT). All stand in for MUMPS.

        refine_steps: iterative refinement of each Newton step against the FP64 residual, for
        a tangent formed in lower precision (the mixed assembly's FP32 K): the action of the
        true tangent on the step is a central difference of the FP64 internal force
        (two residual-only assemblies), and the correction reuses the KKT factorisation. 0
        (the default) is the reference's algorithm exactly."""
        if kkt not in ("host", "device", "device_mixed"):
            raise ValueError("kkt must be 'host', 'device' or 'device_mixed'")
        self.kkt = kkt
        self.refine_steps = int(refine_steps)
        self.tol_force, self.tol_energy, self.tol_geom = tol_force, tol_energy, tol_geom
        self.ls_max_iters, self.div = ls_max_iters, div
        self.ls_fail_on_no_descent = ls_fail_on_no_descent
        self.verbose = verbose
        self.ind_rows = np.zeros(0, np.int64)
        self.last_ls_iters = 0
        self.last_ls_attempts = 0
        self.history = []   # (iteration, merit, energy change, geometry error, alpha)
        # Per iteration of the last line_search, its decisions, for comparing runs: a dict with
        # the iteration j, the merit (max projected force), the energy change and geometry
        # error its convergence test saw, whether it converged there, and the halvings tried
        # as (alpha, trial merit).
        self.ls_trace = []

    def initialize_topology(self, J):
        """Independent rows of J: column-pivoted QR of J^T, |R_ii| above
        max(rows, cols) * eps * max |R_ii| (ContinuationSolver.h:101-136)."""
        if J.shape[0] == 0 or J.shape[1] == 0:
            self.ind_rows = np.zeros(0, np.int64)
            return
        Jt = (J.toarray() if sp.issparse(J) else np.asarray(J)).T
        if not np.all(np.isfinite(Jt)):
            raise RuntimeError("Constraint Jacobian contains NaN or Inf.")
        _, R, perm = sla.qr(Jt, mode="economic", pivoting=True)
        d = np.abs(np.diag(R))
        tol = max(J.shape) * np.finfo(np.float64).eps * (d.max() if len(d) else 0.0)
        self.ind_rows = np.sort(perm[: len(d)][d > tol]).astype(np.int64)

    def filter_rows(self, J):
        return J[self.ind_rows] if J.shape[0] else J

    @staticmethod
    def with_load_stiffness(prob, K, x, lam):
        """applyLoadStiffness (ContinuationSolver.h:84-95): K - lambda K_load when the problem
        supplies a load stiffness (``load_stiffness(x)`` returning its upper triangle), else K
        unchanged."""
        f = getattr(prob, "load_stiffness", None)
        if f is None:
            return K
        KL = f(x)
        if KL is None:
            return K
        if KL.shape != K.shape:
            raise ValueError(f"loadStiffness: K_load is {KL.shape[0]}x{KL.shape[1]}, K is {K.shape[0]}x{K.shape[1]}")
        return (sp.csc_matrix(K) - lam * sp.csc_matrix(KL)).tocsc()

    @staticmethod
    def kkt_solve(K_upper, J, rhs, kkt="host"):
        """[K J^T; J 0] sol = rhs with K given by its upper triangle."""
        return _KKT(K_upper, J, kkt).solve(rhs)

    def line_search(self, prob: PlateProblem, lam: float, d: np.ndarray) -> bool:
        ns = d.size
        if ns != prob.num_dofs():
            raise ValueError(f"LineSearch: state vector has {ns} entries, problem has {prob.num_dofs()} DOFs")
        d0 = d.copy()
        self.last_ls_iters = -1
        self.history = []
        self.ls_trace = []
        c_all, J_all = prob.constraints(d)
        self.initialize_topology(J_all)
        nc = len(self.ind_rows)
        energy_change = 1.0
        for j in range(1, self.ls_max_iters + 1):
            self.last_ls_attempts = j
            c_all, J_all = prob.constraints(d)
            J_ind = self.filter_rows(J_all)
            c_ind = c_all[self.ind_rows]
            R = prob.internal_force(d) - lam * prob.external_force(d)
            proj = _Projector(J_ind)
            max_force = float(np.abs(proj.project(R)).max())
            geom_error = float(np.abs(c_ind).max()) if nc else 0.0
            if j > 1 and max_force <= self.tol_force and energy_change <= self.tol_energy and \
                    geom_error <= self.tol_geom:
                self.last_ls_iters = j
                self.ls_trace.append({"j": j, "merit": max_force, "energy_change": energy_change,
                                      "geom_error": geom_error, "converged": True, "trials": []})
                return True
            if max_force >= self.div or np.isnan(max_force):
                d[:] = d0
                return False
            K, _ = prob.assemble(d)
            K = self.with_load_stiffness(prob, K, d, lam)
            xb = proj.corrector(c_ind, ns)
            Kxb = K @ xb + sp.triu(K, k=1).T @ xb         # selfadjointView<Upper> * xb
            rhs = np.zeros(ns + nc)
            rhs[:ns] = -(R + Kxb)
            kkt = _KKT(K, J_ind, self.kkt)
            sol = kkt.solve(rhs)
            if not np.all(np.isfinite(sol)):
                d[:] = d0
                return False
            dx, mu = sol[:ns].copy(), sol[ns:].copy()
            if self.refine_steps:
                Fint = R + lam * prob.external_force(d)
                for _ in range(self.refine_steps):
                    step = xb + dx
                    sn = float(np.abs(step).max())
                    if sn == 0.0:
                        break
                    h = np.cbrt(np.finfo(np.float64).eps) * max(1.0, float(np.abs(d).max())) / sn
                    Kv = (prob.internal_force(d + h * step) - prob.internal_force(d - h * step)) / (2.0 * h)
                    r = np.zeros(ns + nc)
                    r[:ns] = -(Fint - lam * prob.external_force(d)) - Kv - (J_ind.T @ mu if nc else 0.0)
                    if nc:
                        r[ns:] = -(J_ind @ dx)
                    corr = kkt.solve(r)
                    dx += corr[:ns]
                    mu += corr[ns:]
            alpha, descended = 1.0, False
            d_trial = d
            tried = []
            self.ls_trace.append({"j": j, "merit": max_force, "energy_change": energy_change if j > 1 else None,
                                  "geom_error": geom_error, "converged": False, "trials": tried})
            for iarm in range(1, 7):
                d_trial = d + xb + alpha * dx
                R_trial = prob.internal_force(d_trial) - lam * prob.external_force(d_trial)
                c_t, J_t = prob.constraints(d_trial)
                trial = float(np.abs(_Projector(self.filter_rows(J_t)).project(R_trial)).max())
                tried.append((alpha, trial))
                if trial <= 1.05 * max_force:
                    descended = True
                    break
                alpha *= 0.5
            if not descended and self.ls_fail_on_no_descent:
                d[:] = d0
                return False
            d[:] = d_trial
            energy_change = abs(float((xb + alpha * dx) @ R))
            self.history.append((j, trial, energy_change, geom_error, alpha))
            if self.verbose:
                print(f"{j:3d}      {trial:12.5e}         {energy_change:12.5e}         {geom_error:12.5e}")
        d[:] = d0
        return False


def tracking_displacement(prob: PlateProblem, x) -> float:
    """trackingDisplacement (plate/PlateProblem.h:14-44), the scalar the reference's
    continuation exports per step: the mean displacement along the load direction over the
    Gauss points of every loaded point and edge domain (|force| > 1e-12); with no loaded
    domain, the mean deflection w over the nodes. (Fold domains carry no loads here.)"""
    X = np.asarray(x, np.float64).reshape(-1, 3)
    total, count = 0.0, 0
    for dom, tab in list(prob.points) + list(prob.edges):
        f = np.asarray(dom.bc.force, np.float64)
        if np.linalg.norm(f) > 1e-12:
            u = tab.P @ X
            total += float((u @ (f / np.linalg.norm(f))).sum())
            count += tab.n_gp
    if count > 0:
        return total / count
    return float(X[:, 2].mean())


def load_steps(solver: ContinuationSolver, prob: PlateProblem, lambdas, x0=None, traces=None):
    """Static load stepping: one LineSearch per load factor, each starting from the
    previous solution. Returns the converged states and the Newton iterations per step
    (LineSearch's count: the converging check is iteration j, so j - 1 tangent solves).
    traces: a list that receives each step's line-search trace (solver.ls_trace)."""
    x = np.zeros(prob.num_dofs()) if x0 is None else np.array(x0, np.float64)
    states, iters = [], []
    for lam in lambdas:
        ok = solver.line_search(prob, float(lam), x)
        if traces is not None:
            traces.append(list(solver.ls_trace))
        if not ok:
            raise RuntimeError(f"LineSearch failed to converge at load factor {lam}")
        states.append(x.copy())
        iters.append(solver.last_ls_iters)
    return states, iters


def first_divergence(ref_traces, traces, tol_force=None, tol_energy=None):
    """Where two runs' line-search decisions first differ, from their traces (ls_trace per
    load step): the load step and Newton iteration, and
    - for a halving one run accepted and the other rejected: its index and, per run, the
      ratio trial / (1.05 merit) that decided it (<= 1 accepts);
    - for a convergence test one run passed and the other failed: each run's merit and
      energy change there, and their ratios to the tolerances when given.
    None when every decision agrees."""
    def conv_info(e):
        out = {"merit": e["merit"], "energy_change": e["energy_change"]}
        if tol_force:
            out["merit_over_tol"] = e["merit"] / tol_force
        if tol_energy and e["energy_change"] is not None:
            out["energy_over_tol"] = e["energy_change"] / tol_energy
        return out

    for k, (ra, rb) in enumerate(zip(ref_traces, traces)):
        for ea, eb in zip(ra, rb):
            if ea["converged"] != eb["converged"]:
                return {"step": k, "iteration": ea["j"], "kind": "convergence test",
                        "ref": conv_info(ea), "run": conv_info(eb)}
            if ea["converged"]:
                break
            ta, tb = ea["trials"], eb["trials"]
            ma, mb = ea["merit"], eb["merit"]
            for h in range(max(len(ta), len(tb))):
                acc_a = h < len(ta) and ta[h][1] <= 1.05 * ma
                acc_b = h < len(tb) and tb[h][1] <= 1.05 * mb
                if h >= len(ta) or h >= len(tb) or acc_a != acc_b:
                    ratio = lambda t, m: (t[h][1] / (1.05 * m)) if h < len(t) else None  # noqa: E731
                    return {"step": k, "iteration": ea["j"], "kind": "halving", "halving": h,
                            "ratio_ref": ratio(ta, ma), "ratio_run": ratio(tb, mb),
                            "merit_rel_diff": abs(ma - mb) / abs(ma) if ma else None}
    return None


def gpu_problem(model, face_load=None, edges=(), mixed: bool = False, deterministic: bool = False,
                flag_rig: bool = False, points=(), exact_hinge: bool = False) -> PlateProblem:
    """PlateProblem of a PlateModel (api.py): the GPU's shape functions for the faces, the
    folds, every edge domain and every point domain (LineDomain of point supports), and its
    assembler as the backend."""
    from .api import shape_functions
    p = model.plate
    n = len(p.node_xy)
    kw = dict(rho=p.rho, order=p.order, creases=p.creases, rho_node=p.rho_node, kernel=p.kernel)
    model.ctx.set_nodes(p.node_xy)
    faces = ShapeTable.from_shape_set(model.faces, n)
    sides = []
    for (Ls, Rs), fd in zip(model.fold_sets, p.folds):
        sides.append(FoldSides(ShapeTable.from_shape_set(Ls, n), ShapeTable.from_shape_set(Rs, n),
                               np.asarray(fd.left.tangent, np.float64), fd.theta0, fd.rigid,
                               Kt=fd.Kt, weight=np.asarray(fd.left.weight, np.float64)))
    edge_tables = [(dom, ShapeTable.from_shape_set(shape_functions(model.ctx, dom.xy, **kw), n)) for dom in edges]
    point_tables = [(dom, ShapeTable.from_shape_set(shape_functions(model.ctx, dom.xy, **kw), n)) for dom in points]
    return PlateProblem(n, GpuAssembly(model.asm, mixed, deterministic, exact_hinge), faces, p.faces.weight,
                        face_load=face_load, edges=edge_tables, folds=sides, flag_rig=flag_rig,
                        points=point_tables)
