"""Seeded synthetic plates for the Gauss-point hot path.

The reference reads Gmsh meshes; no public benchmark or dataset is involved, so every
workload here is generated from a seed. The generator restates the reference's set-up
steps that shape the inputs of the hot path:

* quad quadrature, ``Quadrature::generate`` (core/include/curvami/Quadrature.h:29-44,
  154-217): bilinear map, |det J| weights, element order, ix outer / iy inner; the
  3x3 rule is the reference's, the 4x4 rule an extension;
* line quadrature of a crease with one point per segment (``line_degree = 1``,
  Quadrature.h:14-27, 99-128): midpoint, weight = length, unit tangent, normal
  (-t_y, t_x);
* fold left/right points offset by +/-1e-7 along the normal (plate/Meshless.h:30-46);
* crease Gauss points exactly on a crease split in two half-weight twins
  (plate/SetupHelper.h:60-106);
* crease end extension when an end lies on the convex hull of the nodes
  (core/include/curvami/MeshUtils.h:12-45, 112-131).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

GAUSS = {
    1: (np.array([0.0]), np.array([2.0])),
    2: (np.array([-1.0 / math.sqrt(3.0), 1.0 / math.sqrt(3.0)]), np.array([1.0, 1.0])),
    3: (np.array([-math.sqrt(3.0 / 5.0), 0.0, math.sqrt(3.0 / 5.0)]),
        np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])),
    # 4-point Gauss-Legendre: extension (the reference stops at 3x3).
    4: (np.array([-math.sqrt(3.0 / 7.0 + 2.0 / 7.0 * math.sqrt(6.0 / 5.0)),
                  -math.sqrt(3.0 / 7.0 - 2.0 / 7.0 * math.sqrt(6.0 / 5.0)),
                  math.sqrt(3.0 / 7.0 - 2.0 / 7.0 * math.sqrt(6.0 / 5.0)),
                  math.sqrt(3.0 / 7.0 + 2.0 / 7.0 * math.sqrt(6.0 / 5.0))]),
        np.array([(18.0 - math.sqrt(30.0)) / 36.0, (18.0 + math.sqrt(30.0)) / 36.0,
                  (18.0 + math.sqrt(30.0)) / 36.0, (18.0 - math.sqrt(30.0)) / 36.0])),
}


@dataclass
class PointSet:
    """Gauss points of one integration domain (faces, or one side of a fold)."""
    xy: np.ndarray                   # (n, 2)
    weight: np.ndarray               # (n,)
    tangent: np.ndarray | None = None


@dataclass
class Fold:
    left: PointSet
    right: PointSet
    Kt: float
    theta0: float = 0.0
    rigid: bool = False


@dataclass
class Plate:
    name: str
    node_xy: np.ndarray              # (n_nodes, 2)
    faces: PointSet
    creases: list                    # dicts: vertices (m,2), extend_start, extend_end, is_closed
    folds: list = field(default_factory=list)
    rho: float = 1.0
    rho_node: np.ndarray | None = None
    order: int = 2
    kernel: int = 0                  # 0 quartic (reference), 1 cubic B-spline (extension)
    E: float = 1.0
    nu: float = 0.3
    thickness: float = 0.05
    seed: int = 0
    meta: dict = field(default_factory=dict)
    points: dict = field(default_factory=dict)   # entity tag -> PointSet (mesh point elements)

    @property
    def n_nodes(self) -> int:
        return len(self.node_xy)


# ------------------------------------------------------------------------------------
# geometry helpers
# ------------------------------------------------------------------------------------

def grid_nodes(nx: int, ny: int, h: float, jitter: float = 0.0, rng=None) -> np.ndarray:
    """Row-major nx*ny node grid with spacing h; interior nodes jittered uniformly by
    +/-jitter per coordinate, boundary nodes only along their edge (so the convex hull
    stays the rectangle)."""
    xs = np.arange(nx) * h
    ys = np.arange(ny) * h
    X, Y = np.meshgrid(xs, ys)                 # (ny, nx): row j, column i
    X = X.copy(); Y = Y.copy()
    if jitter > 0.0:
        jx = rng.uniform(-jitter, jitter, size=X.shape)
        jy = rng.uniform(-jitter, jitter, size=Y.shape)
        jx[:, 0] = 0.0; jx[:, -1] = 0.0
        jy[0, :] = 0.0; jy[-1, :] = 0.0
        X += jx; Y += jy
    return np.stack([X.ravel(), Y.ravel()], axis=1)


def quad_gauss_points(node_xy: np.ndarray, nx: int, ny: int, rule: int) -> PointSet:
    """Tensor Gauss rule on every grid cell (Quadrature.h:154-217), element order row
    by row, corners (i,j),(i+1,j),(i+1,j+1),(i,j+1); within a cell ix outer, iy inner."""
    q, w = GAUSS[rule]
    jj, ii = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    ii = ii.ravel(); jj = jj.ravel()
    c0 = jj * nx + ii
    p = np.stack([node_xy[c0], node_xy[c0 + 1], node_xy[c0 + 1 + nx], node_xy[c0 + nx]], axis=1)
    XI, ETA = np.meshgrid(q, q, indexing="ij")           # ix outer, iy inner
    WX, WY = np.meshgrid(w, w, indexing="ij")
    xi = XI.ravel()[None, :]; eta = ETA.ravel()[None, :]
    N1 = 0.25 * (1.0 - xi) * (1.0 - eta)
    N2 = 0.25 * (1.0 + xi) * (1.0 - eta)
    N3 = 0.25 * (1.0 + xi) * (1.0 + eta)
    N4 = 0.25 * (1.0 - xi) * (1.0 + eta)
    px = p[:, :, 0][:, :, None]; py = p[:, :, 1][:, :, None]
    J11 = (-0.25 * (1.0 - eta) * px[:, 0] + 0.25 * (1.0 - eta) * px[:, 1]
           + 0.25 * (1.0 + eta) * px[:, 2] - 0.25 * (1.0 + eta) * px[:, 3])
    J12 = (-0.25 * (1.0 - eta) * py[:, 0] + 0.25 * (1.0 - eta) * py[:, 1]
           + 0.25 * (1.0 + eta) * py[:, 2] - 0.25 * (1.0 + eta) * py[:, 3])
    J21 = (-0.25 * (1.0 - xi) * px[:, 0] - 0.25 * (1.0 + xi) * px[:, 1]
           + 0.25 * (1.0 + xi) * px[:, 2] + 0.25 * (1.0 - xi) * px[:, 3])
    J22 = (-0.25 * (1.0 - xi) * py[:, 0] - 0.25 * (1.0 + xi) * py[:, 1]
           + 0.25 * (1.0 + xi) * py[:, 2] + 0.25 * (1.0 - xi) * py[:, 3])
    detJ = np.abs(J11 * J22 - J12 * J21)
    X = N1 * px[:, 0] + N2 * px[:, 1] + N3 * px[:, 2] + N4 * px[:, 3]
    Y = N1 * py[:, 0] + N2 * py[:, 1] + N3 * py[:, 2] + N4 * py[:, 3]
    wts = detJ * (WX.ravel() * WY.ravel())[None, :]
    return PointSet(np.stack([X.ravel(), Y.ravel()], axis=1), wts.ravel())


def convex_hull(P: np.ndarray) -> np.ndarray:
    """Monotone chain (MeshUtils.h:12-30)."""
    pts = sorted(map(tuple, P))
    if len(pts) <= 3:
        return np.array(pts)

    def cross(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

    lower, upper = [], []
    for p in pts:
        while len(lower) >= 2 and cross(lower[-2], lower[-1], p) <= 0:
            lower.pop()
        lower.append(p)
    for p in reversed(pts):
        while len(upper) >= 2 and cross(upper[-2], upper[-1], p) <= 0:
            upper.pop()
        upper.append(p)
    return np.array(lower[:-1] + upper[:-1])


def on_hull_boundary(pt, hull, tol=1e-4) -> bool:
    """MeshUtils.h:33-45."""
    n = len(hull)
    for i in range(n):
        A = hull[i]; B = hull[(i + 1) % n]
        AB = B - A
        L2 = float(AB @ AB)
        if L2 == 0:
            continue
        t = max(0.0, min(1.0, float((pt - A) @ AB) / L2))
        if np.linalg.norm(pt - (A + t * AB)) <= tol:
            return True
    return False


def make_crease(vertices: np.ndarray, node_xy: np.ndarray, hull=None) -> dict:
    """A crease polyline with the reference's hull-based end extension flags."""
    if hull is None:
        hull = convex_hull(_hull_candidates(node_xy))
    v = np.ascontiguousarray(vertices, np.float64)
    return {"vertices": v, "extend_start": on_hull_boundary(v[0], hull),
            "extend_end": on_hull_boundary(v[-1], hull), "is_closed": False}


def _hull_candidates(node_xy):
    # The hull only depends on extreme points; pre-filter for speed on big grids.
    lo = node_xy.min(0); hi = node_xy.max(0)
    span = hi - lo
    m = ((node_xy[:, 0] - lo[0] < 0.02 * span[0]) | (hi[0] - node_xy[:, 0] < 0.02 * span[0])
         | (node_xy[:, 1] - lo[1] < 0.02 * span[1]) | (hi[1] - node_xy[:, 1] < 0.02 * span[1]))
    return node_xy[m]


def crease_gauss_points(vertices: np.ndarray):
    """One Gauss point per crease segment (line_degree = 1): midpoint, weight = length,
    unit tangent p1->p2, normal (-t_y, t_x) (Quadrature.h:99-128)."""
    p1 = vertices[:-1]; p2 = vertices[1:]
    t = p2 - p1
    L = np.linalg.norm(t, axis=1)
    keep = L > 0
    p1, p2, t, L = p1[keep], p2[keep], t[keep], L[keep]
    t = t / L[:, None]
    n = np.stack([-t[:, 1], t[:, 0]], axis=1)
    X = 0.5 * p1 + 0.5 * p2
    return X, L * 1.0, t, n


def make_fold(vertices, Kt, theta0=0.0, rigid=False) -> Fold:
    """Meshless::addFold (plate/Meshless.h:30-46): left = X + 1e-7 n, right = X - 1e-7 n."""
    X, w, t, n = crease_gauss_points(np.asarray(vertices, np.float64))
    s = 1e-7
    L = PointSet(X + s * n, w.copy(), t.copy())
    R = PointSet(X - s * n, w.copy(), t.copy())
    return Fold(L, R, float(Kt), float(theta0), bool(rigid))


def split_on_creases(faces: PointSet, creases, eps=1e-9, s=1e-7) -> tuple[PointSet, int]:
    """SetupHelper::splitGaussPointsOnCreases (plate/SetupHelper.h:60-106)."""
    xy = faces.xy.copy(); w = faces.weight.copy()
    best_d = np.full(len(xy), np.inf)
    best_n = np.zeros_like(xy)
    # Only a point within eps of a segment can be split, so each segment is tested against
    # the points inside its bounding box grown by eps (found on the x-sorted order); the
    # nearest segment of such a point is among those tested (ties: lower index, as before).
    order = np.argsort(xy[:, 0], kind="stable")
    xs = xy[order, 0]
    pad = 2.0 * eps
    for cr in creases:
        V = np.asarray(cr["vertices"], np.float64)
        for i in range(len(V) - 1):
            A, B = V[i], V[i + 1]
            v = B - A
            v2 = float(v @ v)
            if v2 == 0.0:
                continue
            lo = np.searchsorted(xs, min(A[0], B[0]) - pad, "left")
            hi = np.searchsorted(xs, max(A[0], B[0]) + pad, "right")
            cand = order[lo:hi]
            cand = cand[(xy[cand, 1] >= min(A[1], B[1]) - pad) & (xy[cand, 1] <= max(A[1], B[1]) + pad)]
            if len(cand) == 0:
                continue
            P = xy[cand]
            t = np.clip(((P - A) @ v) / v2, 0.0, 1.0)
            C = A[None, :] + t[:, None] * v[None, :]
            d = np.linalg.norm(P - C, axis=1)
            better = d < best_d[cand]
            best_d[cand[better]] = d[better]
            best_n[cand[better]] = np.array([-v[1], v[0]]) / math.sqrt(v2)
    hit = np.nonzero((best_d < eps) & ((best_n ** 2).sum(1) > 0))[0]
    if len(hit) == 0:
        return faces, 0
    twins = xy[hit] - s * best_n[hit]
    xy[hit] += s * best_n[hit]
    w[hit] *= 0.5
    return PointSet(np.concatenate([xy, twins]), np.concatenate([w, w[hit]])), len(hit)


def fourier_field(node_xy, rng, n_modes=8, lam=(20.0, 200.0), max_slope_w=math.tan(math.radians(60.0)),
                  inplane_frac=0.1) -> np.ndarray:
    """Smooth nodal displacement x (3 per node): each component a sum of n_modes
    seeded plane waves a_k sin(2 pi k.X / lambda_k + phi_k), lambda_k ~ U[lam]; w scaled
    so max |grad w| over the nodes equals max_slope_w (rotations up to 60 deg), u and v
    scaled to inplane_frac of that slope."""
    X = node_xy
    comps = []
    for c in range(3):
        val = np.zeros(len(X)); gx = np.zeros(len(X)); gy = np.zeros(len(X))
        for _ in range(n_modes):
            th = rng.uniform(0, 2 * math.pi)
            lk = rng.uniform(*lam)
            ph = rng.uniform(0, 2 * math.pi)
            a = rng.normal()
            kx, ky = 2 * math.pi * math.cos(th) / lk, 2 * math.pi * math.sin(th) / lk
            arg = kx * X[:, 0] + ky * X[:, 1] + ph
            val += a * np.sin(arg)
            gx += a * kx * np.cos(arg)
            gy += a * ky * np.cos(arg)
        slope = np.sqrt(gx ** 2 + gy ** 2).max()
        target = max_slope_w if c == 2 else inplane_frac * max_slope_w
        comps.append(val * (target / slope))
    return np.stack(comps, axis=1).ravel()


# ------------------------------------------------------------------------------------
# workloads
# ------------------------------------------------------------------------------------

def square_plate(n_side: int, h: float, rule: int, *, jitter: float = 0.0, seed: int = 0,
                 crease="row", Kt: float = 1e-3, rho_factor: float = 3.0, order: int = 2,
                 kernel: int = 0, E: float = 1.0, nu: float = 0.3, thickness: float = 0.05,
                 name: str = "square") -> Plate:
    """n_side x n_side node grid, spacing h, a tensor Gauss rule per cell and one crease:
    "row" a straight crease on the middle node column (x = (n_side-1)/2 h), "arc" a
    circular arc of radius 0.6 * side centred at the origin, None for no crease."""
    rng = np.random.default_rng(seed)
    nodes = grid_nodes(n_side, n_side, h, jitter, rng)
    faces = quad_gauss_points(nodes, n_side, n_side, rule)
    hull = convex_hull(_hull_candidates(nodes))
    side = (n_side - 1) * h
    creases, folds = [], []
    if crease == "row":
        col = (n_side - 1) // 2
        verts = nodes[np.arange(n_side) * n_side + col]
        creases.append(make_crease(verts, nodes, hull))
        folds.append(make_fold(verts, Kt))
    elif crease == "arc":
        R = 0.6 * side
        L = R * math.pi / 2
        nseg = max(8, int(math.ceil(L / (0.5 * h))))
        ang = np.linspace(0.0, math.pi / 2, nseg + 1)
        verts = np.stack([R * np.cos(ang), R * np.sin(ang)], axis=1)
        verts[0, 1] = 0.0; verts[-1, 0] = 0.0
        creases.append(make_crease(verts, nodes, hull))
        folds.append(make_fold(verts, Kt))
    faces, nsplit = split_on_creases(faces, creases)
    return Plate(name=name, node_xy=nodes, faces=faces, creases=creases, folds=folds,
                 rho=rho_factor * h, order=order, kernel=kernel, E=E, nu=nu,
                 thickness=thickness, seed=seed,
                 meta={"n_side": n_side, "h": h, "rule": rule, "jitter": jitter,
                       "crease": crease, "split": nsplit})


def four_crease_plate(n_side: int = 401, h: float = 0.5, rule: int = 4, seed: int = 1005, Kt: float = 1e-3,
                      rho_factor: float = 3.5, kernel: int = 0, max_skew_deg: float = 15.0) -> Plate:
    """n_side x n_side nodes of spacing h jittered by +/-0.2 h, and four straight creases from
    the centre node to the boundary, the sector angles 90 deg +/- delta (delta ~ U[0, max_skew]
    per crease, seeded): creases 0 and 2 rigid, 1 and 3 elastic with Kt. Each crease is a
    polyline of segments about h/2 long, ending at the centre with an end cap and extended
    at the boundary. rho = 3.5h: a point beside the junction sees only its own sector."""
    rng = np.random.default_rng(seed)
    nodes = grid_nodes(n_side, n_side, h, 0.2 * h, rng)
    c = (n_side // 2) * n_side + n_side // 2
    centre = nodes[c].copy()
    faces = quad_gauss_points(nodes, n_side, n_side, rule)
    hull = convex_hull(_hull_candidates(nodes))
    lo, hi = nodes.min(0), nodes.max(0)
    arng = np.random.default_rng([seed, 1])      # the crease directions, apart from the node jitter
    base = arng.uniform(0.0, 2.0 * math.pi)
    angles = [base]
    for k in range(3):
        angles.append(angles[-1] + math.radians(90.0 + arng.uniform(-max_skew_deg, max_skew_deg)))
    creases, folds = [], []
    for k, a in enumerate(angles):
        d = np.array([math.cos(a), math.sin(a)])
        # distance from the centre to the boundary box along d
        tmax = min((hi[i] - centre[i]) / d[i] if d[i] > 0 else (lo[i] - centre[i]) / d[i] if d[i] < 0 else np.inf
                   for i in range(2))
        nseg = max(8, int(math.ceil(tmax / (0.5 * h))))
        verts = centre[None, :] + np.linspace(0.0, tmax, nseg + 1)[:, None] * d[None, :]
        creases.append(make_crease(verts, nodes, hull))
        folds.append(make_fold(verts, Kt, 0.0, rigid=(k % 2 == 0)))
    faces, nsplit = split_on_creases(faces, creases)
    return Plate(name=f"four_creases{n_side}", node_xy=nodes, faces=faces, creases=creases, folds=folds,
                 rho=rho_factor * h, order=2, kernel=kernel, seed=seed,
                 meta={"n_side": n_side, "h": h, "rule": rule, "jitter": 0.2 * h, "crease": "four rays",
                       "sector_deg": [math.degrees(b - a) for a, b in zip(angles, angles[1:] + [angles[0] + 2 * math.pi])],
                       "split": nsplit})


def config_smallplate(rule: int = 3, kernel: int = 0, seed: int = 1001,
                      rho_factor: float = 3.5) -> Plate:
    """Plain FP64 method, small: [0,20]^2, 41x41 nodes (h = 0.5), quadratic basis,
    straight elastic hinge on the node column x = 10 (Kt = 1e-3), E = 1, nu = 0.3,
    t = 0.05. rule 3 / quartic is the reference-exact variant, rule 4 / cubic B-spline
    the literal one.

    The support radius defaults to 3.5h, not 3h: with a crease on a node column and
    rho = 3h, the crease points on the far side see the node columns at h and 2h only
    (the column at 3h has weight w(1) = 0), so the quadratic moment matrix is singular
    there and the reference itself stops with "RKPM: moment-matrix pivot collapsed".
    """
    return square_plate(41, 0.5, rule, seed=seed, crease="row", Kt=1e-3, kernel=kernel,
                        rho_factor=rho_factor, name=f"plate41_r{rule}")


def config_assembly(rule: int = 4, n_side: int = 201, kernel: int = 0, seed: int = 1003) -> Plate:
    """Single-plate assembly at scale: 201x201 jittered nodes (+/-0.1 with h = 0.5) on
    [0,100]^2, 4x4 rule (640,000 Gauss points), circular-arc crease of radius 60
    crossing the node layout freely, Kt = 1e-3; x from fourier_field."""
    p = square_plate(n_side, 0.5, rule, jitter=0.1, seed=seed, crease="arc", Kt=1e-3,
                     kernel=kernel, name=f"plate{n_side}_arc_r{rule}")
    return p


def config_shape_points(n_points: int = 1_000_000, n_side: int = 401, per_node_rho: bool = True,
                        seed: int = 1002, kernel: int = 1) -> tuple[Plate, np.ndarray]:
    """Shape-function stage alone: n_points uniform points in [0,200]^2 over a 401x401
    jittered node grid (+/-0.2h), quadratic basis, cubic B-spline window (kernel 1; 0 is the
    reference's quartic), per-node support radius U[2.5h, 3.5h] (extension) or the global
    3h, one straight cut along the node row y = 100 extended to the hull."""
    rng = np.random.default_rng(seed)
    h = 0.5
    nodes = grid_nodes(n_side, n_side, h, 0.2 * h, rng)
    side = (n_side - 1) * h
    pts = rng.uniform(0.0, side, size=(n_points, 2))
    row = (n_side - 1) // 2
    verts = np.array([[0.0, row * h], [side, row * h]])
    hull = convex_hull(_hull_candidates(nodes))
    creases = [make_crease(verts, nodes, hull)]
    rho_node = rng.uniform(2.5 * h, 3.5 * h, size=len(nodes)) if per_node_rho else None
    plate = Plate(name=f"points{n_points}", node_xy=nodes, faces=PointSet(pts, np.ones(n_points)),
                  creases=creases, rho=3.0 * h, rho_node=rho_node, order=2, kernel=kernel, seed=seed,
                  meta={"n_side": n_side, "h": h})
    return plate, pts


def batched_plate(n_side: int, rng, h: float = 0.5, rule: int = 4, jitter: float = 0.1,
                  name: str = "plate") -> Plate:
    """One plate of the batched workload: n_side x n_side jittered nodes, 1-3 creases that
    do not cross — either straight cuts parallel to y placed half-way between node columns
    and at least 6h apart, or concentric circular arcs about the origin at least 6h apart —
    each an elastic hinge with Kt log-uniform in [1e-4, 1e-1]."""
    nodes = grid_nodes(n_side, n_side, h, jitter, rng)
    faces = quad_gauss_points(nodes, n_side, n_side, rule)
    hull = convex_hull(_hull_candidates(nodes))
    side = (n_side - 1) * h
    k = int(rng.integers(1, 4))
    creases, folds = [], []
    if rng.random() < 0.5:
        lo, hi = 4, n_side - 5                      # columns with room for a support on both sides
        cols = []
        for c in rng.permutation(np.arange(lo, max(lo + 1, hi))):
            if all(abs(c - d) >= 6 for d in cols):
                cols.append(int(c))
            if len(cols) == k:
                break
        for c in sorted(cols):
            x0 = (c + 0.5) * h
            nseg = max(4, int(math.ceil(side / h)))
            verts = np.stack([np.full(nseg + 1, x0), np.linspace(0.0, side, nseg + 1)], axis=1)
            creases.append(make_crease(verts, nodes, hull))
            folds.append(make_fold(verts, 10.0 ** rng.uniform(-4, -1)))
    else:
        radii = []
        for R in rng.permutation(np.linspace(0.25 * side, 0.85 * side, 16)):
            if all(abs(R - S) >= 6 * h for S in radii):
                radii.append(float(R))
            if len(radii) == k:
                break
        for R in sorted(radii):
            nseg = max(8, int(math.ceil(R * math.pi / 2 / (0.5 * h))))
            ang = np.linspace(0.0, math.pi / 2, nseg + 1)
            verts = np.stack([R * np.cos(ang), R * np.sin(ang)], axis=1)
            verts[0, 1] = 0.0; verts[-1, 0] = 0.0
            creases.append(make_crease(verts, nodes, hull))
            folds.append(make_fold(verts, 10.0 ** rng.uniform(-4, -1)))
    faces, nsplit = split_on_creases(faces, creases)
    return Plate(name=name, node_xy=nodes, faces=faces, creases=creases, folds=folds, rho=3.0 * h, order=2,
                 kernel=0, seed=0, meta={"n_side": n_side, "h": h, "rule": rule, "jitter": jitter,
                                         "creases": len(creases), "split": nsplit})


def many_cuts_plate(n_side: int = 61, n_cuts: int = 6, h: float = 0.5, rule: int = 3, jitter: float = 0.05,
                    seed: int = 12) -> Plate:
    """More creases than a plate usually carries (the reference loops over any number,
    GlobalRKPM.h:86-112): n_cuts straight cuts parallel to y, half-way between node
    columns and 8 columns apart; even-numbered cuts cross the plate, odd-numbered ones
    start on the lower edge and stop at 60 % of the side, so their tips blend (Enrichment.h
    tip terms). Quadratic basis, rho = 3h, quartic window."""
    rng = np.random.default_rng(seed)
    nodes = grid_nodes(n_side, n_side, h, jitter, rng)
    faces = quad_gauss_points(nodes, n_side, n_side, rule)
    hull = convex_hull(_hull_candidates(nodes))
    side = (n_side - 1) * h
    creases = []
    for k in range(n_cuts):
        x0 = (4 + 8 * k + 0.5) * h
        if x0 > side - 3 * h:
            break
        top = side if k % 2 == 0 else 0.6 * side
        nseg = max(4, int(math.ceil(top / h)))
        verts = np.stack([np.full(nseg + 1, x0), np.linspace(0.0, top, nseg + 1)], axis=1)
        creases.append(make_crease(verts, nodes, hull))
    faces, nsplit = split_on_creases(faces, creases)
    return Plate(name=f"cuts{len(creases)}", node_xy=nodes, faces=faces, creases=creases, folds=[], rho=3.0 * h,
                 order=2, kernel=0, seed=seed, meta={"n_side": n_side, "h": h, "rule": rule, "split": nsplit})


def config_batched(n_plates: int = 64, side_range=(21, 161), seed: int = 1004, rule: int = 4):
    """Batched uneven plates: n_plates independent plates with node sides drawn uniformly
    from side_range (the config's "21^2 to 161^2" read as the side), 1-3 non-crossing
    straight or arc creases each, Kt log-uniform in [1e-4, 1e-1]; with every plate's seeded
    smooth displacement field (fourier_field, wavelengths scaled to the plate)."""
    rng = np.random.default_rng(seed)
    plates, xs = [], []
    for k in range(n_plates):
        n = int(rng.integers(side_range[0], side_range[1] + 1))
        p = batched_plate(n, rng, rule=rule, name=f"batch{k}_n{n}")
        side = (n - 1) * 0.5
        x = fourier_field(p.node_xy, rng, lam=(0.2 * side + 1.0, 2.0 * side + 1.0))
        plates.append(p)
        xs.append(x)
    return plates, xs
