"""Shared set-up of the progressive-creasing tests: the reference's centre-crease smoke
case (a 20 x 20 sheet, a crease grown from the centre to half-length 0.5 in 5 steps) and a
creasing plate over the CPU oracle (test infrastructure), beside the GPU one of
curvami_gb300.creasing.

The smoke case's published result (examples/smoke_centre_crease/README.md:14-20 of the
reference): the last step's row of smoke_steps.csv reads, to round-off,
E_mem 4.006e-08, E_ben 9.404e-06, E_hin 1.594e-05, mean theta 0.1962 deg."""
import math
import os

import numpy as np

from curvami_gb300 import creasing as PC
from curvami_gb300 import solver as S

SMOKE = PC.CENTRE_CREASE
GOLDEN_LAST_STEP = {"step": 5, "E_mem": 4.006e-08, "E_ben": 9.404e-06, "E_hin": 1.594e-05, "theta_mean_deg": 0.1962}
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def smoke_case(path, ideal=False, log_file=None):
    """The smoke case (20 x 20 cells) with the node coordinates gmsh wrote for the
    reference's example (tests/golden/smoke_centre_crease_nodes.npy), or the ideal grid."""
    xy = None if ideal else np.load(os.path.join(GOLDEN, "smoke_centre_crease_nodes.npy"))
    return PC.centre_crease_case(path, 20, node_xy=xy, log_file=log_file)


def smoke_plate(path, ideal=False):
    c = smoke_case(path, ideal)
    return c.plate, c.spec


def smoke_fixture():
    import json

    with open(os.path.join(GOLDEN, "smoke_centre_crease.json")) as f:
        return json.load(f)


# Paper A (examples/paperA_centre_crease/CB_n80_t0.5_xi10.json): the smoke case's run on the
# 80 x 80 mesh CB_n80.msh with hinge stiffness Kt = xi D / L, xi = 10, L = 1.
PAPER_A_KT = 10.0 * 1.098901098901099


def paper_a_case(path, log_file=None):
    xy = np.load(os.path.join(GOLDEN, "paper_a_cb_n80_nodes.npy"))
    c = PC.centre_crease_case(path, 80, node_xy=xy, log_file=log_file)
    c.plate.folds[0].Kt = PAPER_A_KT
    return c


def point_bcs():
    return smoke_case("/tmp/_smoke_bcs.msh", ideal=True).point_bcs


def smoke_config(log_file=None):
    return smoke_case("/tmp/_smoke_cfg.msh", ideal=True, log_file=log_file).config


def smoke_solver(kkt="host"):
    return S.ContinuationSolver(tol_force=SMOKE["tol_force"], tol_energy=SMOKE["tol_energy"],
                                ls_max_iters=SMOKE["ls_max_iters"], kkt=kkt)


def smoke_line(p):
    return PC.Line(folds=[0], full=p.creases[0], mode=SMOKE["mode"], tip_step=SMOKE["tip_step"])


class OracleCreasingPlate:
    """The creasing-plate methods over the CPU oracle: FRNN once, RKPM again at every
    rebuild, updateStiffness + the (exact-tangent) hinge for the LineSearch problem."""

    def __init__(self, o, p, spec, bcs, exact_tangent=True, static_schedule=False):
        """static_schedule: the oracle's assembly splits the Gauss points statically over its
        threads, so its sums round the same way on every run (the reference's guided schedule
        otherwise)."""
        self.o, self.plate, self.specs = o, p, [spec]
        self.static_schedule = bool(static_schedule)
        self.n = len(p.node_xy)
        self.exact = exact_tangent
        self._nb = {}
        self.cuts = list(p.creases)
        self.A, self.B, self.D = o.abd(p.E, p.nu, p.thickness)
        self.threads = os.cpu_count() or 1
        self.faces = self._shapes("faces", p.faces.xy)
        fd = p.folds[0]
        self.sides = [(self._shapes("L", fd.left.xy), self._shapes("R", fd.right.xy))]
        self.pts = {tag: self._shapes(("P", tag), p.points[tag].xy) for tag in bcs}
        self.fold_dict = {"left": self.sides[0][0], "right": self.sides[0][1], "weight": fd.left.weight,
                          "tangent": fd.left.tangent, "Kt": fd.Kt, "theta0": 0.0,
                          "theta0_gp": np.zeros(len(fd.left.xy)), "active": np.zeros(len(fd.left.xy), np.int8)}
        (self.outer, self.inner, self.col_ptr, self.col_nodes,
         self.mp) = o.pattern(self.n, self.faces["ptr"], self.faces["idx"], [self.fold_dict])
        points = []
        for tag, bc in bcs.items():
            z = np.zeros((len(p.points[tag].xy), 2))
            points.append((S.LineDomain(p.points[tag].xy, p.points[tag].weight, z, z, bc), None))
        self.bc_tags = list(bcs)
        self.problem = S.PlateProblem(self.n, self, None, p.faces.weight, points=points,
                                      folds=[S.FoldSides(None, None, np.asarray(fd.left.tangent), 0.0)])
        self._tables()

    def _shapes(self, key, pts):
        p = self.plate
        if key not in self._nb:
            self._nb[key] = (pts, *self.o.frnn(p.node_xy, pts, p.rho, p.rho_node))
        pts, ptr, idx, s = self._nb[key]
        psi, dpsi, ddpsi, bad, rc = self.o.rkpm(p.node_xy, pts, ptr, idx, s, p.rho, p.order, self.cuts,
                                                p.rho_node, p.kernel)
        assert rc == 0
        return dict(ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi)

    def _table(self, d):
        return S.ShapeTable(d["ptr"], d["idx"], d["psi"], d["dpsi"], self.n)

    def _tables(self):
        prob = self.problem
        prob.faces = self._table(self.faces)
        prob.folds[0].left = self._table(self.sides[0][0])
        prob.folds[0].right = self._table(self.sides[0][1])
        prob.points = [(dom, self._table(self.pts[tag])) for (dom, _), tag in zip(prob.points, self.bc_tags)]
        prob._f_ext = None

    # assembly backend (pattern / assemble)
    def pattern(self):
        return self.outer, self.inner

    def assemble(self, x, want_K, hinge=True):
        f = self.faces
        K, F = self.o.update_stiffness(self.n, self.plate.faces.weight, f["ptr"], f["idx"], f["dpsi"], f["ddpsi"],
                                       self.outer, self.mp, x, self.A, self.B, self.D, want_K=want_K,
                                       n_threads=self.threads, static_schedule=self.static_schedule)
        if hinge:
            K, F = self.o.hinge(self.n, x, [self.fold_dict], self.outer, self.col_ptr, self.col_nodes, K, F,
                                exact_tangent=self.exact and want_K)
        return (K if want_K else None), F

    # creasing-plate methods
    n_folds = 1

    @property
    def rho(self):
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

    def theta_star(self, f):
        return self.specs[f].theta_star

    def crease_tag(self, f):
        return self.specs[f].crease_tag

    def set_fold_state(self, f, theta0_gp, active):
        self.fold_dict["theta0_gp"] = np.array(theta0_gp, np.float64)
        self.fold_dict["active"] = np.array(active, np.int8)
        self.problem.folds[f].theta0_gp = np.array(theta0_gp, np.float64)
        self.problem.folds[f].active = np.array(active, np.int8)

    def rebuild(self, cuts):
        self.cuts = list(cuts)
        p = self.plate
        self.faces = self._shapes("faces", p.faces.xy)
        fd = p.folds[0]
        self.sides = [(self._shapes("L", fd.left.xy), self._shapes("R", fd.right.xy))]
        self.fold_dict["left"], self.fold_dict["right"] = self.sides[0]
        self.pts = {tag: self._shapes(("P", tag), p.points[tag].xy) for tag in self.pts}
        self._tables()

    def tables(self):
        return self.problem.faces, [(s.left, s.right) for s in self.problem.folds]

    def energies(self, x):
        f = self.faces
        em, eb = self.o.strain_energies(self.plate.faces.weight, f["ptr"], f["idx"], f["dpsi"], f["ddpsi"], x,
                                        self.A, self.B, self.D)
        return em, eb, self.o.hinge_energy(x, [self.fold_dict])


def assert_golden_row(rec, rel=None):
    """The last step's row against the published one, each quantity to within half a unit of
    its last printed digit (plus 2e-4 relative: the mesh here is the .geo's ideal grid, the
    published run used gmsh's node positions, which differ by up to 3e-12)."""
    for key in ("E_mem", "E_ben", "E_hin", "theta_mean_deg"):
        want = GOLDEN_LAST_STEP[key]
        digits = 4 if key != "theta_mean_deg" else 4
        half_ulp = 0.5 * 10.0 ** (math.floor(math.log10(abs(want))) - (digits - 1))
        tol = half_ulp + (rel if rel is not None else 2e-4) * abs(want)
        assert abs(rec[key] - want) <= tol, (key, rec[key], want, tol)
