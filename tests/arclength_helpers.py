"""Shared set-up of the arc-length tests: a small plate with four creases from the centre
(synth.four_crease_plate), creases 0 and 2 driven through stiff hinges, 1 and 3 passive
elastic hinges, three pinned points in the sector between creases 0 and 1 (the reference's
point supports u = v = w = 0, v = w = 0, w = 0), over the oracle or the GPU."""
import math

import numpy as np

from curvami_gb300 import arclength as A
from curvami_gb300 import solver as S
from curvami_gb300 import synth

from newton_helpers import OracleAssembly


def four_crease_case(n_side=13, Kt_driver=1e-1, Kt_passive=1e-3, target_deg=60.0, seed=1005, skew_deg=15.0):
    p = synth.four_crease_plate(n_side=n_side, h=0.5, rule=3, seed=seed, Kt=Kt_passive, rho_factor=3.5,
                                max_skew_deg=skew_deg)
    for k, f in enumerate(p.folds):
        f.rigid = False
        f.Kt = Kt_driver if k % 2 == 0 else Kt_passive
    doms = A.sector_supports(p, 0, 1)
    drivers = [A.Driver(0, 0.0, math.radians(target_deg)), A.Driver(2, 0.0, math.radians(target_deg))]
    return p, doms, drivers


class OracleAssemblyTheta(OracleAssembly):
    """OracleAssembly with settable fold rest angles and, by default, the exact hinge tangent
    (Meshless::fold_exact_tangent), as the arc-length runs use it."""

    exact_tangent = True

    def set_fold_theta0(self, f, theta0):
        self.folds[f]["theta0"] = float(theta0)

    def assemble(self, x, want_K, hinge=True):
        K, F = super().assemble(x, want_K, hinge=False)
        if hinge:
            K, F = self.o.hinge(self.n, x, self.folds, self.outer, self.col_ptr, self.col_nodes, K, F,
                                exact_tangent=self.exact_tangent)
        return (K if want_K else None), F


def oracle_arc_problem(o, p, doms, exact_tangent=True):
    n = len(p.node_xy)

    def shapes(pts):
        ptr, idx, s = o.frnn(p.node_xy, pts, p.rho, p.rho_node)
        psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, pts, ptr, idx, s, p.rho, p.order, p.creases,
                                           p.rho_node, p.kernel)
        assert rc == 0
        return dict(ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi)

    def table(d):
        return S.ShapeTable(d["ptr"], d["idx"], d["psi"], d["dpsi"], n)

    faces = shapes(p.faces.xy)
    folds_o, sides = [], []
    for fd in p.folds:
        L, R = shapes(fd.left.xy), shapes(fd.right.xy)
        folds_o.append({"left": L, "right": R, "weight": fd.left.weight, "tangent": fd.left.tangent,
                        "Kt": fd.Kt, "theta0": fd.theta0})
        sides.append(S.FoldSides(table(L), table(R), np.asarray(fd.left.tangent, np.float64), fd.theta0,
                                 Kt=fd.Kt, weight=np.asarray(fd.left.weight, np.float64)))
    backend = OracleAssemblyTheta(o, p, faces, folds_o)
    backend.exact_tangent = bool(exact_tangent)
    points = [(dom, table(shapes(dom.xy))) for dom in doms]
    return S.PlateProblem(n, backend, table(faces), p.faces.weight, folds=sides, points=points)
