"""Shared set-up of the Newton-driver tests: a small clamped plate with a straight elastic
hinge and a face load, and an assembly backend over the CPU oracle (test infrastructure)."""
import os

import numpy as np

from curvami_gb300 import solver as S
from curvami_gb300 import synth


def small_plate(n_side=13):
    """Plain FP64 method, small, scaled down: [0, 6]^2 at h = 0.5, 3x3 rule, cubic B-spline
    window, rho = 3.5h, crease on the middle node column, Kt = 1e-3, E = 1, nu = 0.3, t = 0.05."""
    return synth.square_plate(n_side, 0.5, 3, crease="row", Kt=1e-3, kernel=1, rho_factor=3.5, seed=1001)


def clamped_left_edge(p):
    side = float(p.node_xy[:, 1].max() - p.node_xy[:, 1].min())
    n_seg = int(round(side / 0.5))
    return S.clamped_edge((0.0, 0.0), (0.0, side), n_seg)


class OracleAssembly:
    """pattern() / assemble(x, want_K, hinge) over the oracle's updateStiffness and hinge."""

    def __init__(self, o, p, faces, folds_o):
        self.o, self.p, self.f, self.folds = o, p, faces, folds_o
        self.n = len(p.node_xy)
        self.A, self.B, self.D = o.abd(p.E, p.nu, p.thickness)
        (self.outer, self.inner, self.col_ptr, self.col_nodes,
         self.mp) = o.pattern(self.n, faces["ptr"], faces["idx"], folds_o)
        self.threads = os.cpu_count() or 1

    def pattern(self):
        return self.outer, self.inner

    def assemble(self, x, want_K, hinge=True):
        f = self.f
        K, F = self.o.update_stiffness(self.n, self.p.faces.weight, f["ptr"], f["idx"], f["dpsi"], f["ddpsi"],
                                       self.outer, self.mp, x, self.A, self.B, self.D, want_K=want_K,
                                       n_threads=self.threads, static_schedule=True)
        if hinge:
            K, F = self.o.hinge(self.n, x, self.folds, self.outer, self.col_ptr, self.col_nodes, K, F)
        return (K if want_K else None), F


def oracle_problem(o, p, face_load, edge):
    """PlateProblem over the oracle: oracle shape functions for faces, folds and the edge."""
    n = len(p.node_xy)

    def shapes(pts):
        ptr, idx, s = o.frnn(p.node_xy, pts, p.rho, p.rho_node)
        psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, pts, ptr, idx, s, p.rho, p.order, p.creases,
                                           p.rho_node, p.kernel)
        assert rc == 0
        return dict(ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi)

    faces = shapes(p.faces.xy)
    folds_o, sides = [], []
    for fd in p.folds:
        L, R = shapes(fd.left.xy), shapes(fd.right.xy)
        folds_o.append({"left": L, "right": R, "weight": fd.left.weight, "tangent": fd.left.tangent,
                        "Kt": fd.Kt, "theta0": fd.theta0})
        sides.append(S.FoldSides(S.ShapeTable(L["ptr"], L["idx"], L["psi"], L["dpsi"], n),
                                 S.ShapeTable(R["ptr"], R["idx"], R["psi"], R["dpsi"], n),
                                 fd.left.tangent, fd.theta0))
    e = shapes(edge.xy)
    backend = OracleAssembly(o, p, faces, folds_o)
    table = S.ShapeTable(faces["ptr"], faces["idx"], faces["psi"], faces["dpsi"], n)
    return S.PlateProblem(n, backend, table, p.faces.weight, face_load=face_load,
                          edges=[(edge, S.ShapeTable(e["ptr"], e["idx"], e["psi"], e["dpsi"], n))],
                          folds=sides)
