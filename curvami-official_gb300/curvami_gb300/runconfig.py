"""Run configurations in the reference's JSON format.

``main.cpp`` (run_solver, main.cpp:28-330) turns one JSON file into a plate, its folds,
supports and solver settings before it dispatches the analysis. This module restates the
part of that set-up the Gauss-point path and its continuation drivers need, so the
reference's own example files drive the GPU assembly unchanged:

  * material: one isotropic ply (E, nu, h) through the laminate A/B/D (main.cpp:52-59);
  * mesh: the msh 4.1 Gauss points, rho = (3 + 3) x the median third-neighbour spacing and
    the reproducibility order 3 of ``Meshless plate(3)`` (main.cpp:64-75);
  * folds: per entry its crease tag, hinge stiffness, rigid / driver flags, mountain
    (sign -1) or valley, start and target angles in degrees; a fold's initial rest angle is
    sign x angle_start (main.cpp:105-168);
  * cuts: lists of crease tags walked into the curves that cut the RKPM supports, else one
    curve per fold (main.cpp:171-184);
  * point_bcs / edge_bcs: u, v, w (and rot, force) on the point and edge domains of an
    entity tag (main.cpp:200-242);
  * solver: the arc-length settings with main.cpp's defaults (main.cpp:252-282).

Left out, as outside the hot path: natural curvature from the file (set it with
``Context.set_natural_curvature``), fold ties other than pointwise, j_integral, outputs,
restart bookkeeping (the drivers take ``restart_file`` themselves).
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import mesh
from . import solver as S


@dataclass
class FoldConfig:
    """One "folds" entry: the fields of Fold that main.cpp sets (angles in radians)."""
    crease_tag: int
    stiffness: float
    rigid: bool
    driver: bool
    sign: float
    angle_start: float
    angle_target: float


@dataclass
class RunConfig:
    analysis_type: str
    plate: object                    # synth.Plate
    folds: list                      # FoldConfig, in the plate's fold order
    points: list                     # LineDomain of every point domain with a support
    edges: list                      # LineDomain of every edge domain with a support or load
    solver: dict                     # the "solver" block with main.cpp's defaults filled in
    raw: dict = field(default_factory=dict)

    def drivers(self):
        from .arclength import Driver

        return [Driver(k, f.angle_start, f.angle_target, f.sign) for k, f in enumerate(self.folds) if f.driver]

    def arc_length_solver(self, **override):
        """ArcLengthSolver with the file's settings (main.cpp:252-282); keyword arguments
        override them (kkt, exact_fold_gradient, kmax for a shortened run, ...)."""
        from .arclength import ArcLengthSolver

        s = self.solver
        kw = dict(ds=s["ds"], dsmin=s["dsmin"], dsmax=s["dsmax"], max_iters=s["max_iters"], psi=s["psi"],
                  kmax=s["kmax"], asla_hold_after_reversal=s["asla_hold_after_reversal"],
                  no_progress_window=s["no_progress_window"], no_progress_efficiency=s["no_progress_efficiency"],
                  no_progress_abort=s["no_progress_abort"], tol_force=s["tol_force"], tol_energy=s["tol_energy"],
                  ls_max_iters=s["ls_max_iters"])
        kw.update(override)
        return ArcLengthSolver(**kw)


def solver_settings(cfg: dict) -> dict:
    """The "solver" block with main.cpp's defaults (main.cpp:252-282; tol_force and
    tol_energy default to ContinuationSolver's 1e-8)."""
    s = dict(cfg.get("solver", {}))
    ds = float(s.get("ds", 0.1))
    return {
        "ds": ds, "dsmax": float(s.get("dsmax", 1e3 * ds)), "dsmin": float(s.get("dsmin", 1e-3 * ds)),
        "max_iters": int(s.get("max_iters", 30)), "psi": float(s.get("psi", 1.0)), "kmax": int(s.get("kmax", 500)),
        "ls_max_iters": int(s.get("ls_max_iters", 500)), "tol_force": float(s.get("tol_force", 1e-8)),
        "tol_energy": float(s.get("tol_energy", 1e-8)),
        "snapback_inertia_veto": bool(s.get("snapback_inertia_veto", False)),
        "asla_hold_after_reversal": bool(s.get("asla_hold_after_reversal", False)),
        "no_progress_abort": bool(s.get("no_progress_abort", True)),
        "no_progress_window": int(s.get("no_progress_window", 24)),
        "no_progress_efficiency": float(s.get("no_progress_efficiency", 0.15)),
        "max_load": float(s.get("max_load", 1.0)), "target_tol_deg": float(s.get("target_tol_deg", 2.0)),
        "fold_exact_tangent": bool(s.get("fold_exact_tangent", False)),
    }


def fold_configs(cfg: dict, edge_tags) -> list:
    """The "folds" entries whose crease tag has line elements, in file order (main.cpp:106-168;
    an unknown tag is skipped there with a warning)."""
    out = []
    for f in cfg.get("folds", []):
        tag = int(f["crease_tag"])
        if tag not in edge_tags:
            continue
        sign = -1.0 if str(f.get("type", "")).lower() == "mountain" else 1.0
        out.append(FoldConfig(tag, float(f.get("stiffness", 0.0)), bool(f["is_rigid"]), bool(f.get("is_driver", False)),
                              sign, float(f.get("angle_start", 0.0)) * math.pi / 180.0,
                              float(f.get("angle_target", 0.0)) * math.pi / 180.0))
    return out


def _bc(c: dict) -> S.BoundaryCondition:
    return S.BoundaryCondition("u" in c, "v" in c, "w" in c, float(c.get("u", 0.0)), float(c.get("v", 0.0)),
                               float(c.get("w", 0.0)), "rot" in c, float(c.get("rot", 0.0)),
                               tuple(float(v) for v in c.get("force", (0.0, 0.0, 0.0))))


def from_elements(cfg: dict, node_xy, elements, kernel: int = 0) -> RunConfig:
    """RunConfig of a parsed configuration and the nodes and elements of its mesh."""
    etags = {int(e.entity_tag) for e in elements if e.type == 1}
    folds = fold_configs(cfg, etags)
    m = cfg["material"]
    cuts = [list(c) for c in cfg["cuts"]] if "cuts" in cfg else None
    p = mesh.plate_from_elements(node_xy, elements, [f.crease_tag for f in folds], [f.stiffness for f in folds],
                                 order=3, kernel=kernel, E=float(m["E"]), nu=float(m["nu"]),
                                 thickness=float(m["h"]), theta0=[f.sign * f.angle_start for f in folds],
                                 cuts=cuts, rigid=[f.rigid for f in folds], name=str(cfg.get("mesh_file", "mesh")))
    points = []
    for c in cfg.get("point_bcs", []):
        ps = p.points.get(int(c["tag"]))
        if ps is None or len(ps.xy) == 0:
            continue
        k = len(ps.xy)
        points.append(S.LineDomain(np.asarray(ps.xy, np.float64), np.asarray(ps.weight, np.float64),
                                   np.tile([1.0, 0.0], (k, 1)), np.tile([0.0, 1.0], (k, 1)), _bc(c)))
    edges = []
    for c in cfg.get("edge_bcs", []):
        e = p.meta["edges"].get(int(c["tag"]))
        if e is None or len(e[0]) == 0:
            continue
        edges.append(S.LineDomain(e[0], e[1], e[2], e[3], _bc(c)))
    return RunConfig(str(cfg.get("analysis_type", "")), p, folds, points, edges, solver_settings(cfg), cfg)


def load(config_path: str, root: str | None = None, kernel: int = 0) -> RunConfig:
    """RunConfig of a JSON file; its mesh_file is read relative to `root` (default: the
    directory two levels above the file, where the reference's examples keep it)."""
    with open(config_path) as f:
        cfg = json.load(f)
    base = root if root is not None else os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(config_path))))
    xy, elements = mesh.read_msh41(os.path.join(base, cfg["mesh_file"]))
    return from_elements(cfg, xy, elements, kernel)


def gpu_problem(rc: RunConfig, model, mixed: bool = False, deterministic: bool = False):
    """PlateProblem of a RunConfig over a PlateModel of rc.plate (the GPU assembly), with the
    hinge tangent the file asks for."""
    return S.gpu_problem(model, edges=rc.edges, points=rc.points, mixed=mixed, deterministic=deterministic,
                         exact_hinge=rc.solver["fold_exact_tangent"])
