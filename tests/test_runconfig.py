"""Run configurations in the reference's JSON format (curvami_gb300/runconfig.py, main.cpp:28-330)
on a synthetic msh 4.1 mesh: fold order, signs and angles, cuts, unknown crease tags, point and
edge supports, and main.cpp's solver defaults."""
import math

import numpy as np
import pytest

from curvami_gb300 import mesh, runconfig, synth


def grid_with_two_creases(n=9, h=0.5):
    xy = synth.grid_nodes(n, n, h, 0.0, np.random.default_rng(0))
    els = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i
            els.append(mesh.Element(3, 1, (a, a + 1, a + n + 1, a + n)))
    mid = n // 2
    for j in range(mid):                                    # tag 5: lower half of the middle column
        els.append(mesh.Element(1, 5, (j * n + mid, (j + 1) * n + mid)))
    for j in range(mid, n - 1):                             # tag 6: upper half
        els.append(mesh.Element(1, 6, (j * n + mid, (j + 1) * n + mid)))
    for j in range(n - 1):                                  # tag 2: the edge x = 0
        els.append(mesh.Element(1, 2, (j * n, (j + 1) * n)))
    els.append(mesh.Element(15, 7, (n - 1,)))
    return xy, els


def config(**over):
    cfg = {
        "mesh_file": "synthetic.msh",
        "analysis_type": "TargetDirectedArcLength",
        "material": {"E": 2.0, "nu": 0.25, "h": 0.1},
        "folds": [
            {"crease_tag": 6, "angle_start": 10.0, "angle_target": 90.0, "stiffness": 2.0, "is_rigid": False,
             "is_driver": True, "type": "mountain"},
            {"crease_tag": 99, "angle_target": 30.0, "is_rigid": False},          # not in the mesh: skipped
            {"crease_tag": 5, "angle_target": -45.0, "stiffness": 0.5, "is_rigid": True},
        ],
        "cuts": [[5, 6]],
        "point_bcs": [{"tag": 7, "u": 0.0, "w": 0.25}],
        "edge_bcs": [{"tag": 2, "u": 0.0, "v": 0.0, "w": 0.0, "rot": 0.0, "force": [0.0, 0.0, 1.0]}],
        "solver": {"ds": 0.2, "max_iters": 12, "psi": 0.0},
    }
    cfg.update(over)
    return cfg


def test_folds_cuts_and_supports():
    xy, els = grid_with_two_creases()
    rc = runconfig.from_elements(config(), xy, els)
    p = rc.plate
    assert [f.crease_tag for f in rc.folds] == [6, 5]
    f6, f5 = rc.folds
    assert f6.sign == -1.0 and f6.driver and not f6.rigid and f6.stiffness == 2.0
    assert f6.angle_start == pytest.approx(math.radians(10.0)) and f6.angle_target == pytest.approx(math.radians(90.0))
    assert f5.sign == 1.0 and f5.rigid and not f5.driver
    # The fold's rest angle starts at sign x angle_start (main.cpp:121-126).
    assert p.folds[0].theta0 == pytest.approx(-math.radians(10.0)) and p.folds[1].theta0 == 0.0
    assert p.folds[0].Kt == 2.0 and p.folds[1].Kt == 0.5 and p.folds[1].rigid and not p.folds[0].rigid
    # One cut made of both tags: a single polyline through the whole column.
    assert len(p.creases) == 1 and len(p.creases[0]["vertices"]) == 9
    assert (p.E, p.nu, p.thickness, p.order) == (2.0, 0.25, 0.1, 3)
    assert [len(f.left.xy) for f in p.folds] == [4, 4]
    (pt,) = rc.points
    assert (pt.bc.active_u, pt.bc.active_v, pt.bc.active_w, pt.bc.val_w) == (True, False, True, 0.25)
    (ed,) = rc.edges
    assert len(ed.xy) == 8 and ed.bc.active_rot and ed.bc.force == (0.0, 0.0, 1.0)
    assert [d.fold for d in rc.drivers()] == [0]


def test_without_cuts_each_fold_is_its_own_crease():
    xy, els = grid_with_two_creases()
    cfg = config()
    del cfg["cuts"]
    rc = runconfig.from_elements(cfg, xy, els)
    assert len(rc.plate.creases) == 2
    assert [len(c["vertices"]) for c in rc.plate.creases] == [5, 5]


def test_solver_defaults_follow_main_cpp():
    s = runconfig.solver_settings(config())
    assert s["ds"] == 0.2 and s["dsmax"] == pytest.approx(200.0) and s["dsmin"] == pytest.approx(2e-4)
    assert s["max_iters"] == 12 and s["psi"] == 0.0 and s["kmax"] == 500 and s["ls_max_iters"] == 500
    assert s["tol_force"] == 1e-8 and s["tol_energy"] == 1e-8 and s["no_progress_window"] == 24
    assert not s["fold_exact_tangent"] and not s["snapback_inertia_veto"]
    sol = runconfig.from_elements(config(), *grid_with_two_creases()).arc_length_solver(kmax=3)
    assert (sol.ds, sol.dsmax, sol.max_iters, sol.psi, sol.kmax) == (0.2, pytest.approx(200.0), 12, 0.0, 3)
