"""The fold terms of the domain-integral energy release rate (curvami_gb300/jintegral.py,
JIntegral.h:303-418, 551-746), with the point states of the faces and of both sides of the
fold from the oracle's Kinematics::compute + Constitutive.

- the hinges' virtual work equals sum_I g_I e . F_hinge,I with the oracle hinge's nodal force,
  for any nodal g and in-plane e (the reference's hingeVirtualWork is that directional
  derivative), with per-point rest angles and inactive points;
- for g_I = f(X_I), f linear, the nodal form equals the analytic form (linear reproduction);
- the crease points' fold angles are the oracle's foldAngleAndGrad angles;
- d(psi)/ds: central differences in s order, one-sided at the ends, signed by T . T0;
- an isometric fold of one half of the plate about a straight crease through the tip (x = XC) has
  B = 0 at every face point and on both sides of the crease: f_n = f_T = 0, the fold angle
  is the rotation everywhere, and every G form vanishes, the line terms by the symmetry of
  the crease points about the tip;
- the _fold.csv and _crease.csv files carry the reference's columns;
- qAnalytic's gradient and second gradient are the derivatives of qValue;
- the GPU point states give the oracle states' fold terms (GPU test).
"""
import math

import numpy as np
import pytest

from curvami_gb300 import jintegral as J
from curvami_gb300 import synth
from oracle import Oracle
from test_jintegral import oracle_state


@pytest.fixture(scope="module")
def o():
    return Oracle(native=True)


def shapes(o, p, pts):
    ptr, idx, s = o.frnn(p.node_xy, pts, p.rho, p.rho_node)
    psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, pts, ptr, idx, s, p.rho, p.order, p.creases, p.rho_node,
                                       p.kernel)
    assert rc == 0
    return dict(ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi)


XC = 5.1   # the crease line x = XC, between two node columns


@pytest.fixture(scope="module")
def folded(o):
    """21 x 21 nodes (h = 0.5), 3 x 3 rule, a straight crease x = XC over the whole plate in
    20 segments (Kt = 2e-3)."""
    p = synth.square_plate(21, 0.5, 3, jitter=0.0, crease=None, seed=5)
    verts = np.stack([np.full(21, XC), np.linspace(0.0, 10.0, 21)], 1)
    p.creases = [synth.make_crease(verts, p.node_xy)]
    p.folds = [synth.make_fold(verts, 2e-3)]
    p.faces, _ = synth.split_on_creases(p.faces, p.creases)
    f = p.folds[0]
    return p, shapes(o, p, p.faces.xy), shapes(o, p, f.left.xy), shapes(o, p, f.right.xy)


def fold_states(o, p, shL, shR, x, theta0=0.0, theta0_gp=None, active=None):
    f = p.folds[0]
    return [J.FoldState(f.left.xy, f.right.xy, f.left.weight, f.left.tangent, oracle_state(o, p, shL, x),
                        oracle_state(o, p, shR, x), shL, shR, f.Kt, theta0, False, theta0_gp, active)]


def oracle_fold(p, shL, shR, theta0=0.0, theta0_gp=None, active=None):
    f = p.folds[0]
    d = {"left": shL, "right": shR, "weight": f.left.weight, "tangent": f.left.tangent, "Kt": f.Kt,
         "theta0": theta0}
    if theta0_gp is not None:
        d["theta0_gp"] = theta0_gp
    if active is not None:
        d["active"] = np.asarray(active, np.int8)
    return d


def face_force(o, p, sh, x):
    outer, inner, col_ptr, col_nodes, mp = o.pattern(p.n_nodes, sh["ptr"], sh["idx"])
    A, B, D = o.abd(p.E, p.nu, p.thickness)
    return o.update_stiffness(p.n_nodes, p.faces.weight, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"], outer, mp,
                              x, A, B, D, want_K=False)[1]


def isometric_fold(p, alpha):
    """Rotate the half x < XC about the crease line x = XC by alpha."""
    X = p.node_xy[:, 0]
    left = X < XC
    u = np.zeros((p.n_nodes, 3))
    u[left, 0] = (X[left] - XC) * math.cos(alpha) + XC - X[left]
    u[left, 2] = -(X[left] - XC) * math.sin(alpha)
    return u.ravel()


def test_hinge_virtual_work_is_the_hinge_nodal_force(o, folded):
    p, sh, shL, shR = folded
    rng = np.random.default_rng(11)
    x = 0.05 * synth.fourier_field(p.node_xy, rng, lam=(3.0, 9.0))
    n_gp = len(p.folds[0].left.weight)
    t0 = 0.02 * rng.standard_normal(n_gp)
    act = rng.random(n_gp) > 0.3
    folds = fold_states(o, p, shL, shR, x, 0.01, t0, act)
    _, Fh = o.hinge(p.n_nodes, x, [oracle_fold(p, shL, shR, 0.01, t0, act)])
    Fh = Fh.reshape(-1, 3)
    for e in (np.array([1.0, 0.0]), np.array([math.cos(0.7), math.sin(0.7)])):
        g = rng.standard_normal(p.n_nodes)
        ref = float(g @ (Fh[:, :2] @ e))
        got = J.hinge_virtual_work(folds, g, e)
        assert abs(got - ref) <= 1e-11 * float(np.abs(g[:, None] * Fh[:, :2]).sum())
    # linear f: nodal values and the analytic gradient give the same work
    a = np.array([0.3, -0.8])
    g = p.node_xy @ a + 0.4
    e = np.array([0.6, 0.8])
    w_n = J.hinge_virtual_work(folds, g, e)
    w_a = J.hinge_virtual_work_analytic(folds, e, lambda X: np.broadcast_to(a, X.shape))
    # (bar: the one-sided supports 1e-7 from the cut reproduce gradients to about 1e-10)
    assert abs(w_n - w_a) <= 1e-8 * abs(w_a) and abs(w_a) > 0.0


def test_crease_point_angles_are_the_oracle_fold_angles(o, folded):
    p, sh, shL, shR = folded
    x = 0.05 * synth.fourier_field(p.node_xy, np.random.default_rng(12), lam=(3.0, 9.0))
    folds = fold_states(o, p, shL, shR, x, 0.03)
    (c,) = J.crease_points(folds)
    stL, stR = folds[0].state_left, folds[0].state_right
    for j in range(len(c["i"])):
        F12 = np.concatenate([stL[j, 3:9], stR[j, 3:9]])
        th, _ = o.fold_angle(F12, c["T"][j, 0], c["T"][j, 1])
        assert abs(c["theta"][j] - th) <= 1e-13
        assert abs(c["psi"][j] - 0.5 * p.folds[0].Kt * (th - 0.03) ** 2) <= 1e-16 + 1e-12 * c["psi"][j]
    assert np.array_equal(c["i"], np.arange(len(p.folds[0].left.weight)))


def test_dpsi_ds_order_ends_and_sign():
    s = np.array([2.0, 0.0, 1.0, 3.0])
    psi = np.array([4.0, 0.0, 1.0, 9.0])
    T = np.array([[1.0, 0.0], [1.0, 0.0], [-1.0, 0.0], [1.0, 0.0]])
    d = J.dpsi_ds(s, psi, T, np.array([1.0, 0.0]))
    # order by s: points 1, 2, 0, 3
    assert d[1] == (1.0 - 0.0) / 1.0                       # one-sided at the start
    assert d[2] == -(4.0 - 0.0) / 2.0                      # central, against T0
    assert d[0] == (9.0 - 1.0) / 2.0
    assert d[3] == (9.0 - 4.0) / 1.0                       # one-sided at the end
    assert np.array_equal(J.dpsi_ds(np.zeros(3), np.arange(3.0), T[:3], T[0]), np.zeros(3))
    assert len(J.dpsi_ds([], [], np.zeros((0, 2)), T[0])) == 0


def test_isometric_fold_releases_nothing(o, folded):
    p, sh, shL, shR = folded
    alpha = 0.6
    x = isometric_fold(p, alpha)
    folds = fold_states(o, p, shL, shR, x, 0.1)
    st = oracle_state(o, p, sh, x)
    F = face_force(o, p, sh, x)
    assert float(np.abs(F).max()) <= 1e-14
    s = J.Settings(tip=(XC, 5.0), dir=(math.cos(0.5), math.sin(0.5)), rings=[J.Ring(1.6, 3.2), J.Ring(2.0, 4.0)],
                   fold_band=1.0, fold_band_plateau=0.2)
    cps = []
    res = J.compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, sh["ptr"], sh["idx"], sh["dpsi"],
                               sh["ddpsi"], p.thickness, s, folds, F, cps)
    (c,) = cps
    psi = 0.5 * p.folds[0].Kt * (alpha - 0.1) ** 2
    assert np.abs(np.abs(c["theta"]) - alpha).max() <= 1e-12
    assert np.abs(c["Bp"]).max() <= 1e-13 and np.abs(c["Bm"]).max() <= 1e-13
    assert np.abs(c["fn"]).max() <= 1e-13 and np.abs(c["fT"]).max() <= 1e-12
    scale = psi * float(c["w"].sum()) / p.thickness
    for r in res:
        assert r["n_crease"] > 0
        for k in ("G1", "G1_h", "line_h", "line_a", "Gfold_h", "Gfold_a", "GD_h", "GD_a", "Gtip_h", "Gtip_a",
                  "resid_h", "Gfold_band_h", "Gfold_band_a", "vw_band_s", "resid_band"):
            assert abs(r[k]) <= 1e-10 * scale, k
        # the hinge terms are the hinge's own virtual work, matched to the nodal force above;
        # here they are finite and enter the _r / _s forms as the reference subtracts them
        assert r["GD_r"] == pytest.approx(r["G1_h"] - r["resid_h"] - r["hinge_h"] - r["line_h"], abs=1e-15)
        assert r["G1_s"] == pytest.approx(r["G1"] - r["vw1_s"] - r["hw1_s"], abs=1e-15)


def test_fold_and_crease_csv(tmp_path, o, folded):
    p, sh, shL, shR = folded
    x = 0.05 * synth.fourier_field(p.node_xy, np.random.default_rng(13), lam=(3.0, 9.0))
    folds = fold_states(o, p, shL, shR, x)
    st = oracle_state(o, p, sh, x)
    s = J.Settings(tip=(XC, 5.0), dir=(1.0, 0.0), rings=[J.Ring(1.6, 3.2)])
    cps = []
    res = J.compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, sh["ptr"], sh["idx"], sh["dpsi"],
                               sh["ddpsi"], p.thickness, s, folds, face_force(o, p, sh, x), cps)
    path = str(tmp_path / "G.csv")
    J.write_csv(path, 2, s, res, p.thickness, True, crease=cps)
    J.write_csv(path, 3, s, res, p.thickness, False, crease=cps)
    fold = open(str(tmp_path / "G_fold.csv")).read().splitlines()
    crease = open(str(tmp_path / "G_crease.csv")).read().splitlines()
    assert fold[0].startswith("# fold terms of the energy release rate (along d)")
    assert fold[1].split(",") == J.FOLD_COLUMNS and len(fold) == 2 + 2
    assert crease[1].split(",") == J.CREASE_COLUMNS
    n_c = len(cps[0]["i"])
    assert len(crease) == 2 + 2 * n_c
    row = crease[2].split(",")
    assert row[:3] == ["2", "0", "0"] and len(row) == len(J.CREASE_COLUMNS)
    assert float(row[J.CREASE_COLUMNS.index("theta")]) == pytest.approx(cps[0]["theta"][0], rel=1e-11)
    # without crease points only the main file is written
    J.write_csv(str(tmp_path / "H.csv"), 2, s, res, p.thickness, True)
    assert not (tmp_path / "H_fold.csv").exists()


def test_fold_terms_need_the_face_force(o, folded):
    p, sh, shL, shR = folded
    x = np.zeros(3 * p.n_nodes)
    folds = fold_states(o, p, shL, shR, x)
    with pytest.raises(ValueError):
        J.compute_from_state(oracle_state(o, p, sh, x), p.faces.xy, p.faces.weight, p.node_xy, sh["ptr"], sh["idx"],
                             sh["dpsi"], sh["ddpsi"], p.thickness, J.Settings(rings=[J.Ring(1.0, 2.0)]), folds)


@pytest.mark.gpu
def test_gpu_fold_terms_match_oracle(o, folded):
    import curvami_gb300 as cg

    p, sh, shL, shR = folded
    model = cg.PlateModel(p)
    rng = np.random.default_rng(14)
    x = isometric_fold(p, 0.4) + 0.02 * synth.fourier_field(p.node_xy, rng, lam=(3.0, 9.0))
    s = J.Settings(tip=(XC, 4.0), dir=(math.cos(0.3), math.sin(0.3)), rings=[J.Ring(1.6, 3.2), J.Ring(2.0, 4.0)],
                   fold_band=1.0, fold_band_plateau=0.2)
    gpu_c = []
    gpu = J.compute(model, x, s, crease_out=gpu_c)
    dn = model.faces.download()
    shf = dict(ptr=dn["ptr"], idx=dn["idx"], psi=dn["psi"], dpsi=dn["dpsi"], ddpsi=dn["ddpsi"])
    sides = [ss.download() for ss in model.fold_sets[0]]
    sides = [dict(ptr=d["ptr"], idx=d["idx"], psi=d["psi"], dpsi=d["dpsi"], ddpsi=d["ddpsi"]) for d in sides]
    folds = fold_states(o, p, sides[0], sides[1], x)
    ref_c = []
    ref = J.compute_from_state(oracle_state(o, p, shf, x), p.faces.xy, p.faces.weight, p.node_xy, shf["ptr"],
                               shf["idx"], shf["dpsi"], shf["ddpsi"], p.thickness, s, folds,
                               face_force(o, p, shf, x), ref_c)
    for a, b in zip(gpu, ref):
        scale = max(abs(b["abs_sum_h"]), abs(b["abs_fold_h"]), abs(b["abs_sum"]), 1e-30)
        for k in J.FOLD_COLUMNS[4:]:
            assert abs(a[k] - b[k]) <= 1e-10 * max(abs(b[k]), scale), k
    for k in ("theta", "psi", "fn", "fT", "dpsi_ds"):
        assert np.allclose(gpu_c[0][k], ref_c[0][k], rtol=1e-10, atol=1e-14), k


def test_q_analytic_is_the_derivative_of_q_value():
    """qAnalytic's gradient and second gradient against central differences of qValue,
    inside the ring (cubic and linear q), and zero outside it."""
    ring = J.Ring(1.0, 2.5)
    rng = np.random.default_rng(15)
    ang = rng.uniform(0.0, 2.0 * math.pi, 40)
    rad = rng.uniform(1.05, 2.45, 40)
    P = np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1)
    hstep = 1e-5
    for linear in (False, True):
        q, g, H = J.q_analytic(P, ring, linear)
        assert np.array_equal(q, J.q_value(np.linalg.norm(P, axis=1), ring, linear))
        for c in range(2):
            e = np.zeros(2); e[c] = hstep
            qp = J.q_value(np.linalg.norm(P + e, axis=1), ring, linear)
            qm = J.q_value(np.linalg.norm(P - e, axis=1), ring, linear)
            assert np.abs((qp - qm) / (2 * hstep) - g[:, c]).max() <= 1e-8
            _, gp, _ = J.q_analytic(P + e, ring, linear)
            _, gm, _ = J.q_analytic(P - e, ring, linear)
            assert np.abs((gp - gm) / (2 * hstep) - H[:, :, c]).max() <= 1e-7
    q, g, H = J.q_analytic(np.array([[0.5, 0.0], [3.0, 0.0]]), ring, False)
    assert np.array_equal(q, [1.0, 0.0]) and not g.any() and not H.any()
