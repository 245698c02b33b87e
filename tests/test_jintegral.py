"""The domain-integral energy release rate (curvami_gb300/jintegral.py) on the CPU, with the
point state from the oracle's Kinematics::compute + Constitutive, and on the GPU state.

- a rigid motion has B = 0: every G vanishes;
- a uniform in-plane stretch has B uniform: the mean-subtracted G_c vanishes to round-off,
  G itself is the quadrature leak B sum w grad q;
- vw1_h h (the virtual work with the interpolated q) equals the assembly's nodal residual
  sum_I q_I d . F_int,I for any displacement (JIntegral.h's own check of vw);
- the GPU state gives the oracle state's values (GPU test);
- the CSV carries the reference's columns.
"""
import math

import numpy as np
import pytest

from curvami_gb300 import jintegral as J
from curvami_gb300 import synth
from oracle import Oracle


@pytest.fixture(scope="module")
def o():
    return Oracle(native=True)


@pytest.fixture(scope="module")
def plate_shapes(o):
    p = synth.square_plate(15, 0.5, 3, jitter=0.05, crease=None, seed=31)
    ptr, idx, s = o.frnn(p.node_xy, p.faces.xy, p.rho)
    psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, p.faces.xy, ptr, idx, s, p.rho, p.order)
    assert rc == 0
    return p, dict(ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi)


def oracle_state(o, p, sh, x):
    A, B, D = (np.asarray(m).reshape(3, 3) for m in o.abd(p.E, p.nu, p.thickness))
    n = len(sh["ptr"]) - 1
    st = np.zeros((n, 33))
    X = np.asarray(x).reshape(-1, 3)
    for g in range(n):
        k = o.kinematics(g, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"], x)
        e = slice(sh["ptr"][g], sh["ptr"][g + 1])
        st[g, 0:3] = (sh["psi"][e][:, None] * X[sh["idx"][e]]).sum(0)
        st[g, 3:21] = k[0:18]
        st[g, 21:27] = k[22:28]
        e0 = np.array([k[22], k[23], 2 * k[24]])
        e1 = np.array([k[25], k[26], 2 * k[27]])
        st[g, 27:30] = A @ e0 + B @ e1
        st[g, 30:33] = B.T @ e0 + D @ e1
    return st


def settings(p):
    c = p.node_xy.mean(0)
    return J.Settings(tip=tuple(c), dir=(math.cos(0.3), math.sin(0.3)), rings=[J.Ring(0.8, 2.0), J.Ring(1.2, 2.6)])


def run(o, p, sh, x, s):
    st = oracle_state(o, p, sh, x)
    return J.compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, sh["ptr"], sh["idx"], sh["dpsi"],
                                sh["ddpsi"], p.thickness, s)


def test_rigid_motion_releases_nothing(o, plate_shapes):
    p, sh = plate_shapes
    th = 0.4
    R = np.array([[math.cos(th), -math.sin(th), 0.0], [math.sin(th), math.cos(th), 0.0], [0.0, 0.0, 1.0]])
    X3 = np.c_[p.node_xy, np.zeros(len(p.node_xy))]
    x = (X3 @ R.T - X3 + np.array([0.3, -0.2, 0.1])).ravel()
    for r in run(o, p, sh, x, settings(p)):
        for k in ("G1", "G2", "G1_c", "G1_h", "G1_d", "G1_m", "G1_s", "vw1_h"):
            assert abs(r[k]) < 1e-12, k


def test_uniform_stretch_mean_subtracted_vanishes(o, plate_shapes):
    p, sh = plate_shapes
    eps = 1e-3
    x = np.c_[eps * p.node_xy[:, 0], 0.5 * eps * p.node_xy[:, 1], np.zeros(len(p.node_xy))].ravel()
    res = run(o, p, sh, x, settings(p))
    st = oracle_state(o, p, sh, x)
    B, _, _ = J.eshelby(J._tensors(st))
    scale = float(np.abs(B).max()) / p.thickness
    for r in res:
        assert r["n_gp"] > 0
        assert abs(r["G1_c"]) < 1e-10 * scale and abs(r["G2_c"]) < 1e-10 * scale
        # G is the leak of the uniform B through the quadrature of grad q
        assert abs(r["G1"]) <= scale * r["grad_q_sum"] * 1.01 + 1e-15


def test_interpolated_virtual_work_is_the_nodal_residual(o, plate_shapes):
    p, sh = plate_shapes
    x = 0.05 * synth.fourier_field(p.node_xy, np.random.default_rng(3), lam=(3.0, 9.0))
    s = settings(p)
    res = run(o, p, sh, x, s)
    A, B, D = o.abd(p.E, p.nu, p.thickness)
    outer, inner, col_ptr, col_nodes, mp = o.pattern(len(p.node_xy), sh["ptr"], sh["idx"])
    _, F = o.update_stiffness(len(p.node_xy), p.faces.weight, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"], outer,
                              mp, x, A, B, D, want_K=False)
    d = np.array(s.dir) / np.linalg.norm(s.dir)
    Fn = F.reshape(-1, 3)
    for r, ring in zip(res, s.rings):
        qn = J.q_value(np.linalg.norm(p.node_xy - np.array(s.tip), axis=1), ring, s.linear_q)
        nodal = float(qn @ (Fn[:, 0] * d[0] + Fn[:, 1] * d[1]))
        assert abs(r["vw1_h"] * p.thickness - nodal) <= 1e-10 * float(np.abs(Fn).sum())


def test_csv_columns(tmp_path, o, plate_shapes):
    p, sh = plate_shapes
    x = np.zeros(3 * len(p.node_xy))
    s = settings(p)
    res = run(o, p, sh, x, s)
    path = str(tmp_path / "G.csv")
    J.write_csv(path, 3, s, res, p.thickness, True)
    J.write_csv(path, 4, s, res, p.thickness, False)
    lines = open(path).read().splitlines()
    assert lines[0].startswith("# energy release rate, domain integral")
    assert lines[1].split(",") == J.CSV_COLUMNS
    assert len(lines) == 2 + 2 * len(s.rings)
    assert lines[2].split(",")[:2] == ["3", "0"] and lines[-1].split(",")[:2] == ["4", "1"]


@pytest.mark.gpu
def test_gpu_state_matches_oracle(o, plate_shapes):
    import curvami_gb300 as cg

    p, _ = plate_shapes
    model = cg.PlateModel(p)
    x = 0.05 * synth.fourier_field(p.node_xy, np.random.default_rng(4), lam=(3.0, 9.0))
    s = settings(p)
    gpu = J.compute(model, x, s)
    dn = model.faces.download()
    ref = run(o, p, dict(ptr=dn["ptr"], idx=dn["idx"], psi=dn["psi"], dpsi=dn["dpsi"], ddpsi=dn["ddpsi"]), x, s)
    for a, b in zip(gpu, ref):
        for k in J.CSV_COLUMNS[2:]:
            assert abs(a[k] - b[k]) <= 1e-10 * max(abs(b[k]), abs(b["abs_sum"]), 1e-30), k


def test_natural_curvature_band_term_balances_the_plate_term(o, plate_shapes):
    """A flat, unloaded plate with a natural-curvature band: E1 = 0, M = D kappa_bar and
    W_h = 1/2 kappa_bar D11 kappa_bar depend on X only through the band, with
    dW_h/dX = M : d(kappa_bar)/dX. So the plate term -(1/h) sum w W_h d.grad q and the band
    term -(1/h) sum w q M : d(kappa_bar)/dX . d add up to -(1/h) int d.grad(q W_h), zero for a
    q that vanishes on the outer ring: G1 + Gband_a and G1_h + Gband_h (G1b_h) vanish to the
    quadrature error while each term does not (JIntegral.h:145-166, 492-520)."""
    p, sh = plate_shapes
    n = len(sh["ptr"]) - 1
    c = p.node_xy.mean(0)
    nc = {"x0": float(c[0]) + 0.3, "width": 0.8, "angle_deg": 20.0, "sense": "valley"}
    kb, _ = J.natural_kappa(p.faces.xy[:, 0], nc)
    D = np.asarray(o.abd(p.E, p.nu, p.thickness)[2]).reshape(3, 3)
    st = np.zeros((n, 33))
    st[:, 3] = 1.0                 # r_X = e_x
    st[:, 7] = 1.0                 # r_Y = e_y
    st[:, 20] = 1.0                # b = e_z
    st[:, 30:33] = kb[:, None] * D[:, 0][None, :]   # M = D (kappa_bar, 0, 0)
    s = J.Settings(tip=tuple(c), dir=(1.0, 0.0), rings=[J.Ring(1.0, 2.5)])
    r = J.compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, sh["ptr"], sh["idx"], sh["dpsi"],
                             sh["ddpsi"], p.thickness, s, natural_curvature=nc, psi=sh["psi"])[0]
    assert abs(r["Gband_a"]) > 0 and abs(r["G1"]) > 0
    assert abs(r["G1"] + r["Gband_a"]) <= 5e-3 * abs(r["Gband_a"])
    assert abs(r["G1b_h"]) <= 5e-3 * abs(r["Gband_h"])
    # without the band every band column is zero and G1b_h is G1_h
    st[:, 30:33] = 0.0
    r0 = J.compute_from_state(st, p.faces.xy, p.faces.weight, p.node_xy, sh["ptr"], sh["idx"], sh["dpsi"],
                              sh["ddpsi"], p.thickness, s)[0]
    assert r0["Gband_h"] == 0.0 and r0["G1b_h"] == r0["G1_h"]
