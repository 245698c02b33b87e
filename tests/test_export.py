"""Post-processing: the exporter's step table, flatness and crease rows, and the stress
sampler (plate/Exporter.h, plate/StressSampler.h), host logic on the CPU and the GPU's
point state against the oracle's Kinematics::compute."""
import math

import numpy as np
import pytest

from curvami_gb300 import export as X


def _state_from(F0, E0, E1, b=(0.0, 0.0, 1.0), u=(0.0, 0.0, 0.0)):
    st = np.zeros((1, 33))
    st[0, 0:3] = u
    st[0, 3:6] = F0[:, 0]
    st[0, 6:9] = F0[:, 1]
    st[0, 18:21] = b
    st[0, 21:24] = [E0[0, 0], E0[1, 1], E0[0, 1]]
    st[0, 24:27] = [E1[0, 0], E1[1, 1], E1[0, 1]]
    return st


def test_surface_stress_uniform_stretch():
    """u = eps X: F = diag(1 + eps, 1) in-plane, E0_xx = eps + eps^2 / 2, S = Q E, sigma = F S F^T / J."""
    eps = 0.01
    F0 = np.array([[1.0 + eps, 0.0], [0.0, 1.0], [0.0, 0.0]])
    E0 = 0.5 * (F0.T @ F0 - np.eye(2))
    st = _state_from(F0, E0, np.zeros((2, 2)))
    E, nu, h = 2.0, 0.25, 0.1
    Q = E / (1 - nu * nu) * np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
    N2, T2 = np.array([1.0, 0.0]), np.array([0.0, 1.0])
    sig_nn, tau, S_nn, J = X.surface_stress(st, Q, 0.5 * h, N2, T2)
    S = Q @ np.array([E0[0, 0], E0[1, 1], 0.0])
    assert J[0] == pytest.approx(1.0 + eps)
    assert S_nn[0] == pytest.approx(S[0])
    assert sig_nn[0] == pytest.approx((1 + eps) ** 2 * S[0] / (1 + eps))
    assert abs(tau[0]) < 1e-15
    zero = X.surface_stress(_state_from(np.eye(3)[:, :2], np.zeros((2, 2)), np.zeros((2, 2))), Q, 0.05, N2, T2)
    assert all(abs(v[0]) < 1e-15 for v in zero[:3]) and zero[3][0] == 1.0


def test_step_table_columns_and_unknown_field(capsys):
    st = _state_from(np.eye(3)[:, :2], np.array([[1e-3, 2e-3], [2e-3, 3e-3]]), np.array([[4.0, 5.0], [5.0, 6.0]]),
                     b=(0.0, math.sin(0.1), math.cos(0.1)), u=(0.1, 0.2, 0.3))
    t = X.step_table(np.array([[1.0, 2.0]]), st, ["E_XX", "K_XY", "bogus"])
    assert t.shape == (1, 10)
    assert np.allclose(t[0, :5], [1.0, 2.0, 0.1, 0.2, 0.3])
    assert t[0, 5] == pytest.approx(-math.degrees(0.1)) and t[0, 6] == pytest.approx(0.0)
    assert t[0, 7] == 1e-3 and t[0, 8] == 5.0 and t[0, 9] == 0.0
    assert "bogus" in capsys.readouterr().err


def test_planarity_and_chain():
    rng = np.random.default_rng(0)
    n = 200
    tab = np.zeros((n, 7))
    tab[:, 0:2] = rng.uniform(-1, 1, (n, 2))
    tab[:, 4] = 0.3 * tab[:, 0] - 0.2 * tab[:, 1] + 0.05         # a tilted plane
    rms, mx, diag = X.planarity(tab)
    assert rms < 1e-7 and mx < 1e-12 and diag == pytest.approx(np.hypot(*(tab[:, :2].max(0) - tab[:, :2].min(0))))
    tab[0, 4] += 0.1
    assert X.planarity(tab)[1] > 0.05
    xs = np.array([0.3, 0.0, 0.9, 0.6, 0.1])
    xy = np.stack([xs, np.zeros_like(xs)], 1)
    order = X.chain_order(xy)
    assert [xs[i] for i in order] in (sorted(xs), sorted(xs, reverse=True))
    cr = X.crease_table([(0, 5, xy, np.full(5, 0.2), np.arange(5.0))])
    assert cr.shape == (5, 7) and np.allclose(cr[:, 4], 0.1 + 0.2 * np.arange(5))


def test_step_writer_roundtrip(tmp_path):
    w = X.StepWriter(str(tmp_path / "run"))
    tab = np.arange(14.0).reshape(2, 7)
    assert w.write(3, tab, [], np.zeros((0, 7)), angles=[12.5], is_driver=[1], E_mem=1.0)
    d = np.load(w.path(3))
    assert np.array_equal(d["data"], tab) and d["angles"][0] == 12.5 and float(d["E_mem"]) == 1.0
    assert list(d["columns"])[:3] == ["X", "Y", "u"]


@pytest.mark.gpu
def test_point_state_matches_oracle_kinematics():
    from oracle.binding import Oracle
    from curvami_gb300.api import PlateModel
    from curvami_gb300 import synth

    o = Oracle(native=False)
    p = synth.config_smallplate(rule=3)
    model = PlateModel(p)
    rng = np.random.default_rng(5)
    x = synth.fourier_field(p.node_xy, rng, lam=(4.0, 20.0))
    st = X.point_state(model.ctx, model.faces, x, model.asm.A, model.asm.B, model.asm.D)
    d = model.faces.download()
    A, B, D = (np.asarray(M).reshape(3, 3) for M in (model.asm.A, model.asm.B, model.asm.D))
    for g in rng.choice(p.faces.xy.shape[0], 200, replace=False):
        k = o.kinematics(int(g), d["ptr"], d["idx"], d["dpsi"], d["ddpsi"], x)
        e = slice(d["ptr"][g], d["ptr"][g + 1])
        u = (d["psi"][e][:, None] * x.reshape(-1, 3)[d["idx"][e]]).sum(0)
        got = st[g]
        assert np.allclose(got[0:3], u, rtol=1e-12, atol=1e-13)
        assert np.allclose(got[3:18], k[0:15], rtol=1e-12, atol=1e-12)
        assert np.allclose(got[18:21], k[15:18], rtol=1e-12, atol=1e-13)
        assert np.allclose(got[21:27], k[22:28], rtol=1e-10, atol=1e-13)
        e0 = np.array([k[22], k[23], 2 * k[24]]); e1 = np.array([k[25], k[26], 2 * k[27]])
        assert np.allclose(got[27:30], A @ e0 + B @ e1, rtol=1e-10, atol=1e-15)
        assert np.allclose(got[30:33], B.T @ e0 + D @ e1, rtol=1e-10, atol=1e-15)


@pytest.mark.gpu
def test_export_step_and_stress_rays_on_smoke_case(tmp_path):
    import creasing_helpers as H
    from curvami_gb300 import creasing as PC
    from curvami_gb300.api import PlateModel

    case = H.smoke_case(str(tmp_path / "smoke.msh"))
    model = PlateModel(case.plate)
    rng = np.random.default_rng(2)
    x = rng.normal(size=3 * len(case.plate.node_xy)) * 1e-3
    w = X.StepWriter(str(tmp_path / "smoke"))
    tab, cr = X.export_step(model, x, 0, ["E_XX", "E_YY", "E_XY", "K_XX", "K_YY", "K_XY"], fold_tags=[5],
                            writer=w, E_mem=1.0)
    assert tab.shape == (3600, 13) and cr.shape == (10, 7)
    assert np.allclose(np.sort(cr[:, 4]), 0.05 + 0.1 * np.arange(10))
    d = np.load(w.path(0))
    assert d["data"].shape == (3600, 13) and float(d["planar_rms"]) > 0.0
    s = X.StressSettings(tip=(0.5, 0.0), dir=(1.0, 0.0), r_max=0.3, dr=0.05, angles_deg=[-90, 0, 90],
                         stem=str(tmp_path / "st"))
    rays = X.stress_rays(model, x, 0, s, case.plate.creases, h=case.plate.thickness)
    assert set(rays) == {-90, 0, 90} and all(r.shape[1] == 16 for r in rays.values())
    head = open(str(tmp_path / "st") + "_s0_p+000.csv").read().splitlines()[1]
    assert head == X.STRESS_COLUMNS
    del PC
