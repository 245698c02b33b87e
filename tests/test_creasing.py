"""Progressive creasing (plate/ProgressiveCreasing.h) over the oracle and the GPU library.

The reference's centre-crease smoke example publishes the last step of its run
(examples/smoke_centre_crease/README.md:14-20): the oracle's run of the same case reproduces
that row to its printed digits, which pins the whole chain (order-3 RKPM with cuts truncated
at the tips, the hinge with its exact tangent, the continuity rows, LineSearch, the energies
and the fold-angle average); the GPU run must then match the oracle's steps."""
import math
import os

import numpy as np
import pytest

import creasing_helpers as H
from curvami_gb300 import creasing as PC
from curvami_gb300 import mesh


# ---- host logic --------------------------------------------------------------------------

def _ab(st):
    return [(s.a, s.b) for s in st]


def test_schedule_middle_out():
    st = PC.schedule("middle_out", 1, 40, 10)
    assert _ab(st) == [(5, 5), (4, 6), (3, 7), (2, 8), (1, 9), (0, 10)]
    assert _ab(PC.schedule("middle_out", 2, 40, 10)) == [(5, 5), (3, 7), (1, 9), (0, 10)]
    assert _ab(PC.schedule("middle_out", 1, 40, 5)) == [(2, 2), (1, 3), (0, 4), (0, 5)]


def test_schedule_one_end_and_skip():
    assert _ab(PC.schedule("one_end", 2, 40, 5)) == [(0, 0), (0, 2), (0, 4), (0, 5)]
    assert _ab(PC.schedule("one_end", 1, 40, 4, skip=(2,))) == [(0, 0), (0, 1), (0, 3), (0, 4)]
    assert _ab(PC.schedule("one_end", 1, 40, 3, skip=(3,))) == [(0, 0), (0, 1), (0, 2), (0, 3)]
    assert _ab(PC.schedule("one_end_reverse", 2, 40, 5)) == [(5, 5), (3, 5), (1, 5), (0, 5)]


def test_schedule_ends_in_and_all_at_once():
    st = PC.schedule("ends_in", 1, 40, 6)
    assert _ab(st) == [(0, 6), (1, 5), (2, 4), (3, 3)] and all(s.outside for s in st)
    assert _ab(PC.schedule("ends_in", 1, 40, 6, skip=(1,))) == [(0, 6), (2, 4), (3, 3)]
    st = PC.schedule("all_at_once", 1, 4, 7)
    assert _ab(st) == [(0, 7)] * 5 and [s.frac for s in st] == [0.0, 0.25, 0.5, 0.75, 1.0]
    with pytest.raises(ValueError):
        PC.schedule("both_ways", 1, 40, 4)


def test_truncate_keeps_end_flags_only_at_path_ends():
    full = {"vertices": np.array([[0, 0], [1, 0], [2, 0], [3, 0]], float), "extend_start": True,
            "extend_end": True, "is_closed": False}
    c = PC.truncate(full, 0, 2)
    assert c["extend_start"] and not c["extend_end"] and len(c["vertices"]) == 3
    c = PC.truncate(full, 1, 3)
    assert not c["extend_start"] and c["extend_end"]
    ring = {"vertices": np.array([[0, 0], [1, 0], [1, 1], [0, 0]], float), "is_closed": True}
    assert PC.truncate(ring, 0, 3)["is_closed"] and not PC.truncate(ring, 0, 2)["is_closed"]


def test_arc_length_projection():
    v = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 2.0]])
    S_ = PC.cumulative_arc_length(v)
    assert np.allclose(S_, [0.0, 1.0, 3.0])
    assert PC.project_arc_length((0.25, 0.1), v, S_) == pytest.approx(0.25)
    assert PC.project_arc_length((1.2, 1.5), v, S_) == pytest.approx(2.5)
    assert PC.project_arc_length((-1.0, 0.0), v, S_) == 0.0


def test_fold_angle_averages_across_the_cut():
    th = np.deg2rad([179.0, -179.0, 178.0])
    w = np.ones(3)
    ref = PC.circular_mean_rad(th, w)
    assert abs(abs(ref) - math.pi) < math.radians(1.0)
    mean = PC.weighted_mean_about_circular_mean_rad(th, w)
    assert abs(abs(math.degrees(mean)) - 179.3333333) < 1e-6
    m, mx = PC.active_fold_angles(th, w, np.array([True, True, False]))
    assert abs(abs(m) - 180.0) < 1e-9 and abs(mx - 181.0) < 1e-9


def test_fixture_nodes_are_the_reference_mesh():
    root = os.environ.get("CURVAMI_REFERENCE")
    src = os.path.join(root or "", "examples", "smoke_centre_crease", "CB_n20.msh")
    if not root or not os.path.exists(src):
        pytest.skip("reference tree not present (set CURVAMI_REFERENCE to its root)")
    rxy, _ = mesh.read_msh41(src)
    fx = np.load(os.path.join(H.GOLDEN, "smoke_centre_crease_nodes.npy"))
    a = {tuple(p) for p in rxy.tolist()}
    b = {tuple(p) for p in fx.tolist()}
    assert a == b


# ---- the smoke case on the oracle (CPU) ---------------------------------------------------

@pytest.fixture(scope="module")
def oracle():
    from oracle.binding import Oracle

    return Oracle(native=False)


def test_smoke_case_oracle_reproduces_published_row(oracle, tmp_path):
    p, spec = H.smoke_plate(str(tmp_path / "smoke.msh"))
    plate = H.OracleCreasingPlate(oracle, p, spec, H.point_bcs())
    x = np.zeros(3 * len(p.node_xy))
    log = tmp_path / "smoke_steps.csv"
    res = PC.run(H.smoke_solver(), plate, x, [H.smoke_line(p)], cfg=H.smoke_config(str(log)))
    assert res.stopped == ""
    assert [r["step"] for r in res.steps] == [0, 1, 2, 3, 4, 5]
    assert all(r["newton_iters"] <= 5 for r in res.steps)   # "within 5 Newton iterations"
    H.assert_golden_row(res.steps[-1])
    fx = H.smoke_fixture()["oracle_steps"]
    for r, g in zip(res.steps, fx):
        for k in ("E_mem", "E_ben", "E_hin", "theta_mean_deg"):
            assert r[k] == pytest.approx(g[k], rel=1e-8, abs=1e-20), (r["step"], k)
    rows = log.read_text().splitlines()
    assert rows[1] == PC.CSV_COLUMNS and len(rows) == 2 + 6
    last = rows[-1].split(",")
    assert int(last[0]) == 5 and float(last[8]) == pytest.approx(res.steps[-1]["E_mem"], rel=1e-9)


def test_refit_l2_is_the_weighted_least_squares_fit(oracle, tmp_path):
    p, spec = H.smoke_plate(str(tmp_path / "smoke.msh"))
    plate = H.OracleCreasingPlate(oracle, p, spec, H.point_bcs())
    rng = np.random.default_rng(7)
    x = rng.normal(size=3 * len(p.node_xy)) * 1e-3
    ref = PC.Refitter("l2", 1.0)
    target = ref.sample(plate, x)
    plate.rebuild([PC.truncate(p.creases[0], 3, 7)])
    a = ref.fit(plate, target, x)
    faces, _ = plate.tables()
    sw = np.sqrt(p.faces.weight)[:, None]
    A = faces.P.toarray() * sw
    want = np.linalg.lstsq(A, target["face"][0] * sw, rcond=None)[0]
    got = a.reshape(-1, 3)
    assert np.abs(A @ got - A @ want).max() <= 1e-9 * np.abs(A @ want).max()
    with pytest.raises(ValueError):
        PC.Refitter("h2", 1.0)


# ---- the GPU path -------------------------------------------------------------------------

def _gpu_smoke(tmp_path, mixed=False):
    from curvami_gb300.api import PlateModel

    p, spec = H.smoke_plate(str(tmp_path / "smoke.msh"))
    model = PlateModel(p)
    plate = PC.GpuCreasingPlate(model, H.point_bcs(), [spec], exact_tangent=True, mixed=mixed)
    return p, model, plate


@pytest.mark.gpu
def test_smoke_case_gpu_matches_oracle_and_published_row(tmp_path):
    p, model, plate = _gpu_smoke(tmp_path)
    x = np.zeros(3 * len(p.node_xy))
    res = PC.run(H.smoke_solver(), plate, x, [H.smoke_line(p)], cfg=H.smoke_config())
    assert res.stopped == ""
    assert all(r["newton_iters"] <= 5 for r in res.steps)
    H.assert_golden_row(res.steps[-1])
    for r, g in zip(res.steps, H.smoke_fixture()["oracle_steps"]):
        assert r["newton_iters"] == g["newton_iters"]
        for k in ("E_mem", "E_ben", "E_hin", "theta_mean_deg", "theta_max_deg"):
            assert r[k] == pytest.approx(g[k], rel=1e-8, abs=1e-20), (r["step"], k)


@pytest.mark.gpu
def test_smoke_case_gpu_mixed_reaches_the_same_states(tmp_path):
    """The mixed assembly (FP32 tangent) converges to the same equilibria: its residual is
    FP64, only the Newton path may differ."""
    p, model, plate = _gpu_smoke(tmp_path, mixed=True)
    x = np.zeros(3 * len(p.node_xy))
    res = PC.run(H.smoke_solver(), plate, x, [H.smoke_line(p)], cfg=H.smoke_config())
    assert res.stopped == ""
    H.assert_golden_row(res.steps[-1])
    for r, g in zip(res.steps, H.smoke_fixture()["oracle_steps"]):
        for k in ("E_mem", "E_ben", "E_hin", "theta_mean_deg"):
            assert r[k] == pytest.approx(g[k], rel=1e-6, abs=1e-20), (r["step"], k)


@pytest.mark.gpu
def test_rebuild_equals_fresh_build_and_updates_assembly(tmp_path):
    """cgb_shape_rebuild gives the bits of a fresh cgb_shape_build with the same cuts, and an
    assembler built before the rebuild (FP32 copies, sliced-ELL copy, a captured graph)
    assembles what a new assembler on the rebuilt set assembles."""
    import torch
    from curvami_gb300 import _lib as L
    from curvami_gb300.api import NonLinearAssembler, shape_functions

    p, model, plate = _gpu_smoke(tmp_path)
    cut = [PC.truncate(p.creases[0], 2, 7)]
    kw = dict(rho=p.rho, order=p.order, kernel=p.kernel)
    rng = np.random.default_rng(3)
    x = rng.normal(size=3 * len(p.node_xy)) * 0.02
    flags = L.TANGENT | L.HINGE | L.DETERMINISTIC
    for mixed in (False, True):
        f = flags | (L.MIXED if mixed else 0)
        model.asm.assemble(x, f)                       # make the assembler's derived copies
    d_x = torch.from_numpy(x).cuda()
    d_K = torch.zeros(model.asm.nnz, dtype=torch.float64, device="cuda")
    d_F = torch.zeros(3 * len(p.node_xy), dtype=torch.float64, device="cuda")
    g = model.asm.graph(d_x.data_ptr(), d_K.data_ptr(), d_F.data_ptr(), flags | L.MIXED)
    model.rebuild(cut)
    fresh = shape_functions(model.ctx, p.faces.xy, creases=cut, **kw)
    a, b = model.faces.download(), fresh.download()
    for k in ("idx", "psi", "dpsi", "ddpsi"):
        assert np.array_equal(a[k], b[k]), k
    fold = dict(model.fold_specs[0])
    asm2 = NonLinearAssembler(model.ctx, fresh, p.faces.weight, [fold])
    asm2.set_material(model.asm.A, model.asm.B, model.asm.D)
    for mixed in (False, True):
        f = flags | (L.MIXED if mixed else 0)
        K1, F1 = model.asm.assemble(x, f)
        K2, F2 = asm2.assemble(x, f)
        assert np.array_equal(K1, K2) and np.array_equal(F1, F2), mixed
    g.launch()
    model.ctx.synchronize()
    K2, F2 = asm2.assemble(x, flags | L.MIXED)
    assert np.array_equal(d_K.cpu().numpy(), K2) and np.array_equal(d_F.cpu().numpy(), F2)
    g.close()
    asm2.close()


@pytest.mark.gpu
def test_fold_state_energy_and_hinge_match_oracle(tmp_path):
    from oracle.binding import Oracle
    from curvami_gb300 import _lib as L

    o = Oracle(native=False)
    p, model, plate = _gpu_smoke(tmp_path)
    oplate = H.OracleCreasingPlate(o, p, H.smoke_plate(str(tmp_path / "s2.msh"))[1], H.point_bcs())
    n = len(p.folds[0].left.xy)
    active = (np.arange(n) % 3 != 0).astype(np.int8)
    theta0 = np.linspace(-0.02, 0.03, n)
    plate.set_fold_state(0, theta0, active)
    oplate.set_fold_state(0, theta0, active)
    rng = np.random.default_rng(11)
    x = rng.normal(size=3 * len(p.node_xy)) * 0.01
    eg = plate.energies(x)
    eo = oplate.energies(x)
    assert np.allclose(eg, eo, rtol=1e-10, atol=1e-300)
    K1, F1 = model.asm.assemble(x, L.TANGENT | L.HINGE | L.HINGE_EXACT)
    K2, F2 = oplate.assemble(x, True)
    assert np.abs(F1 - F2).max() <= 1e-10 * np.abs(F2).max()
    assert np.linalg.norm(K1 - K2) <= 1e-10 * np.linalg.norm(K2)
