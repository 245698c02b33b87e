"""GPU parity: the sm_103a library through its C ABI against the CPU oracle.

Bars: neighbour sets, distances, the K pattern and the Gauss-point -> CSC map bit-exact;
FP64 shape functions to 1e-12 of each array's scale where the supports are well
conditioned (crease-truncated supports are ill-conditioned, looser bound stated); the
FP64 assembly on identical shape functions to 1e-13; the mixed assembly's residual to
1e-12 (the metric requires <= 1e-10) and its tangent to 1e-5 (FP32); the deterministic
scatter bitwise run to run.
"""
import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import synth
from oracle import Oracle

pytestmark = pytest.mark.gpu

# The mixed tangent's default is the CUDA-core one (cgb_tuning.tangent_kind 0).
TENSOR_DEFAULT = False


@pytest.fixture(scope="module")
def o():
    return Oracle()


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as ge

    ge.build()
    c = cg.Context(0)
    yield c


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def oracle_shapes(o, p, pts):
    ptr, idx, s = o.frnn(p.node_xy, pts, p.rho, p.rho_node)
    psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, pts, ptr, idx, s, p.rho, p.order, p.creases, p.rho_node,
                                       p.kernel)
    return dict(ptr=ptr, idx=idx, s=s, psi=psi, dpsi=dpsi, ddpsi=ddpsi, bad=bad, rc=rc)


def crease_distance(p, pts):
    d = np.full(len(pts), np.inf)
    for cr in p.creases:
        V = np.asarray(cr["vertices"])
        for a, b in zip(V[:-1], V[1:]):
            v = b - a
            t = np.clip(((pts - a) @ v) / (v @ v), 0.0, 1.0)
            d = np.minimum(d, np.linalg.norm(pts - (a + t[:, None] * v), axis=1))
    return d


SHAPE_CASES = {
    "row_r3_quartic": lambda: synth.square_plate(21, 0.5, 3, crease="row", seed=1),
    "arc_r4_jitter": lambda: synth.square_plate(25, 0.5, 4, jitter=0.1, crease="arc", seed=2),
    "nocrease_order1": lambda: synth.square_plate(15, 0.5, 3, jitter=0.05, crease=None, order=1, seed=3),
    "nocrease_order3": lambda: synth.square_plate(15, 0.5, 3, jitter=0.05, crease=None, order=3,
                                                  rho_factor=4.5, seed=3),
    "cubic_bspline": lambda: synth.square_plate(15, 0.5, 4, jitter=0.05, crease="row", kernel=1, seed=4),
    "three_arcs": lambda: synth.batched_plate(31, np.random.default_rng(6)),
    "three_cuts": lambda: synth.batched_plate(31, np.random.default_rng(7)),
    "six_cuts_with_tips": lambda: synth.many_cuts_plate(61, 6),
}


@pytest.mark.parametrize("name", sorted(SHAPE_CASES))
def test_shape_functions(o, ctx, name):
    p = SHAPE_CASES[name]()
    ctx.set_nodes(p.node_xy)
    sh = cg.shape_functions(ctx, p.faces.xy, p.rho, p.order, p.creases, p.rho_node, p.kernel).download()
    ref = oracle_shapes(o, p, p.faces.xy)
    assert np.array_equal(sh["ptr"], ref["ptr"])
    assert np.array_equal(sh["idx"], ref["idx"])
    assert np.array_equal(sh["s"], ref["s"])
    # Points whose support a crease truncates have ill-conditioned moment matrices (the
    # visible nodes lie on one side), so two FP64 evaluations differ there by about
    # cond(M) * eps; away from the creases the bar is 1e-12.
    far = np.repeat(crease_distance(p, p.faces.xy) > p.rho, np.diff(ref["ptr"]))
    for k in ("psi", "dpsi", "ddpsi"):
        assert rel(sh[k][far], ref[k][far]) < 1e-12, k
        assert rel(sh[k], ref[k]) < 1e-8, k


def test_shape_functions_per_node_radius(o, ctx):
    plate, pts = synth.config_shape_points(n_points=20000, n_side=61, per_node_rho=True, seed=11)
    ctx.set_nodes(plate.node_xy)
    sh = cg.shape_functions(ctx, pts, plate.rho, 2, plate.creases, plate.rho_node, plate.kernel).download()
    ref = oracle_shapes(o, plate, pts)
    assert np.array_equal(sh["ptr"], ref["ptr"]) and np.array_equal(sh["idx"], ref["idx"])
    assert np.array_equal(sh["s"], ref["s"])
    far = np.repeat(crease_distance(plate, pts) > 1.75, np.diff(ref["ptr"]))
    for k in ("psi", "dpsi", "ddpsi"):
        assert rel(sh[k][far], ref[k][far]) < 1e-12, k
        assert rel(sh[k], ref[k]) < 1e-8, k


def test_empty_and_isolated_points(o, ctx):
    p = synth.square_plate(9, 0.5, 2, crease=None)
    ctx.set_nodes(p.node_xy)
    sh = cg.shape_functions(ctx, np.zeros((0, 2)), p.rho, 2)
    assert sh.n_gp == 0 and sh.nnz == 0
    with pytest.raises(cg.CGBError) as e:  # no neighbours: singular moment matrix
        cg.shape_functions(ctx, np.array([[100.0, 100.0]]), p.rho, 2)
    assert e.value.code == 3 and "singular moment matrix" in str(e.value)


def test_singular_support_message(ctx):
    nodes = np.array([[0.0, 0.0], [0.5, 0.0], [1.0, 0.0]])
    ctx.set_nodes(nodes)
    with pytest.raises(cg.CGBError) as e:
        cg.shape_functions(ctx, np.array([[0.5, 0.0]]), 1.5, 2)
    assert e.value.code in (3, 4)
    assert str(e.value).startswith("RKPM:")


# ---- assembly ---------------------------------------------------------------------------

class Case:
    """A plate with GPU shape functions for folds, oracle shape functions uploaded for the
    faces (so both sides assemble from identical inputs), and the oracle's K and F."""

    def __init__(self, o, ctx, p, x):
        self.p, self.x = p, x
        ctx.set_nodes(p.node_xy)
        self.model = cg.PlateModel(p, ctx)
        self.ref = oracle_shapes(o, p, p.faces.xy)
        r = self.ref
        self.faces_o = cg.shape_from_host(ctx, r["ptr"], r["idx"], r["dpsi"], r["ddpsi"], r["psi"])
        self.asm = cg.NonLinearAssembler(ctx, self.faces_o, p.faces.weight, self.model.fold_specs)
        self.asm.set_material(*cg.abd_isotropic(p.E, p.nu, p.thickness))
        self.folds = []
        for (L, R), f in zip(self.model.fold_sets, p.folds):
            dl, dr = L.download(), R.download()
            self.folds.append({"left": {"ptr": dl["ptr"], "idx": dl["idx"], "dpsi": dl["dpsi"]},
                               "right": {"ptr": dr["ptr"], "idx": dr["idx"], "dpsi": dr["dpsi"]},
                               "weight": f.left.weight, "tangent": f.left.tangent, "Kt": f.Kt,
                               "theta0": f.theta0})
        (self.outer, self.inner, self.col_ptr, self.col_nodes,
         self.mp) = o.pattern(p.n_nodes, r["ptr"], r["idx"], self.folds)
        self.A, self.B, self.D = o.abd(p.E, p.nu, p.thickness)
        self.o = o

    def oracle(self, x, hinge=True, exact=False, want_K=True):
        r = self.ref
        K, F = self.o.update_stiffness(self.p.n_nodes, self.p.faces.weight, r["ptr"], r["idx"], r["dpsi"],
                                       r["ddpsi"], self.outer, self.mp, x, self.A, self.B, self.D,
                                       want_K=want_K)
        if hinge:
            K, F = self.o.hinge(self.p.n_nodes, x, self.folds, self.outer, self.col_ptr, self.col_nodes,
                                K, F, exact_tangent=exact)
        return K, F


@pytest.fixture(scope="module")
def arc_case(o, ctx):
    p = synth.square_plate(23, 0.5, 4, jitter=0.08, seed=21, crease="arc", Kt=1e-3)
    x = 0.3 * synth.fourier_field(p.node_xy, np.random.default_rng(22), lam=(3.0, 10.0))
    return Case(o, ctx, p, x)


@pytest.fixture(scope="module")
def row_case(o, ctx):
    p = synth.config_smallplate(rule=3)
    x = 0.2 * synth.fourier_field(p.node_xy, np.random.default_rng(23), lam=(5.0, 20.0))
    return Case(o, ctx, p, x)


@pytest.mark.parametrize("which", ["arc", "row"])
def test_pattern_and_map_bit_exact(which, arc_case, row_case):
    c = arc_case if which == "arc" else row_case
    outer, inner = c.asm.pattern()
    assert np.array_equal(outer, c.outer) and np.array_equal(inner, c.inner)
    assert np.array_equal(c.asm.csr_mapping(), c.mp)
    # the GPU-built shape set gives the same pattern
    o2, i2 = c.model.asm.pattern()
    assert np.array_equal(o2, c.outer) and np.array_equal(i2, c.inner)


@pytest.mark.parametrize("which", ["arc", "row"])
@pytest.mark.parametrize("det", [False, True])
def test_fp64_assembly(which, det, arc_case, row_case):
    c = arc_case if which == "arc" else row_case
    Ko, Fo = c.oracle(c.x)
    fl = cg.TANGENT | cg.HINGE | (cg.DETERMINISTIC if det else 0)
    K, F = c.asm.assemble(c.x, fl)
    assert rel(K, Ko) < 1e-13
    assert rel(F, Fo) < 1e-13


@pytest.mark.parametrize("which", ["arc", "row"])
@pytest.mark.parametrize("det", [False, True])
def test_mixed_assembly(which, det, arc_case, row_case):
    c = arc_case if which == "arc" else row_case
    Ko, Fo = c.oracle(c.x)
    fl = cg.TANGENT | cg.HINGE | cg.MIXED | (cg.DETERMINISTIC if det else 0)
    K, F = c.asm.assemble(c.x, fl)
    assert rel(F, Fo) < 1e-12  # FP64 residual
    assert rel(K, Ko) < 1e-5   # FP32-class tangent
    # Frobenius: 1e-6 for the default FP32 CUDA cores (measured 1e-7); the tensor-core
    # tangent's 3xTF32 products (the lo x lo term dropped) accumulate in the tensor core's
    # FP32: 3e-6 (measured 0.9e-6 - 1.3e-6).
    assert np.linalg.norm(K - Ko) / np.linalg.norm(Ko) < (3e-6 if TENSOR_DEFAULT else 1e-6)


def test_residual_only_matches(arc_case):
    c = arc_case
    _, F_full = c.asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.DETERMINISTIC)
    _, F_res = c.asm.assemble(c.x, cg.HINGE | cg.DETERMINISTIC)
    assert np.array_equal(F_full, F_res)  # same fixed-order sums with and without K
    _, F_res = c.asm.assemble(c.x, cg.HINGE)
    assert rel(F_res, F_full) < 1e-14     # atomics: same terms, order varies
    _, Fo = c.oracle(c.x, want_K=False)
    assert rel(F_res, Fo) < 1e-13


def test_no_hinge_flag(arc_case):
    c = arc_case
    Ko, Fo = c.oracle(c.x, hinge=False)
    K, F = c.asm.assemble(c.x, cg.TANGENT)
    assert rel(K, Ko) < 1e-13 and rel(F, Fo) < 1e-13


def test_exact_hinge_tangent(arc_case):
    c = arc_case
    Ko, Fo = c.oracle(c.x, exact=True)
    K, F = c.asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.HINGE_EXACT)
    # the Hessian is a central difference of the gradient (step 1e-6), so the two
    # implementations agree to the difference stencil's sensitivity, not to round-off
    assert rel(K, Ko) < 1e-9 and rel(F, Fo) < 1e-13


def test_deterministic_bitwise(ctx, arc_case):
    c = arc_case
    # a second assembler over the same inputs builds the same ordered lists (an assembler
    # takes its node count from the context's nodes when it is created)
    ctx.set_nodes(c.p.node_xy)
    other = cg.NonLinearAssembler(ctx, c.faces_o, c.p.faces.weight, c.model.fold_specs)
    other.set_material(*cg.abd_isotropic(c.p.E, c.p.nu, c.p.thickness))
    for fl in (cg.TANGENT | cg.HINGE | cg.DETERMINISTIC, cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC):
        K1, F1 = c.asm.assemble(c.x, fl)
        K2, F2 = c.asm.assemble(c.x, fl)
        K3, F3 = other.assemble(c.x, fl)
        assert np.array_equal(K1, K2) and np.array_equal(F1, F2)
        assert np.array_equal(K1, K3) and np.array_equal(F1, F3)


def test_assembly_with_coupling(ctx, arc_case):
    """B != 0 (an unsymmetric [0/45] layup): the general P = A Bm + B Bb, Q = B Bm + D Bb
    path of every tangent kernel (FP64, FP32 merged, deterministic) against the oracle."""
    c = arc_case
    A, B, D = cg.abd_laminate([(1.0, 0.6, 0.25, 0.3, 0.0, 0.02), (1.4, 0.9, 0.3, 0.45, 45.0, 0.03)])
    assert np.abs(B).max() > 0
    ctx.set_nodes(c.p.node_xy)
    asm = cg.NonLinearAssembler(ctx, c.faces_o, c.p.faces.weight, c.model.fold_specs)
    asm.set_material(A, B, D)
    r = c.ref
    Ko, Fo = c.o.update_stiffness(c.p.n_nodes, c.p.faces.weight, r["ptr"], r["idx"], r["dpsi"], r["ddpsi"],
                                  c.outer, c.mp, c.x, A, B, D)
    Ko, Fo = c.o.hinge(c.p.n_nodes, c.x, c.folds, c.outer, c.col_ptr, c.col_nodes, Ko, Fo)
    for fl, tolK in ((0, 1e-13), (cg.DETERMINISTIC, 1e-13), (cg.MIXED, 1e-5), (cg.MIXED | cg.DETERMINISTIC, 1e-5)):
        K, F = asm.assemble(c.x, cg.TANGENT | cg.HINGE | fl)
        assert rel(F, Fo) < 1e-12, fl
        assert rel(K, Ko) < tolK, fl
    K1, F1 = asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC)
    K2, F2 = asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC)
    assert np.array_equal(K1, K2) and np.array_equal(F1, F2)
    # The tensor-core tangent's general (B != 0) records: the same bars (Frobenius 3e-6).
    asm.set_tuning(0, 0, 0, cg.TANGENT_TENSOR)
    assert asm.tensor_stats()["tensor_groups"] > 0
    for fl in (cg.MIXED, cg.MIXED | cg.DETERMINISTIC):
        K, F = asm.assemble(c.x, cg.TANGENT | cg.HINGE | fl)
        assert rel(F, Fo) < 1e-12, fl
        assert rel(K, Ko) < 1e-5 and np.linalg.norm(K - Ko) / np.linalg.norm(Ko) < 3e-6, fl


def test_assembler_stats(arc_case):
    c = arc_case
    n = np.diff(c.ref["ptr"])
    st = c.asm.stats()
    assert st["pairs"] == int((n * (n + 1) // 2).sum())
    assert st["blocks"] == c.asm.nnz // 9
    assert 0 < st["entries"] < st["pairs"] and st["direct_groups"] == 0


def test_mixed_wide_supports(o, ctx):
    """About 60 neighbours per point: a group of 16 points has more pairs than the merge
    setup sorts, so the FP32 tangent scatters those groups pair by pair and the
    deterministic mode keeps one unit per pair."""
    p = synth.square_plate(17, 0.5, 3, jitter=0.05, seed=31, crease="arc", rho_factor=4.5)
    x = 0.3 * synth.fourier_field(p.node_xy, np.random.default_rng(32), lam=(3.0, 10.0))
    c = Case(o, ctx, p, x)
    assert int(np.diff(c.ref["ptr"]).max()) >= 45
    assert c.asm.stats()["direct_groups"] > 0
    Ko, Fo = c.oracle(c.x)
    for det in (0, cg.DETERMINISTIC):
        K, F = c.asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.MIXED | det)
        assert rel(F, Fo) < 1e-12
        assert rel(K, Ko) < 1e-5
    K1, F1 = c.asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC)
    K2, F2 = c.asm.assemble(c.x, cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC)
    assert np.array_equal(K1, K2) and np.array_equal(F1, F2)


def test_tangent_check_on_gpu(arc_case):
    """main.cpp:651-710 on the GPU's own residual and tangent."""
    import scipy.sparse as sp

    c = arc_case
    n = 3 * c.p.n_nodes
    for mixed, bound in ((False, 1e-6), (True, 1e-5)):
        fl = cg.TANGENT | cg.HINGE | cg.HINGE_EXACT | (cg.MIXED if mixed else 0)
        K, _ = c.asm.assemble(c.x, fl)
        Kd = sp.csc_matrix((K, c.inner, c.outer), shape=(n, n)).toarray()
        U = np.triu(Kd)
        Ks = U + U.T - np.diag(np.diag(Kd))
        rng = np.random.default_rng(12345)
        h = 1e-6 * max(1.0, abs(c.x).max())
        worst = 0.0
        for _ in range(3):
            v = rng.uniform(-1, 1, n)
            v /= np.linalg.norm(v)
            _, Fp = c.asm.assemble(c.x + h * v, cg.HINGE)
            _, Fm = c.asm.assemble(c.x - h * v, cg.HINGE)
            fd = (Fp - Fm) / (2 * h)
            worst = max(worst, np.linalg.norm(fd - Ks @ v) / np.linalg.norm(fd))
        assert worst < bound, (mixed, worst)


def test_energies(arc_case):
    c = arc_case
    r = c.ref
    em, eb = c.o.strain_energies(c.p.faces.weight, r["ptr"], r["idx"], r["dpsi"], r["ddpsi"], c.x, c.A, c.B, c.D)
    eh = c.o.hinge_energy(c.x, c.folds)
    g = c.asm.energies(c.x)
    assert abs(g[0] - em) <= 1e-12 * abs(em)
    assert abs(g[1] - eb) <= 1e-12 * abs(eb)
    assert abs(g[2] - eh) <= 1e-12 * abs(eh)


def test_inactive_crease_points_and_rest_angles(o, ctx):
    p = synth.square_plate(17, 0.5, 3, seed=31, crease="row", Kt=5e-3, rho_factor=3.5)
    x = 0.2 * synth.fourier_field(p.node_xy, np.random.default_rng(3), lam=(3.0, 9.0))
    ctx.set_nodes(p.node_xy)
    model = cg.PlateModel(p, ctx)
    nf = len(p.folds[0].left.xy)
    rng = np.random.default_rng(4)
    active = (rng.uniform(size=nf) > 0.3).astype(np.int8)
    theta0 = rng.uniform(-0.2, 0.2, nf)
    spec = dict(model.fold_specs[0], active=active, theta0_gp=theta0)
    asm = cg.NonLinearAssembler(ctx, model.faces, p.faces.weight, [spec])
    asm.set_material(*cg.abd_isotropic(p.E, p.nu, p.thickness))
    K, F = asm.assemble(x, cg.TANGENT | cg.HINGE)
    Kd, Fd = asm.assemble(x, cg.TANGENT | cg.HINGE | cg.DETERMINISTIC)
    sh = model.faces.download()
    (L, R) = model.fold_sets[0]
    dl, dr = L.download(), R.download()
    folds = [{"left": {"ptr": dl["ptr"], "idx": dl["idx"], "dpsi": dl["dpsi"]},
              "right": {"ptr": dr["ptr"], "idx": dr["idx"], "dpsi": dr["dpsi"]},
              "weight": p.folds[0].left.weight, "tangent": p.folds[0].left.tangent, "Kt": 5e-3,
              "active": active, "theta0_gp": theta0}]
    outer, inner, col_ptr, col_nodes, mp = o.pattern(p.n_nodes, sh["ptr"], sh["idx"], folds)
    A, B, D = o.abd(p.E, p.nu, p.thickness)
    Ko, Fo = o.update_stiffness(p.n_nodes, p.faces.weight, sh["ptr"], sh["idx"], sh["dpsi"], sh["ddpsi"],
                                outer, mp, x, A, B, D)
    Ko, Fo = o.hinge(p.n_nodes, x, folds, outer, col_ptr, col_nodes, Ko, Fo)
    assert rel(K, Ko) < 1e-13 and rel(F, Fo) < 1e-13
    assert rel(Kd, Ko) < 1e-13 and rel(Fd, Fo) < 1e-13


def test_full_size_properties(ctx):
    """At the benchmark's full size (640,000 Gauss points): mixed vs FP64 residual within
    the metric's 1e-10, atomic vs deterministic agreement, residual-only consistency."""
    p = synth.config_assembly()
    x = synth.fourier_field(p.node_xy, np.random.default_rng(1004))
    ctx.set_nodes(p.node_xy)
    m = cg.PlateModel(p, ctx)
    assert m.faces.n_gp == 640000
    K64, F64 = m.asm.assemble(x, cg.TANGENT | cg.HINGE)
    Kmx, Fmx = m.asm.assemble(x, cg.TANGENT | cg.HINGE | cg.MIXED)
    Kd, Fd = m.asm.assemble(x, cg.TANGENT | cg.HINGE | cg.DETERMINISTIC)
    assert rel(Fmx, F64) <= 1e-10
    assert np.linalg.norm(Kmx - K64) / np.linalg.norm(K64) < 1e-6
    assert rel(Kd, K64) < 1e-12 and rel(Fd, F64) < 1e-12
    _, Fr = m.asm.assemble(x, cg.HINGE | cg.MIXED)
    assert rel(Fr, Fmx) < 1e-14
    # K's checksum is independent of the scatter order up to round-off
    assert abs(Kd.sum() - K64.sum()) <= 1e-10 * np.abs(K64).sum()


def test_assemble_into_page_locked_host_memory(ctx):
    """cgb_assemble into page-locked host buffers (as the end-to-end benchmark uses) gives
    what it gives into ordinary host memory: bitwise with the deterministic scatter, to the
    atomic scatter's run-to-run rounding otherwise."""
    import torch

    p = synth.square_plate(21, 0.5, 3, jitter=0.1, crease="arc", seed=8)
    model = cg.PlateModel(p, ctx)
    x = synth.fourier_field(p.node_xy, np.random.default_rng(9), lam=(4.0, 20.0))
    asm = model.asm
    for flags in (cg.TANGENT | cg.HINGE | cg.MIXED, cg.TANGENT | cg.HINGE, cg.TANGENT | cg.MIXED | cg.DETERMINISTIC):
        K_pl, F_pl = asm.assemble(x, flags)
        K_h = torch.empty(asm.nnz, dtype=torch.float64, pin_memory=True).numpy()
        F_h = torch.empty(asm.n_dofs, dtype=torch.float64, pin_memory=True).numpy()
        x_h = torch.empty(asm.n_dofs, dtype=torch.float64, pin_memory=True).numpy()
        x_h[:] = x
        asm.assemble(x_h, flags, K_out=K_h, F_out=F_h)
        if flags & cg.DETERMINISTIC:
            assert np.array_equal(K_h, K_pl) and np.array_equal(F_h, F_pl)
        else:   # atomic scatter: the order of the additions may differ between calls
            k_tol = 1e-6 if flags & cg.MIXED else 1e-12      # FP32 / FP64 accumulation
            assert np.abs(K_h - K_pl).max() <= k_tol * np.abs(K_pl).max()
            assert np.abs(F_h - F_pl).max() <= 1e-12 * np.abs(F_pl).max()


def test_large_K_host_and_device_entry_points_agree():
    """A K of more than 64 MB: the deterministic K through cgb_assemble (page-locked and
    ordinary host buffers) equals, bitwise, K assembled by cgb_assemble_device on a caller's
    stream and copied by torch."""
    import torch

    p = synth.square_plate(141, 0.5, 2, jitter=0.1, crease="arc", seed=12)
    ctx = cg.Context(0)              # its own context: the test moves it onto a torch stream
    model = cg.PlateModel(p, ctx)
    asm = model.asm
    assert asm.nnz * 8 >= 64 << 20
    x = synth.fourier_field(p.node_xy, np.random.default_rng(13), lam=(4.0, 40.0))
    flags = cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC
    K_h = torch.empty(asm.nnz, dtype=torch.float64, pin_memory=True).numpy()
    F_h = torch.empty(asm.n_dofs, dtype=torch.float64, pin_memory=True).numpy()
    asm.assemble(x, flags, K_out=K_h, F_out=F_h)
    K_pg, F_pg = asm.assemble(x, flags)                      # ordinary host memory
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    x_d = torch.from_numpy(x).cuda()
    K_d = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
    F_d = torch.empty(asm.n_dofs, dtype=torch.float64, device="cuda")
    asm.assemble_device(x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), flags)
    ctx.synchronize()
    K_dev = K_d.cpu().numpy()
    assert np.array_equal(K_h, K_dev) and np.array_equal(K_pg, K_dev)
    assert np.array_equal(F_h, F_d.cpu().numpy())
