"""The single-plate assembly workload (201x201 jittered nodes, 4x4 rule, arc crease of
radius 0.6 x side, elastic hinge Kt = 1e-3, quadratic RKPM at rho = 3h, 8-mode Fourier
displacement with rotations up to 60 deg) generated at 61x61 nodes (57,600 Gauss points),
assembled on the GPU and by the oracle (NonLinearAssembler::updateStiffness +
Constraints::evaluateElasticFold restated, plate/Assembly.h:158-345,
plate/Constraints.h:341-436) at the same x.

Two comparisons, both against the oracle's K and F on the oracle's own pattern (bit-exact
with the GPU's):
- stage B on identical inputs: the GPU assembly fed the oracle's shape functions (faces
  and both crease sides). The residual bar of the mixed assembly is the metric's 1e-10
  (measured ~1e-15: the residual is FP64); the FP64 assembly 1e-12; the FP32 tangent 1e-5
  (max) / 1e-6 (Frobenius).
- end to end: the GPU's own shape functions, then its assembly. Near the crease the moment
  matrices of truncated supports are ill-conditioned, so two FP64 implementations of
  stage A differ there by about cond(M) eps; the bar is 1e-8 on F and K.
"""
import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import synth
from oracle import Oracle

pytestmark = pytest.mark.gpu


def rel_inf(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def rel_fro(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case():
    import __graft_entry__ as ge

    ge.build()
    ctx = cg.Context(0)
    p = synth.config_assembly(rule=4, n_side=61)
    x = synth.fourier_field(p.node_xy, np.random.default_rng(1004))
    o = Oracle()
    ptr, idx, s = o.frnn(p.node_xy, p.faces.xy, p.rho)
    psi, dpsi, ddpsi, bad, rc = o.rkpm(p.node_xy, p.faces.xy, ptr, idx, s, p.rho, p.order, p.creases)
    assert rc == 0
    folds = []
    for f in p.folds:
        side = {}
        for nm, ps in (("left", f.left), ("right", f.right)):
            fp, fi, fs = o.frnn(p.node_xy, ps.xy, p.rho)
            _, fd, _, _, rcf = o.rkpm(p.node_xy, ps.xy, fp, fi, fs, p.rho, p.order, p.creases)
            assert rcf == 0
            side[nm] = {"ptr": fp, "idx": fi, "dpsi": fd}
        folds.append({"left": side["left"], "right": side["right"], "weight": f.left.weight,
                      "tangent": f.left.tangent, "Kt": f.Kt, "theta0": f.theta0})
    outer, inner, col_ptr, col_nodes, mp = o.pattern(p.n_nodes, ptr, idx, folds)
    A, B, D = o.abd(p.E, p.nu, p.thickness)
    Ko, Fo = o.update_stiffness(p.n_nodes, p.faces.weight, ptr, idx, dpsi, ddpsi, outer, mp, x, A, B, D)
    Ko, Fo = o.hinge(p.n_nodes, x, folds, outer, col_ptr, col_nodes, Ko, Fo)
    ctx.set_nodes(p.node_xy)
    model = cg.PlateModel(p, ctx)
    # The oracle's shape functions on the GPU, for stage B on identical inputs.
    faces_o = cg.shape_from_host(ctx, ptr, idx, dpsi, ddpsi, psi)
    gfolds = []
    for f in folds:
        sides = {nm: cg.shape_from_host(ctx, f[nm]["ptr"], f[nm]["idx"], f[nm]["dpsi"],
                                        np.zeros((len(f[nm]["idx"]), 3))) for nm in ("left", "right")}
        gfolds.append(dict(f, left=sides["left"], right=sides["right"]))
    asm_o = cg.NonLinearAssembler(ctx, faces_o, p.faces.weight, gfolds)
    asm_o.set_material(*cg.abd_isotropic(p.E, p.nu, p.thickness))
    return dict(p=p, x=x, outer=outer, inner=inner, Ko=Ko, Fo=Fo, model=model, asm_o=asm_o,
                keep=(faces_o, gfolds))


def test_patterns_bit_exact(case):
    for asm in (case["asm_o"], case["model"].asm):
        outer, inner = asm.pattern()
        assert np.array_equal(outer, case["outer"]) and np.array_equal(inner, case["inner"])


@pytest.mark.parametrize("det", [False, True])
def test_stage_b_on_oracle_shape_functions(case, det):
    x, Ko, Fo = case["x"], case["Ko"], case["Fo"]
    d = cg.DETERMINISTIC if det else 0
    K, F = case["asm_o"].assemble(x, cg.TANGENT | cg.HINGE | d)
    print(f"fp64 det={det}: F {rel_inf(F, Fo):.2e} K {rel_inf(K, Ko):.2e}")
    assert rel_inf(F, Fo) <= 1e-12 and rel_inf(K, Ko) <= 1e-12
    K, F = case["asm_o"].assemble(x, cg.TANGENT | cg.HINGE | cg.MIXED | d)
    print(f"mixed det={det}: F {rel_inf(F, Fo):.2e} K max {rel_inf(K, Ko):.2e} fro {rel_fro(K, Ko):.2e}")
    assert rel_inf(F, Fo) <= 1e-10     # the metric's residual bar
    # FP32-class tangent: the default FP32 CUDA-core tangent to 1e-6 in the Frobenius norm
    # (the 3xTF32 tensor-core one, tests/test_tensor_tangent.py, to 3e-6)
    assert rel_inf(K, Ko) <= 1e-5 and rel_fro(K, Ko) <= 1e-6


def test_end_to_end_on_gpu_shape_functions(case):
    x, Ko, Fo = case["x"], case["Ko"], case["Fo"]
    asm = case["model"].asm
    for name, fl in (("fp64", cg.TANGENT | cg.HINGE), ("mixed", cg.TANGENT | cg.HINGE | cg.MIXED)):
        K, F = asm.assemble(x, fl)
        print(f"{name} end to end: F {rel_inf(F, Fo):.2e} K max {rel_inf(K, Ko):.2e} fro {rel_fro(K, Ko):.2e}")
        assert rel_inf(F, Fo) <= 1e-8
        assert rel_inf(K, Ko) <= (1e-8 if name == "fp64" else 1e-5)
