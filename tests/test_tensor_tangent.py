"""The tensor-core tangent (tcgen05, 3xTF32 with FP32 accumulation in tensor memory) against
the oracle and against the CUDA-core FP32 tangent, through the C ABI on the GPU.

Each cell of 16 Gauss points whose neighbour union has at most 42 nodes is formed as one
128-row tensor-core product; the others stay on the CUDA cores. Bars: K within 1e-5 (max)
and 3e-6 (Frobenius) of the oracle's (3xTF32 with the lo x lo products dropped and FP32
accumulation in the tensor core: measured 0.9e-6 - 1.3e-6, against 1e-7 for the FP32 CUDA
cores); the two tangents within 3e-6 of each other; F unchanged (the FP64 residual); the deterministic
scatter bitwise run to run; plates whose cells all leave the tensor path, and plates that
mix both, give the same K as the CUDA-core tangent.
"""
import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import synth
from oracle import Oracle

from test_gpu_parity import Case, rel

pytestmark = pytest.mark.gpu

MIX = cg.TANGENT | cg.HINGE | cg.MIXED


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as ge

    ge.build()
    return cg.Context(0)


@pytest.fixture(scope="module")
def o():
    return Oracle()


def fro(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("det", [False, True])
def test_tensor_tangent_against_oracle(ctx, o, det):
    p = synth.square_plate(25, 0.5, 4, jitter=0.1, seed=31, crease="arc", Kt=1e-3)
    x = 0.3 * synth.fourier_field(p.node_xy, np.random.default_rng(32), lam=(3.0, 12.0))
    c = Case(o, ctx, p, x)
    ts = c.asm.tensor_stats()
    assert ts["tensor_groups"] > 0
    Ko, Fo = c.oracle(x)
    fl = MIX | (cg.DETERMINISTIC if det else 0)
    c.asm.set_tuning(0, 0, 0, cg.TANGENT_TENSOR)
    K, F = c.asm.assemble(x, fl)
    print(f"tensor det={det}: K max {rel(K, Ko):.2e} fro {fro(K, Ko):.2e}, F {rel(F, Fo):.2e}, {ts}")
    assert rel(F, Fo) < 1e-12
    assert rel(K, Ko) < 1e-5 and fro(K, Ko) < 3e-6
    c.asm.set_tuning(0, 0, 0, cg.TANGENT_CORES)
    Kc, Fc = c.asm.assemble(x, fl)
    assert rel(K, Kc) < 1e-5 and fro(K, Kc) < 3e-6
    if det:
        c.asm.set_tuning(0, 0, 0, cg.TANGENT_TENSOR)
        K2, F2 = c.asm.assemble(x, fl)
        assert np.array_equal(K, K2) and np.array_equal(F, F2)


def test_tensor_and_core_cells_mixed_in_one_plate(ctx):
    """rho = 3.5h: most cells' node unions exceed 42 nodes and stay on the CUDA cores, the
    rest go to the tensor cores; the chunked launch splits both kinds per chunk."""
    p = synth.square_plate(61, 0.5, 4, jitter=0.1, seed=33, crease="arc", Kt=1e-3, rho_factor=3.5)
    x = 0.3 * synth.fourier_field(p.node_xy, np.random.default_rng(34), lam=(5.0, 30.0))
    m = cg.PlateModel(p, ctx)
    ts = m.asm.tensor_stats()
    print(ts)
    out = {}
    for kind in (cg.TANGENT_CORES, cg.TANGENT_TENSOR):
        for chunks in (1, 4):
            m.asm.set_tuning(chunks, 0, 0, kind)
            out[(kind, chunks)] = m.asm.assemble(x, MIX)
    Kc, Fc = out[(cg.TANGENT_CORES, 1)]
    for key, (K, F) in out.items():
        assert rel(K, Kc) < 1e-5 and fro(K, Kc) < 3e-6, key
        assert rel(F, Fc) < 1e-13, key


def test_full_size_tensor_tangent(ctx):
    """The benchmark workload (640,000 Gauss points): the tensor tangent against the FP64
    assembly of the same library (FP32 accuracy) and against the CUDA-core tangent."""
    p = synth.config_assembly()
    x = synth.fourier_field(p.node_xy, np.random.default_rng(1004))
    m = cg.PlateModel(p, ctx)
    ts = m.asm.tensor_stats()
    assert ts["tensor_groups"] > 0.95 * (ts["tensor_groups"] + ts["core_groups"])
    K64, F64 = m.asm.assemble(x, cg.TANGENT | cg.HINGE)
    m.asm.set_tuning(0, 0, 0, cg.TANGENT_TENSOR)
    Kt, Ft = m.asm.assemble(x, MIX)
    m.asm.set_tuning(0, 0, 0, cg.TANGENT_CORES)
    Kc, Fc = m.asm.assemble(x, MIX)
    print(f"tensor vs fp64: max {rel(Kt, K64):.2e} fro {fro(Kt, K64):.2e}; cores vs fp64: max {rel(Kc, K64):.2e} "
          f"fro {fro(Kc, K64):.2e}; {ts}")
    assert rel(Ft, F64) <= 1e-10
    assert fro(Kt, K64) < 3e-6 and rel(Kt, K64) < 1e-5
    assert fro(Kt, Kc) < 3e-6
