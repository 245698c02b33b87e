"""Failure detection on the GPU without a fault: a staging wait of the FP32-class tangent
that never completes gives up after its bounded time, the kernel returns, the host reads the
device error word as CGB_ERR_DEVICE, and the context stays usable."""
import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["tensor", "cores"])
def test_stage_wait_gives_up_and_is_reported(kind):
    """Both FP32-class tangents (the tensor-core one and the CUDA-core one) stage their
    cells' neighbour data the same way; either gives up, reports and leaves the context
    usable."""
    import __graft_entry__ as ge

    ge.build()
    ctx = cg.Context(0)
    p = synth.square_plate(15, 0.5, 4, jitter=0.05, seed=61, crease="arc", Kt=1e-3)   # 4x4 rule: cells of 16 points
    x = 0.2 * synth.fourier_field(p.node_xy, np.random.default_rng(62), lam=(3.0, 10.0))
    m = cg.PlateModel(p, ctx)
    m.asm.set_tuning(0, 0, 0, cg.TANGENT_TENSOR if kind == "tensor" else cg.TANGENT_CORES)
    if kind == "tensor":
        assert m.asm.tensor_stats()["tensor_groups"] > 0
    fl = cg.TANGENT | cg.HINGE | cg.MIXED
    K0, F0 = m.asm.assemble(x, fl)
    ctx.check(ctx.lib.cgb_test_stage_timeout(m.asm.h, 1))
    with pytest.raises(cg.CGBError) as e:
        m.asm.assemble(x, fl)
    assert e.value.code == 7 and "did not complete" in str(e.value)
    ctx.check(ctx.lib.cgb_test_stage_timeout(m.asm.h, 0))
    K1, F1 = m.asm.assemble(x, fl)          # the context and the assembler still work
    assert np.abs(K1 - K0).max() <= 1e-6 * np.abs(K0).max()
    assert np.abs(F1 - F0).max() <= 1e-13 * np.abs(F0).max()
