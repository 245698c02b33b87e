"""The allocation-free entry point cgb_assemble_face_noalloc, through the C ABI.

It exists for callers that cannot allocate GPU memory while they assemble (cudaMalloc
may synchronise the device, is not allowed during stream capture, or is reserved to a
host framework's own pool): they hold every input in their own device memory and the
library keeps its one scratch array (the FP32 block accumulator) in a fixed,
file-scope device array. The test allocates the caller's arrays itself (torch), then
checks two calls in a row against the allocating entry point (cgb_assemble_device with
CGB_TANGENT | CGB_MIXED): the residual to 1e-13 and the FP32 tangent to 1e-5 of its
scale (two FP32 atomic summation orders), the bars the mixed path meets elsewhere. It
then checks the refusals (bad sizes on the host; neighbour counts above max_neighbours
on the device, reported at the next synchronisation without a fault) and that a call
without face points reads no input and returns zero K and F. Collected last, so a
failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_path():
    torch = pytest.importorskip("torch")
    import __graft_entry__ as ge

    ge.build()
    ctx = cg.Context(0)
    p = synth.config_smallplate(rule=4)  # 41x41 nodes, 25,600 Gauss points
    ctx.set_nodes(p.node_xy)
    faces = cg.shape_functions(ctx, p.faces.xy, p.rho, p.order, p.creases, p.rho_node, p.kernel)
    asm = cg.NonLinearAssembler(ctx, faces, p.faces.weight)
    A, B, D = cg.abd_isotropic(p.E, p.nu, p.thickness)
    asm.set_material(A, B, D)
    assert asm.nnz // 9 <= _lib.NOALLOC_MAX_BLOCKS

    # The caller's own device copies of the inputs, in the reference's formats.
    sh = faces.download()
    outer, _ = asm.pattern()
    csr_map = asm.csr_mapping()
    n = np.diff(sh["ptr"])
    map_ptr = np.concatenate([[0], np.cumsum(n * (n + 1) // 2)]).astype(np.int64)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    d = {"nbr_ptr": dev(sh["ptr"]), "nbr_idx": dev(sh["idx"]), "dpsi": dev(sh["dpsi"]),
         "ddpsi": dev(sh["ddpsi"]), "weight": dev(p.faces.weight), "map_ptr": dev(map_ptr),
         "csr_map": dev(csr_map), "outer": dev(outer)}
    prob = _lib.FaceProblem()
    prob.n_gp = faces.n_gp
    prob.n_nodes = p.n_nodes
    prob.max_neighbours = faces.max_n
    prob.nnz = asm.nnz
    for k, t in d.items():
        setattr(prob, k, t.data_ptr())
    for name, M in (("A", A), ("B", B), ("D", D)):
        getattr(prob, name)[:] = [float(v) for v in np.asarray(M).ravel()]

    rng = np.random.default_rng(8)
    for call in range(2):
        x = 0.2 * synth.fourier_field(p.node_xy, rng, lam=(5.0, 20.0))
        x_d = dev(x)
        K_ref = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
        F_ref = torch.empty(3 * p.n_nodes, dtype=torch.float64, device="cuda")
        asm.assemble_device(x_d.data_ptr(), K_ref.data_ptr(), F_ref.data_ptr(), cg.TANGENT | cg.MIXED)
        ctx.synchronize()
        K = torch.full((asm.nnz,), np.nan, dtype=torch.float64, device="cuda")
        F = torch.full((3 * p.n_nodes,), np.nan, dtype=torch.float64, device="cuda")
        rc = ctx.lib.cgb_assemble_face_noalloc(ctx.h, C.byref(prob), C.c_void_p(x_d.data_ptr()),
                                               C.c_void_p(K.data_ptr()), C.c_void_p(F.data_ptr()))
        assert rc == 0, ctx.lib.cgb_last_error(ctx.h)
        ctx.synchronize()
        K, F, K_ref, F_ref = (t.cpu().numpy() for t in (K, F, K_ref, F_ref))
        assert np.isfinite(K).all() and np.isfinite(F).all()
        assert np.abs(F - F_ref).max() <= 1e-13 * np.abs(F_ref).max(), call
        assert np.abs(K - K_ref).max() <= 1e-5 * np.abs(K_ref).max(), call

    # Sizes beyond the fixed accumulator are refused with a clear error.
    nnz = prob.nnz
    prob.nnz = 9 * (_lib.NOALLOC_MAX_BLOCKS + 1)
    rc = ctx.lib.cgb_assemble_face_noalloc(ctx.h, C.byref(prob), C.c_void_p(x_d.data_ptr()),
                                           C.c_void_p(1), C.c_void_p(1))
    assert rc == _lib.CGB_ERR_CAPACITY
    assert b"exceeds the fixed accumulator" in ctx.lib.cgb_last_error(ctx.h)
    prob.nnz = nnz

    def call(pr, K, F):
        return ctx.lib.cgb_assemble_face_noalloc(ctx.h, C.byref(pr), C.c_void_p(x_d.data_ptr()),
                                                 C.c_void_p(K.data_ptr()), C.c_void_p(F.data_ptr()))

    K = torch.full((asm.nnz,), np.nan, dtype=torch.float64, device="cuda")
    F = torch.full((3 * p.n_nodes,), np.nan, dtype=torch.float64, device="cuda")
    # Refusals on the host: nothing is launched.
    for field, bad in (("n_nodes", 0), ("n_gp", -1), ("nnz", -9), ("nnz", nnz + 1), ("max_neighbours", -1)):
        good = getattr(prob, field)
        setattr(prob, field, bad)
        assert call(prob, K, F) == _lib.CGB_ERR_INVALID, field
        setattr(prob, field, good)
    prob.max_neighbours = 100000
    assert call(prob, K, F) == _lib.CGB_ERR_CAPACITY
    assert b"too many neighbours" in ctx.lib.cgb_last_error(ctx.h)
    prob.max_neighbours = faces.max_n
    outer_ptr = prob.outer
    prob.outer = None
    assert call(prob, K, F) == _lib.CGB_ERR_INVALID
    assert b"NULL input array" in ctx.lib.cgb_last_error(ctx.h)
    ctx.synchronize()

    # No face point: no input array is read (all NULL here) and K and F come back zero.
    empty = _lib.FaceProblem()
    empty.n_gp = 0
    empty.n_nodes = p.n_nodes
    empty.max_neighbours = 0
    empty.nnz = asm.nnz
    assert call(empty, K, F) == 0, ctx.lib.cgb_last_error(ctx.h)
    ctx.synchronize()
    assert not K.cpu().numpy().any() and not F.cpu().numpy().any()
    prob.outer = outer_ptr

    # A max_neighbours below the true largest count: the points that do not fit the
    # staging are skipped on the device and the next synchronisation reports it.
    prob.max_neighbours = faces.max_n - 1
    assert call(prob, K, F) == 0, ctx.lib.cgb_last_error(ctx.h)
    with pytest.raises(cg.CGBError) as ei:
        ctx.synchronize()
    assert ei.value.code == _lib.CGB_ERR_DEVICE and "out of range" in str(ei.value)
    # The context stays usable: the correct sizes give the allocating path's result again.
    prob.max_neighbours = faces.max_n
    assert call(prob, K, F) == 0
    ctx.synchronize()
    assert np.abs(F.cpu().numpy() - F_ref).max() <= 1e-13 * np.abs(F_ref).max()
