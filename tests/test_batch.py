"""Batched plates (one assembler over several independent plates), CUDA-graph replay of an
assembly, and the launch-shape tuning knobs, through the C ABI on the GPU."""
import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as ge

    ge.build()
    return cg.Context(0)


def plates():
    return [synth.square_plate(13, 0.5, 3, jitter=0.05, seed=41, crease="row", Kt=1e-3, rho_factor=3.5),
            synth.square_plate(19, 0.5, 4, jitter=0.08, seed=42, crease="arc", Kt=1e-2),
            synth.square_plate(9, 0.5, 2, jitter=0.0, seed=43, crease=None)]


def fields(ps, seed=7):
    rng = np.random.default_rng(seed)
    return [0.2 * synth.fourier_field(p.node_xy, rng, lam=(3.0, 10.0)) for p in ps]


def test_batch_equals_plates_one_by_one(ctx):
    ps = plates()
    xs = fields(ps)
    batch = cg.PlateBatch(ps, ctx)
    x = np.concatenate(xs)
    for fl in (cg.DETERMINISTIC, 0, cg.MIXED):
        Kb, Fb = batch.asm.assemble(x, cg.TANGENT | cg.HINGE | fl)
        for k, (p, xk) in enumerate(zip(ps, xs)):
            m = cg.PlateModel(p, ctx)
            K, F = m.asm.assemble(xk, cg.TANGENT | cg.HINGE | fl)
            o_b, _ = batch.asm.pattern()
            o_k, i_k = m.asm.pattern()
            assert np.array_equal(np.diff(o_b[batch.dofs(k).start: batch.dofs(k).stop + 1]), np.diff(o_k))
            Ks, Fs = Kb[batch.k_values(k)], Fb[batch.dofs(k)]
            if fl == cg.DETERMINISTIC:
                # the same ordered sums, shifted ids: bitwise
                assert np.array_equal(Ks, K) and np.array_equal(Fs, F)
            else:
                tol = 1e-6 if fl == cg.MIXED else 1e-13
                assert np.abs(Ks - K).max() <= tol * np.abs(K).max()
                assert np.abs(Fs - F).max() <= 1e-13 * np.abs(F).max()


def test_graph_replay_matches_direct_call(ctx):
    import torch

    ps = plates()
    batch = cg.PlateBatch(ps, ctx)
    x = np.concatenate(fields(ps))
    asm = batch.asm
    dev = torch.device("cuda")
    d_x = torch.from_numpy(x).to(dev)
    d_K = torch.empty(asm.nnz, dtype=torch.float64, device=dev)
    d_F = torch.empty(asm.n_dofs, dtype=torch.float64, device=dev)
    fl = cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC
    K0, F0 = asm.assemble(x, fl)
    g = asm.graph(d_x.data_ptr(), d_K.data_ptr(), d_F.data_ptr(), fl)
    d_K.zero_(); d_F.zero_()
    torch.cuda.synchronize()
    g.launch()
    ctx.synchronize()
    assert np.array_equal(d_K.cpu().numpy(), K0) and np.array_equal(d_F.cpu().numpy(), F0)
    # the graph reads x at replay time
    x2 = np.concatenate(fields(ps, seed=8))
    d_x.copy_(torch.from_numpy(x2).to(dev))
    torch.cuda.synchronize()
    g.launch()
    ctx.synchronize()
    K2, F2 = asm.assemble(x2, fl)
    assert np.array_equal(d_K.cpu().numpy(), K2) and np.array_equal(d_F.cpu().numpy(), F2)
    # an assembler with a live graph refuses destruction
    assert ctx.lib.cgb_assembler_destroy(asm.h) == 1
    g.close()


def test_tuning_changes_launch_shape_not_results(ctx):
    ps = plates()
    batch = cg.PlateBatch(ps, ctx)
    x = np.concatenate(fields(ps))
    fl = cg.TANGENT | cg.HINGE | cg.DETERMINISTIC
    K0, F0 = batch.asm.assemble(x, fl)
    for t in [(1, 64, 1), (3, 128, 2), (8, 256, 3), (3, 128, 0, cg.TANGENT_CORES)]:
        batch.asm.set_tuning(*t)
        K, F = batch.asm.assemble(x, fl)
        assert np.array_equal(K, K0) and np.array_equal(F, F0)
        Km, Fm = batch.asm.assemble(x, fl | cg.MIXED)
        assert np.abs(Km - K0).max() <= 1e-6 * np.abs(K0).max()
    with pytest.raises(cg.CGBError):
        batch.asm.set_tuning(17, 0, 0)
    with pytest.raises(cg.CGBError):
        batch.asm.set_tuning(0, 96, 0)
    with pytest.raises(cg.CGBError):
        batch.asm.set_tuning(0, 0, 0, 7)


def test_autotune_picks_and_caches(ctx, tmp_path):
    import torch

    from curvami_gb300 import autotune as at

    ps = plates()
    batch = cg.PlateBatch(ps, ctx)
    asm = batch.asm
    dev = torch.device("cuda")
    d_x = torch.from_numpy(np.concatenate(fields(ps))).to(dev)
    d_K = torch.empty(asm.nnz, dtype=torch.float64, device=dev)
    d_F = torch.empty(asm.n_dofs, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    fl = cg.TANGENT | cg.HINGE | cg.MIXED
    cache = str(tmp_path / "tune.json")
    cand = {"n_chunks": (1, 2), "residual_threads": (128, 256), "tangent_ctas_per_sm": (0,)}
    r1 = at.autotune(asm, d_x.data_ptr(), d_K.data_ptr(), d_F.data_ptr(), fl, candidates=cand,
                     cache_path=cache, repeats=2)
    assert not r1["cached"] and len(r1["tried"]) == 4
    assert tuple(r1["tuning"]) in [(c, r, 0, 0) for c in (1, 2) for r in (128, 256)]
    assert asm.tuning == tuple(r1["tuning"])
    r2 = at.autotune(asm, d_x.data_ptr(), d_K.data_ptr(), d_F.data_ptr(), fl, candidates=cand,
                     cache_path=cache, repeats=2)
    assert r2["cached"] and tuple(r2["tuning"]) == tuple(r1["tuning"])
