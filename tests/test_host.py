"""Host-side logic without a GPU: the synthetic workload generators, the crease split and
the autotuner's search and cache."""
import math
import time

import numpy as np
import pytest

from curvami_gb300 import autotune as at
from curvami_gb300 import synth


def test_batched_workload_shapes():
    plates, xs = synth.config_batched(6, side_range=(21, 41), seed=3)
    assert len(plates) == 6 and len(xs) == 6
    for p, x in zip(plates, xs):
        n = p.meta["n_side"]
        assert 21 <= n <= 41 and len(p.node_xy) == n * n and x.shape == (3 * n * n,)
        assert 1 <= len(p.creases) == len(p.folds) <= 3
        assert all(1e-4 <= f.Kt <= 1e-1 for f in p.folds)
        h = p.meta["h"]
        V = [np.asarray(c["vertices"]) for c in p.creases]
        if np.allclose(V[0][:, 0], V[0][0, 0]):        # straight, parallel to y
            xs0 = sorted(v[0, 0] for v in V)
            assert all(b - a >= 6 * h - 1e-12 for a, b in zip(xs0, xs0[1:]))
            assert all(abs((x0 / h) % 1.0 - 0.5) < 1e-9 for x0 in xs0)   # half-way between columns
        else:                                          # concentric arcs
            R = sorted(float(np.hypot(*v[len(v) // 2])) for v in V)
            assert all(b - a >= 6 * h - 1e-9 for a, b in zip(R, R[1:]))


def test_crease_split_matches_brute_force():
    nodes = synth.grid_nodes(21, 21, 0.5, 0.0, np.random.default_rng(0))
    faces = synth.quad_gauss_points(nodes, 21, 21, 3)
    hull = synth.convex_hull(synth._hull_candidates(nodes))
    cr = [synth.make_crease(np.array([[2.75, 0.0], [2.75, 10.0]]), nodes, hull),
          synth.make_crease(np.array([[0.0, 5.25], [4.0, 5.25], [10.0, 5.25]]), nodes, hull)]
    out, n_split = synth.split_on_creases(faces, cr)
    # brute force: distance of every point to every segment (SetupHelper.h:60-106)
    xy = faces.xy
    best = np.full(len(xy), np.inf)
    for c in cr:
        V = np.asarray(c["vertices"])
        for A, B in zip(V[:-1], V[1:]):
            v = B - A
            t = np.clip(((xy - A) @ v) / (v @ v), 0, 1)
            best = np.minimum(best, np.linalg.norm(xy - (A + t[:, None] * v), axis=1))
    hits = np.nonzero(best < 1e-9)[0]
    assert n_split == len(hits) > 0
    assert len(out.xy) == len(xy) + len(hits)
    assert math.isclose(out.weight.sum(), faces.weight.sum(), rel_tol=1e-14)


class _FakeAsm:
    """Stands in for NonLinearAssembler: each launch shape has a fixed cost."""

    class _Ctx:
        def synchronize(self):
            pass

    class _Faces:
        n_gp = 123456

    def __init__(self):
        self.ctx = self._Ctx()
        self.faces = self._Faces()
        self.tuning = None
        self.calls = 0

    def stats(self):
        return {"pairs": 50_000_000, "blocks": 400_000, "entries": 5_000_000, "direct_groups": 0}

    def set_tuning(self, c, r, t, k=0):
        self.tuning = (c, r, t, k)

    def assemble_device(self, *a):
        self.calls += 1
        c, r, t, k = self.tuning
        time.sleep(0.001 * (abs(c - 2) + (r == 128) + t + k))   # best: (2, 256, 0, 0)


def test_autotune_search_and_cache(tmp_path):
    asm = _FakeAsm()
    cache = str(tmp_path / "t.json")
    r = at.autotune(asm, 1, 2, 3, flags=7, device_name="fake", cache_path=cache, repeats=2)
    assert tuple(r["tuning"]) == (2, 256, 0, 0) and asm.tuning == (2, 256, 0, 0) and not r["cached"]
    assert len(r["tried"]) == 20 and at.spread(r) > 1.0
    calls = asm.calls
    r2 = at.autotune(asm, 1, 2, 3, flags=7, device_name="fake", cache_path=cache)
    assert r2["cached"] and tuple(r2["tuning"]) == (2, 256, 0, 0) and asm.calls == calls
    # another flag set is another key
    r3 = at.autotune(asm, 1, 2, 3, flags=3, device_name="fake", cache_path=cache, repeats=1,
                     candidates={"n_chunks": (1, 2), "residual_threads": (256,), "tangent_ctas_per_sm": (0,)})
    assert not r3["cached"] and tuple(r3["tuning"]) == (2, 256, 0, 0)


def test_four_crease_plate_layout():
    """Four creases from the centre node to the boundary, sectors 90 +/- 15 deg summing to 360,
    creases 0 and 2 rigid, an end cap at the centre and an extension at the boundary."""
    import math
    from curvami_gb300 import synth

    p = synth.four_crease_plate(41, rule=2, seed=1005)
    assert len(p.creases) == 4 and len(p.folds) == 4
    sec = p.meta["sector_deg"]
    assert abs(sum(sec) - 360.0) < 1e-9 and all(60.0 <= a <= 150.0 for a in sec[:3])
    c = p.node_xy[(41 // 2) * 41 + 41 // 2]
    for cr in p.creases:
        assert np.allclose(cr["vertices"][0], c) and not cr["extend_start"] and cr["extend_end"]
    assert [f.rigid for f in p.folds] == [True, False, True, False]
    assert len(p.faces.xy) == 40 * 40 * 4


def test_tracking_displacement():
    """trackingDisplacement: mean displacement along the load over loaded domains, else the
    mean deflection of the nodes (plate/PlateProblem.h:14-44)."""
    import scipy.sparse as sp

    from curvami_gb300 import solver as S

    n = 4
    x = np.arange(3 * n, dtype=np.float64)

    class Tab:
        def __init__(self, P):
            self.P = sp.csr_matrix(P)
            self.n_gp = P.shape[0]

    class Prob:
        points, edges = [], []

    prob = Prob()
    assert S.tracking_displacement(prob, x) == pytest.approx(np.mean(x[2::3]))
    dom = S.LineDomain(np.zeros((2, 2)), np.ones(2), np.zeros((2, 2)), np.zeros((2, 2)),
                       S.BoundaryCondition(force=(0.0, 0.0, -2.0)))
    P = np.array([[0.5, 0.5, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0]])
    prob.edges = [(dom, Tab(P))]
    w = P @ x.reshape(-1, 3)[:, 2]
    assert S.tracking_displacement(prob, x) == pytest.approx(-w.mean())
