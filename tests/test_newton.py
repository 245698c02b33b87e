"""The host Newton driver (curvami_gb300/solver.py): LineSearch of the reference's
ContinuationSolver over a clamped plate with an elastic hinge and a face load.

CPU tests drive it over the oracle's assembly; the GPU test drives it over the library
(FP64 and mixed) and compares Newton iteration counts per load step and the converged
load-displacement path with the oracle run (bar: counts equal, states within 1e-6)."""
import json
import os
import time

import numpy as np
import pytest

from curvami_gb300 import solver as S
from curvami_gb300 import synth
from oracle import Oracle

from newton_helpers import clamped_left_edge, oracle_problem, small_plate

TOL = dict(tol_force=1e-16, tol_energy=1e-24)   # the plate's forces are O(1e-10)


@pytest.fixture(scope="module")
def o():
    return Oracle()


def test_fold_angle_gradient_matches_oracle(o):
    rng = np.random.default_rng(5)
    F = np.tile(np.array([1.0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 1, 0]), (16, 1)) + 0.3 * rng.standard_normal((16, 12))
    t = rng.standard_normal((16, 2))
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    th, g = S.fold_angle_and_grad(F, t[:, 0], t[:, 1])
    for k in range(16):
        tho, go = o.fold_angle(F[k], t[k, 0], t[k, 1])
        assert abs(th[k] - tho) < 1e-14
        assert np.abs(g[k] - go).max() < 1e-12 * max(1.0, np.abs(go).max())


def test_constraint_rows(o):
    p = small_plate(9)
    edge = clamped_left_edge(p)
    prob = oracle_problem(o, p, (0.0, 0.0, 1e-9), edge)
    x = 1e-3 * np.random.default_rng(1).standard_normal(prob.num_dofs())
    c, J = prob.constraints(x)
    n_edge, n_crease = len(edge.xy), len(p.folds[0].left.xy)
    assert J.shape == (4 * n_edge + 3 * n_crease, prob.num_dofs())
    # the constraints are linear in x for elastic hinges: c(x) = J x
    assert np.abs(J @ x - c).max() < 1e-15
    # rows of the first edge point: u, v, w, then the normal slope
    assert np.allclose(J[0].toarray()[0, 0::3], prob.edges[0][1].P[0].toarray()[0])


def test_rigid_folds_hold_their_angle(o):
    """flagRig: no hinge force, a fold-angle row per crease point (Constraints.h:280-304);
    the converged state keeps every crease point at its rest angle."""
    p = small_plate(9)
    prob = oracle_problem(o, p, (0.0, 0.0, 3e-10), clamped_left_edge(p))
    prob.flag_rig = True
    c0, J0 = prob.constraints(np.zeros(prob.num_dofs()))
    n_edge, n_crease = len(prob.edges[0][0].xy), len(p.folds[0].left.xy)
    assert J0.shape[0] == 4 * n_edge + 4 * n_crease      # u, v, w, slope; 3 ties + 1 angle
    states, iters = S.load_steps(S.ContinuationSolver(**TOL), prob, [0.5, 1.0])
    x = states[-1]
    c, J = prob.constraints(x)
    assert np.abs(c).max() < 1e-12
    # the rows are consistent: J is the derivative of c (central differences)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(prob.num_dofs()) * 1e-3
    cp, _ = prob.constraints(x + 1e-6 * v)
    cm, _ = prob.constraints(x - 1e-6 * v)
    assert np.abs((cp - cm) / 2e-6 - J @ v).max() < 1e-7 * max(1.0, np.abs(J @ v).max())
    assert np.abs(x[2::3]).max() > 0


def test_line_search_converges_and_is_linear_at_small_load(o):
    p = small_plate(9)
    edge = clamped_left_edge(p)
    prob = oracle_problem(o, p, (0.0, 0.0, 3e-11), edge)
    solver = S.ContinuationSolver(**TOL)
    states, iters = S.load_steps(solver, prob, [0.5, 1.0])
    x1, x2 = states
    c, _ = prob.constraints(x2)
    assert np.abs(c).max() < 1e-12
    w1, w2 = x1[2::3], x2[2::3]
    assert w2.max() > 0.0
    assert np.abs(w2 - 2.0 * w1).max() < 1e-3 * np.abs(w2).max()   # near-linear regime
    # the last iterations converge quadratically: the tangent matches the residual
    merits = [h[1] for h in solver.history]
    assert merits[-1] < 1e-4 * merits[-3]


class _RoundedTangent:
    """The oracle's assembly with K rounded to FP32 and perturbed by relative noise, standing
    in for a lower-precision tangent."""

    def __init__(self, backend, noise=3e-7):
        self.b, self.noise, self.rng = backend, noise, np.random.default_rng(0)

    def pattern(self):
        return self.b.pattern()

    def assemble(self, x, want_K, hinge=True):
        K, F = self.b.assemble(x, want_K, hinge)
        if K is not None:
            K = K.astype(np.float32).astype(np.float64) * (1.0 + self.noise * self.rng.standard_normal(K.shape))
        return K, F


def test_refined_steps_restore_the_fp64_newton_path(o):
    p = small_plate(13)
    prob = oracle_problem(o, p, (0.0, 0.0, 3e-9), clamped_left_edge(p))
    lams = [0.1, 0.2]
    ref_states, ref = S.load_steps(S.ContinuationSolver(**TOL), prob, lams)
    base = prob.backend
    prob.backend = _RoundedTangent(base)
    _, rough = S.load_steps(S.ContinuationSolver(**TOL), prob, lams)
    prob.backend = _RoundedTangent(base)
    states, refined = S.load_steps(S.ContinuationSolver(refine_steps=1, **TOL), prob, lams)
    assert rough != ref            # the perturbed tangent changes the line search's path ...
    assert refined == ref          # ... one refinement against the FP64 residual restores it
    assert max(np.abs(a - b).max() / np.abs(b).max() for a, b in zip(states, ref_states)) < 1e-8


def gpu_on_oracle_shapes(ctx, o, p, load, edge):
    """The oracle's PlateProblem (its shape functions for the faces, folds and edge) with the
    GPU assembly as the backend, fed the oracle's face and fold-side shape functions: the
    Newton driver over stage B alone on identical inputs."""
    import curvami_gb300 as cg

    prob = oracle_problem(o, p, load, edge)
    ob = prob.backend
    f = ob.f
    faces = cg.shape_from_host(ctx, f["ptr"], f["idx"], f["dpsi"], f["ddpsi"], f["psi"])
    folds = []
    for fd in ob.folds:
        sides = {nm: cg.shape_from_host(ctx, fd[nm]["ptr"], fd[nm]["idx"], fd[nm]["dpsi"], fd[nm]["ddpsi"])
                 for nm in ("left", "right")}
        folds.append(dict(fd, left=sides["left"], right=sides["right"]))
    asm = cg.NonLinearAssembler(ctx, faces, p.faces.weight, folds)
    asm.set_material(*cg.abd_isotropic(p.E, p.nu, p.thickness))
    prob.backend = S.GpuAssembly(asm)
    prob._keep = (faces, folds, asm)
    return prob


def compare_with_oracle(o, p, load, lambdas, kkt="host", all_arms=True):
    """Newton iterations per load step and the worst relative path difference of the GPU
    arms against the oracle arm, with where each arm's backtracking first differs from
    the oracle's (solver.first_divergence). Arms: the GPU's own shape functions with the
    FP64, mixed and mixed-refined assembly, and the FP64 GPU assembly on the oracle's
    shape functions (stage B alone)."""
    import __graft_entry__ as ge
    import curvami_gb300 as cg

    ge.build()
    edge = clamped_left_edge(p)
    t0 = time.perf_counter()
    ref_traces = []
    ref_states, ref_iters = S.load_steps(S.ContinuationSolver(kkt=kkt, **TOL), oracle_problem(o, p, load, edge),
                                         lambdas, traces=ref_traces)
    out = {"oracle": {"iters": ref_iters, "seconds": time.perf_counter() - t0}}
    ctx = cg.Context(0)
    model = cg.PlateModel(p, ctx)
    arms = [("gpu_fp64", False, 0, None), ("gpu_fp64_oracle_shapes", False, 0, "oracle"),
            ("gpu_mixed_refined", True, 1, None)]
    if all_arms:
        arms += [("gpu_mixed", True, 0, None), ("gpu_mixed_refined2", True, 2, None)]
    for name, mixed, refine, shapes in arms:
        # FP64 arms with the deterministic scatter: like the oracle's static schedule, every
        # run rounds the same way, so differences between the runs are reproducible.
        if shapes == "oracle":
            prob = gpu_on_oracle_shapes(ctx, o, p, load, edge)
            prob.backend = S.GpuAssembly(prob.backend.asm, deterministic=True)
        else:
            prob = S.gpu_problem(model, face_load=load, edges=[edge], mixed=mixed, deterministic=not mixed)
        t0 = time.perf_counter()
        traces = []
        states, iters = S.load_steps(S.ContinuationSolver(kkt=kkt, refine_steps=refine, **TOL), prob, lambdas,
                                     traces=traces)
        dev = max(float(np.abs(xs - xr).max() / np.abs(xr).max()) for xs, xr in zip(states, ref_states))
        out[name] = {"iters": iters, "seconds": time.perf_counter() - t0, "path_rel_diff": dev,
                     "assemblies": prob.n_assemble,
                     "residuals": prob.n_residual,
                     "first_divergence": S.first_divergence(ref_traces, traces, TOL["tol_force"], TOL["tol_energy"])}
    out["max_w"] = float(ref_states[-1][2::3].max())
    out["kkt"] = kkt
    return out


def check(out):
    ref = out["oracle"]["iters"]
    # FP64 on the GPU (its own shape functions, or the oracle's): the same Newton path as the
    # oracle's.
    assert out["gpu_fp64"]["iters"] == ref, out
    assert out["gpu_fp64_oracle_shapes"]["iters"] == ref, out
    # FP32 tangent with each Newton step refined once against the FP64 residual: the same
    # iteration counts. Without refinement the FP32 rounding of K (a few 1e-6 relative on
    # entries whose contributions cancel) perturbs the backtracking of the first,
    # pre-asymptotic iterations: a few more iterations, the same converged path.
    assert out["gpu_mixed_refined"]["iters"] == ref, out
    assert all(m >= r for m, r in zip(out["gpu_mixed"]["iters"], ref)), out
    assert sum(out["gpu_mixed"]["iters"]) <= 1.25 * sum(ref), out
    for arm in ("gpu_fp64", "gpu_mixed", "gpu_mixed_refined"):
        assert out[arm]["path_rel_diff"] <= 1e-6, out


@pytest.mark.gpu
def test_newton_counts_match_oracle(o):
    out = compare_with_oracle(o, small_plate(13), (0.0, 0.0, 3e-9), [0.1, 0.2, 0.3])
    print(json.dumps({k: (v["iters"] if isinstance(v, dict) else v) for k, v in out.items()}))
    check(out)


@pytest.mark.gpu
def test_newton_config_small_plate(o):
    """The plain FP64 method's small plate at full size: 41 x 41 nodes, 4 x 4 rule (25,600
    face Gauss points), cubic B-spline window, rho = 3.5h, crease on x = 10 with Kt = 1e-3,
    edge x = 0 clamped, a uniform face load ramped over 10 LineSearch steps (the first
    CGB_NEWTON_STEPS of them, 10 by default). The KKT solves are a dense FP64 LU on the GPU
    for every arm. CGB_NEWTON_REPORT=<json path> writes the comparison."""
    p = synth.square_plate(41, 0.5, 4, crease="row", Kt=1e-3, kernel=1, rho_factor=3.5, seed=1001)
    n_steps = int(os.environ.get("CGB_NEWTON_STEPS", "5"))
    out = compare_with_oracle(o, p, (0.0, 0.0, 3e-10), [0.1 * k for k in range(1, n_steps + 1)], kkt="device",
                              all_arms=bool(os.environ.get("CGB_NEWTON_ALL_ARMS")))
    print(json.dumps({k: ({kk: vv for kk, vv in v.items() if kk in ("iters", "first_divergence", "seconds")}
                          if isinstance(v, dict) else v) for k, v in out.items()}))
    report = os.environ.get("CGB_NEWTON_REPORT")
    if report:
        with open(report, "w") as f:
            json.dump(out, f, indent=1)
    # ~43 Newton iterations per load step, most of them backtracking on the max-norm merit.
    # FP64: the GPU's counts are the oracle's, step by step, unless the two runs part at a
    # convergence test that one passes and the other fails by round-off (the merit there is
    # within a factor 10 of the tolerance in both runs): that shifts the step's count by one.
    # The mixed tangent (FP32-class K, one FP64 refinement per step) changes the
    # pre-asymptotic backtracking, so its count is bounded in total. Every arm's converged
    # load-displacement path is within 1e-6 of the oracle's.
    ref = out["oracle"]["iters"]
    for arm in ("gpu_fp64", "gpu_fp64_oracle_shapes"):
        it = out[arm]["iters"]
        if it != ref:
            d = out[arm]["first_divergence"]
            assert d is not None and d["kind"] == "convergence test", (arm, out)
            for side in ("ref", "run"):
                assert 0.1 <= d[side]["merit_over_tol"] <= 10.0, (arm, out)
            assert all(abs(a - b) <= 1 for a, b in zip(it, ref)), (arm, out)
    for arm in [a for a in ("gpu_mixed_refined", "gpu_mixed_refined2", "gpu_mixed") if a in out]:
        assert abs(sum(out[arm]["iters"]) - sum(ref)) <= 0.15 * sum(ref), (arm, out)
    for arm in [a for a in out if a.startswith("gpu")]:
        assert out[arm]["path_rel_diff"] <= 1e-6, (arm, out)
