"""Benchmark: Gauss-point residual+tangent evaluations per second on one GB300.

Workload (the single-plate assembly at scale): 201x201 jittered nodes (h = 0.5,
+/-0.1 jitter) on [0,100]^2, a 4x4 Gauss rule per cell (640,000 Gauss points),
quadratic RKPM basis with the quartic window and a support radius of 3h, a circular-arc
crease of radius 60 crossing the node layout (elastic hinge, Kt = 1e-3), and a seeded
smooth displacement (8 Fourier modes per component, wavelengths 20-200, rotations up to
60 degrees). A step is one full residual + tangent assembly (faces and hinge) scattered
into the reference's CSC stiffness.

The headline arm is the mixed-precision assembly (FP64 residual, FP32 tangent, atomic
scatter); the FP64 assembly of the same library is timed alongside as the metric's
denominator, with the error of the mixed result against it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's CPU algorithm (the C++ restatement of its
OpenMP loops, built with the reference's release flags) on the host cores, on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "curvami-official_gb300")
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gauss-pt residual+tangent evals/s, mixed vs FP64 GPU at stated error"
UNIT = "GP evals/s"
SEED = 1003
# DRAM bytes (read + write) per Gauss point of the merged FP32 tangent, from one ncu capture
# of the whole 101 x 101 plate in one launch (160,000 points: 318.7 MB read + 20.9 MB
# written); the traffic per point does not depend on the plate size, so it scales to the
# full launch by its points.
TANGENT_DRAM_BYTES_PER_GP = 2122.0
TANGENT_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of face_tangent_merged_kernel over "
                          "the 101 x 101 plate in one launch (bench.py --n-side 101 --profile-mixed 1,128,0,0), "
                          "per Gauss point, times the points of one launch")
WORKLOAD = ("single-plate assembly at scale: 201x201 jittered nodes, 4x4 Gauss rule (640,000 "
            "Gauss points), quadratic RKPM, quartic window, rho = 3h, circular-arc crease R = 60 "
            "with elastic hinge Kt = 1e-3, seeded 8-mode Fourier displacement (rotations up to 60 "
            "deg); one residual + tangent assembly into the CSC stiffness per step")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-side", type=int, default=201, help="nodes per side (201 = the workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="assembly", choices=["assembly", "batched", "shape"],
                    help="assembly: the single-plate assembly at scale (the metric's workload); "
                         "batched: 64 uneven plates in one graph launch per step; "
                         "shape: the shape-function stage alone (1,000,000 points)")
    ap.add_argument("--n-points", type=int, default=1_000_000, help="points of the shape workload")
    ap.add_argument("--plates", type=int, default=64, help="plates of the batched workload")
    ap.add_argument("--no-shape-stage", action="store_true",
                    help="skip the shape-function stage object (shorter runs under a profiler)")
    ap.add_argument("--profile-mixed", default=None, metavar="CHUNKS,THREADS,CTAS,KIND",
                    help="a short run for profilers: only W + K mixed steps of the assembly workload with this "
                         "fixed launch shape (cgb_tuning fields), no autotuner and no other arm; prints one "
                         "JSON line with the step time")
    ap.add_argument("--cpu-rows", type=int, default=None,
                    help="only the first CPU_ROWS cell rows on the CPU (a quick check; default: the whole plate)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def build_workload(n_side):
    from curvami_gb300 import synth

    plate = synth.config_assembly(rule=4, n_side=n_side, seed=SEED)
    x = synth.fourier_field(plate.node_xy, np.random.default_rng(SEED + 1))
    return plate, x


# ---------------------------------------------------------------------------------
# CPU side (the oracle's restatement of the reference's OpenMP assembly)
# ---------------------------------------------------------------------------------

def cpu_workload(plate, x, rows=None):
    """The workload on the oracle: shape functions of the faces and of both sides of the
    crease (GlobalFRNN + GlobalRKPM restated), the union pattern and csrMapping
    (initSparsityPattern restated), the material; then cpu_step assembles. rows=None
    takes the whole plate; rows=r only the Gauss points of the first r cell rows, with
    their own pattern (a quick check, not a measurement of the workload)."""
    from oracle import Oracle

    h = plate.meta["h"]
    keep = np.ones(len(plate.faces.xy), bool) if rows is None else plate.faces.xy[:, 1] < rows * h
    o = Oracle(native=True)
    gp = plate.faces.xy[keep]
    w = plate.faces.weight[keep]
    t0 = time.perf_counter()
    ptr, idx, s = o.frnn(plate.node_xy, gp, plate.rho)
    psi, dpsi, ddpsi, bad, rc = o.rkpm(plate.node_xy, gp, ptr, idx, s, plate.rho, plate.order, plate.creases)
    folds = []
    for f in plate.folds:
        sel = np.ones(len(f.left.xy), bool) if rows is None else f.left.xy[:, 1] < rows * h
        side = {}
        for nm, ps in (("left", f.left), ("right", f.right)):
            fp, fi, fs = o.frnn(plate.node_xy, ps.xy[sel], plate.rho)
            _, fd, _, _, _ = o.rkpm(plate.node_xy, ps.xy[sel], fp, fi, fs, plate.rho, plate.order, plate.creases)
            side[nm] = {"ptr": fp, "idx": fi, "dpsi": fd}
        folds.append({"left": side["left"], "right": side["right"], "weight": f.left.weight[sel],
                      "tangent": f.left.tangent[sel], "Kt": f.Kt, "theta0": f.theta0})
    outer, inner, col_ptr, col_nodes, mp = o.pattern(plate.n_nodes, ptr, idx, folds)
    A, B, D = o.abd(plate.E, plate.nu, plate.thickness)
    return dict(o=o, n_gp=int(keep.sum()), w=w, ptr=ptr, idx=idx, psi=psi, dpsi=dpsi, ddpsi=ddpsi, folds=folds,
                outer=outer, inner=inner, col_ptr=col_ptr, col_nodes=col_nodes, mp=mp, A=A, B=B, D=D, x=x,
                n_nodes=plate.n_nodes, whole=rows is None, setup_s=time.perf_counter() - t0)


def cpu_step(S, threads):
    """NonLinearAssembler::updateStiffness + Constraints::evaluateElasticFold restated
    (the reference's OpenMP loops), K and F of the workload at S["x"]."""
    o = S["o"]
    K, F = o.update_stiffness(S["n_nodes"], S["w"], S["ptr"], S["idx"], S["dpsi"], S["ddpsi"], S["outer"],
                              S["mp"], S["x"], S["A"], S["B"], S["D"], want_K=True, n_threads=threads)
    return o.hinge(S["n_nodes"], S["x"], S["folds"], S["outer"], S["col_ptr"], S["col_nodes"], K, F)


def cpu_time(S, threads, steps, warmup=1):
    for _ in range(warmup):
        cpu_step(S, threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        out = cpu_step(S, threads)
    return (time.perf_counter() - t0) / steps, out


def cpu_sample_text(S):
    what = ("the whole workload (640,000 Gauss points, its pattern and hinge points)" if S["whole"] else
            f"{S['n_gp']} Gauss points of the first cell rows, with their own pattern and hinge points")
    return (f"{what}; per step NonLinearAssembler::updateStiffness + Constraints::evaluateElasticFold restated "
            f"(OpenMP, the reference's -O2 native release flags); shape functions and pattern built once by the "
            f"oracle ({S['setup_s']:.1f} s, not timed)")


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    plate, x = build_workload(args.n_side)
    S = cpu_workload(plate, x, args.cpu_rows)
    cores = os.cpu_count() or 1
    t, _ = cpu_time(S, cores, max(args.steps, 1), max(args.warmup, 1))
    v = S["n_gp"] / t
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "seed": SEED, "threads": cores, "n_gauss_points": S["n_gp"],
                   "same_config": S["whole"]},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": cpu_sample_text(S)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def rel_errors(K, F, Ko, Fo):
    """||dF||_inf / ||F_o||_inf, ||dK||_F / ||K_o||_F and max |dK| / max |K_o| against the
    oracle's K and F (the same CSC pattern, index by index)."""
    return {"F_rel_inf": float(np.abs(F - Fo).max() / np.abs(Fo).max()),
            "K_rel_fro": float(np.linalg.norm(K - Ko) / np.linalg.norm(Ko)),
            "K_rel_max": float(np.abs(K - Ko).max() / np.abs(Ko).max())}


def errors_vs_oracle(cg, ctx, plate, model, S, Ko, Fo):
    """The GPU's K and F against the oracle's on the whole workload at the same x:
    - on_oracle_shape_functions: the GPU assembly fed the oracle's Phi derivatives (faces
      and both crease sides), i.e. stage B alone on identical inputs -- the error the
      metric states;
    - on_gpu_shape_functions: the library end to end (its own stage A, then stage B);
      near the crease the FP64 shape functions of two implementations differ by about
      cond(M) eps (crease-truncated supports), which this includes."""
    g_outer, g_inner = model.asm.pattern()
    same = bool(np.array_equal(g_outer, S["outer"]) and np.array_equal(g_inner, S["inner"]))
    out = {"pattern_bit_exact": same, "n_gauss_points": S["n_gp"], "bar": "F_rel_inf <= 1e-10 (mixed, stage B)"}
    if not same:
        return out
    MIX = cg.TANGENT | cg.HINGE | cg.MIXED
    F64 = cg.TANGENT | cg.HINGE
    x = S["x"]
    gpu = {}
    for name, fl in (("mixed", MIX), ("fp64", F64)):
        K, F = model.asm.assemble(x, fl)
        gpu[name] = rel_errors(K, F, Ko, Fo)
    out["on_gpu_shape_functions"] = gpu
    faces = cg.shape_from_host(ctx, S["ptr"], S["idx"], S["dpsi"], S["ddpsi"], S["psi"])
    folds = []
    for f in S["folds"]:
        sides = {}
        for nm in ("left", "right"):
            d = f[nm]
            sides[nm] = cg.shape_from_host(ctx, d["ptr"], d["idx"], d["dpsi"], np.zeros((len(d["idx"]), 3)))
        folds.append({"left": sides["left"], "right": sides["right"], "weight": f["weight"],
                      "tangent": f["tangent"], "Kt": f["Kt"], "theta0": f["theta0"]})
    asm = cg.NonLinearAssembler(ctx, faces, S["w"], folds)
    asm.set_material(*cg.abd_isotropic(plate.E, plate.nu, plate.thickness))
    o_outer, _ = asm.pattern()
    stage_b = {}
    for name, fl in (("mixed", MIX), ("fp64", F64)):
        K, F = asm.assemble(x, fl)
        stage_b[name] = rel_errors(K, F, Ko, Fo)
    out["on_oracle_shape_functions"] = stage_b
    asm.close()
    for f in folds:
        f["left"].close(); f["right"].close()
    faces.close()
    return out


# ---------------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples (200 ms) over the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fma_peaks(device):
    import ctypes as C

    path = os.path.join(PKG_DIR, "curvami_gb300", "libcgb_peaks.so")
    lib = C.CDLL(path)
    lib.cgb_measure_fma_peaks.restype = C.c_int
    lib.cgb_measure_fma_peaks.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    f64 = C.c_double(); f32 = C.c_double()
    lib.cgb_measure_fma_peaks(device, C.byref(f64), C.byref(f32))
    return f64.value, f32.value


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_gpu(args):
    import torch

    import curvami_gb300 as cg

    from curvami_gb300.replicas import Replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    reps = Replicas()
    barrier = reps.barrier
    max_over_ranks = reps.max

    plate, x = build_workload(args.n_side)
    ctx = cg.Context(local)
    t0 = time.perf_counter()
    model = cg.PlateModel(plate, ctx)
    setup_s = time.perf_counter() - t0
    asm = model.asm
    n_gp = model.faces.n_gp
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    x_d = torch.from_numpy(x).to("cuda")
    K_d = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
    F_d = torch.empty(asm.n_dofs, dtype=torch.float64, device="cuda")
    MIX = cg.TANGENT | cg.HINGE | cg.MIXED
    F64 = cg.TANGENT | cg.HINGE
    DET = cg.TANGENT | cg.HINGE | cg.MIXED | cg.DETERMINISTIC

    def step(flags):
        asm.assemble_device(x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), flags)

    def timed(flags, steps, warmup, sampler=None):
        for _ in range(warmup):
            step(flags)
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(flags)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(e0.elapsed_time(e1) / steps)

    if args.profile_mixed:
        tuning = [int(v) for v in args.profile_mixed.split(",")]
        asm.set_tuning(*tuning)
        ms = timed(MIX, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({"profile_mixed": tuning, "workload": WORKLOAD, "n_side": args.n_side,
                              "n_gauss_points": n_gp, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": ms, "value": n_gp / (ms * 1e-3), "unit": UNIT}))
        return

    # Accuracy of the mixed assembly against the FP64 one on the same input.
    step(F64)
    K64 = K_d.cpu().numpy().copy(); F64v = F_d.cpu().numpy().copy()
    step(MIX)
    Km = K_d.cpu().numpy(); Fm = F_d.cpu().numpy()
    err = {"F_rel_inf": float(np.abs(Fm - F64v).max() / np.abs(F64v).max()),
           "K_rel_fro": float(np.linalg.norm(Km - K64) / np.linalg.norm(K64)),
           "K_rel_max": float(np.abs(Km - K64).max() / np.abs(K64).max())}
    del K64

    # Launch shape per arm from the autotuner (timed on this problem, cached per device,
    # size and flags); the FP64 arm gets its own search over a smaller candidate set.
    from curvami_gb300 import autotune as at

    dev_name = torch.cuda.get_device_name(local).replace(" ", "_")
    tune_mix = at.autotune(asm, x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), MIX, device_name=dev_name)
    tune_f64 = at.autotune(asm, x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), F64, device_name=dev_name,
                           candidates={"n_chunks": (1, 4, 8), "residual_threads": (128, 256),
                                       "tangent_ctas_per_sm": (0,)}, repeats=2)

    W = max(args.warmup, 3)
    asm.set_tuning(*tune_mix["tuning"])
    with ClockSampler(local) as clk:
        ms_mix = timed(MIX, args.steps, W)
    clocks = clk.summary()
    asm.set_tuning(*tune_f64["tuning"])
    ms_f64 = timed(F64, max(3, args.steps // 4), 3)
    asm.set_tuning(*tune_mix["tuning"])
    ms_det = timed(DET, max(3, args.steps // 4), 3)
    ms_res = timed(cg.HINGE | cg.MIXED, args.steps, 3)  # residual only (line-search trials)
    asm.set_tuning(*tune_mix["tuning"][:3], cg.TANGENT_TENSOR)   # the tensor-core tangent, same launch shape
    ms_tensor = timed(MIX, args.steps, 3)
    ctx.profile(True)
    ctx.profile_read(reset=True)
    for _ in range(args.steps):
        step(MIX)
    torch.cuda.synchronize()
    ph_tc_ms, ph_tc_n = ctx.profile_read(reset=True)
    ctx.profile(False)
    tc = asm.tensor_stats()
    asm.set_tuning(*tune_mix["tuning"])

    # Per-phase device times of the mixed step (events inside the library).
    ctx.profile(True)
    ctx.profile_read(reset=True)
    for _ in range(args.steps):
        step(MIX)
    torch.cuda.synchronize()
    ph_ms, ph_n = ctx.profile_read(reset=True)
    asm.set_tuning(*tune_f64["tuning"])
    for _ in range(max(3, args.steps // 4)):
        step(F64)
    torch.cuda.synchronize()
    ph64_ms, ph64_n = ctx.profile_read(reset=True)
    asm.set_tuning(*tune_mix["tuning"])
    ctx.profile(False)
    launches_per_step = int(sum(ph_n.values())) // max(args.steps, 1)

    # End to end through the public API with pinned host buffers: x in, K and F out.
    x_h = torch.empty(asm.n_dofs, dtype=torch.float64, pin_memory=True).numpy()
    x_h[:] = x
    K_h = torch.empty(asm.nnz, dtype=torch.float64, pin_memory=True).numpy()
    F_h = torch.empty(asm.n_dofs, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(W):
        asm.assemble(x_h, MIX, K_out=K_h, F_out=F_h)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        asm.assemble(x_h, MIX, K_out=K_h, F_out=F_h)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    barrier()

    # Roofline. The step runs two kernels per chunk: the FP64 residual kernel ("face") and,
    # on a second stream, the FP32 tangent ("tangent", the merged CUDA-core kernel, which
    # dominates). Its compute roof is the FP32 pipe; HBM is the secondary figure. Times are
    # sums over the step's chunk launches (events on each kernel's own stream).
    ptr = model.faces.download()["ptr"]
    n = np.diff(ptr).astype(np.float64)
    steps = max(args.steps, 1)
    tan_ms = ph_ms["tangent"] / steps
    res_ms = ph_ms["face"] / steps
    work = asm.stats()
    tan_launches = max(int(ph_n["tangent"]) // steps, 1)
    flops_fp64 = float((121 * n + 200).sum())                 # residual path (FP64)
    flops_total = float((181 * n * (n + 1) / 2 + 364 * n + 200).sum())
    flops_fp32 = flops_total - flops_fp64                       # the tangent's share of F_B(n)
    # Compulsory bytes of the tangent per step: per-point state (32 floats), per neighbour
    # the FP32 grad / Hessian Phi (20 B), per pair its 2-byte code, per merged entry its block
    # slot and contribution range (8 B), and the FP32 block accumulator once (48 B per block).
    alg_bytes = float((128 + 20 * n + n * (n + 1)).sum() + 8.0 * work["entries"] + 48.0 * work["blocks"])
    peaks, peak_kind = measured_peaks()
    p64, p32 = fma_peaks(local)
    tf32_peak = peaks["bf16_tflops"] / 2.0
    ach = flops_fp32 / (tan_ms * 1e-3) / 1e12
    # The tensor-core tangent (tcgen05, 3xTF32), timed in the same step: its executed MMA work
    # is five 128 x N x 8 MMAs per point (10,240 N flops).
    tan_tc_ms = ph_tc_ms["tangent"] / steps
    tensor_flops = 10240.0 * tc["point_cols"]
    roofline = {
        "bound": "fp32", "achieved": ach, "peak": p32, "unit": "TFLOP/s", "frac": ach / p32,
        "traffic": TANGENT_DRAM_BYTES_PER_GP * len(n) / tan_launches,
        "traffic_source": TANGENT_TRAFFIC_SOURCE,
        "peak_source": "measured live on this GPU (cgb_measure_fma_peaks: dependent FP32 FMA chains on "
                       "every SM); MEASURED_PEAKS.json has no CUDA-core FP32 figure",
        "kernel": "face_tangent_merged_kernel (FP32 CUDA cores, merged contributions)",
        "binding_unit": ("the L1 / shared-memory data pipe: 90 % of its peak in ncu with the kernel alone "
                         "(1.44 shared wavefronts per pair contribution), FMA pipe 42 %; in the step the FP64 "
                         "residual's loads share that pipe"),
        "achieved_what": "the reference's hand-counted tangent flops, F_B(n) - F_R(n) per Gauss point, per second",
        "launch_ms": tan_ms / tan_launches, "launches_per_step": tan_launches, "step_ms": tan_ms,
        "algorithmic_flops_per_step": flops_fp32, "work": work,
        "hbm": {"achieved_gbs": alg_bytes / (tan_ms * 1e-3) / 1e9, "peak_gbs": peaks["hbm_gbs"],
                "frac": alg_bytes / (tan_ms * 1e-3) / 1e9 / peaks["hbm_gbs"], "algorithmic_bytes_per_step": alg_bytes,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "tensor_core_tangent": {
            "kernel": "face_tangent_tc_kernel (tcgen05.mma kind::tf32, 3xTF32, A in tensor memory, accumulator "
                      "in tensor memory) + face_tangent_merged_kernel for the cells it does not take",
            "step_ms": tan_tc_ms, "launches_per_step": max(int(ph_tc_n["tangent"]) // steps, 1),
            "achieved_tflops": flops_fp32 / (tan_tc_ms * 1e-3) / 1e12,
            "tensor_pipe": {"executed_tflops": tensor_flops / (tan_tc_ms * 1e-3) / 1e12, "peak": tf32_peak,
                            "frac": tensor_flops / (tan_tc_ms * 1e-3) / 1e12 / tf32_peak,
                            "peak_source": f"{peak_kind}: TF32 dense = half of MEASURED_PEAKS.json bf16_tflops",
                            "what": "MMA flops issued (3xTF32, zero rows of each point's support and both "
                                    "triangles of the symmetric cell product included) over the tangent's time"},
            "work": tc},
        "pipes": {
            "fp64_residual": {"kernel": "face_residual_kernel", "step_ms": res_ms,
                              "achieved_tflops": flops_fp64 / (res_ms * 1e-3) / 1e12, "peak_tflops": p64,
                              "frac": flops_fp64 / (res_ms * 1e-3) / 1e12 / p64 if p64 > 0 else None,
                              "flops_per_step": flops_fp64, "peak_source": "measured live (FMA probe)"},
            "fp32_peak_tflops": p32,
        },
    }

    cpu = None
    err_oracle = None
    if rank == 0 and not args.no_cpu_baseline:
        S = cpu_workload(plate, x, args.cpu_rows)
        cores = os.cpu_count() or 1
        t_all, (Ko, Fo) = cpu_time(S, cores, 2)
        cpu = {"value": S["n_gp"] / t_all, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": cpu_sample_text(S) + ", mean of 2 steps after 1 warm-up", "same_config": S["whole"]}
        if S["whole"]:
            err_oracle = errors_vs_oracle(cg, ctx, plate, model, S, Ko, Fo)
        del S, Ko, Fo

    v_mix = world * n_gp / (ms_mix * 1e-3)
    v_f64 = world * n_gp / (ms_f64 * 1e-3)
    shape = None if args.no_shape_stage else shape_stage(cg, ctx, args, rank == 0 and not args.no_cpu_baseline)
    creasing = None if args.no_shape_stage else creasing_run(rank == 0 and not args.no_cpu_baseline)
    post = None if args.no_shape_stage else post_processing(cg, ctx, model, x_d, stream)
    four = None
    arc = None
    batched = None
    if not args.no_shape_stage:
        try:
            four = four_creases_assembly(cg, ctx, stream)
        except cg.CGBError as e:   # a rank-deficient support at the junction is reported, not hidden
            four = {"error": str(e)}
        arc = arc_length_path(cg, ctx)
        batched = batched_object(cg, ctx, args.plates, max(5, args.steps // 2), 3)

    line = {
        "metric": METRIC, "value": v_mix, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": W, "ms_per_step": ms_mix, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp64 residual + fp32 tangent",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": WORKLOAD, "seed": SEED, "n_gauss_points": n_gp, "n_nodes": plate.n_nodes,
                   "nnz_K": asm.nnz, "mean_neighbours": float(n.mean()), "max_neighbours": int(n.max()),
                   "precision": "mixed", "scatter": "atomic",
                   "l2": "inputs larger than L2 every step (grad/Hessian Phi 0.73 GB + slot map 1.0 GB)",
                   "setup_s": setup_s,
                   "launch_shape": {"mixed": list(tune_mix["tuning"]), "fp64": list(tune_f64["tuning"]),
                                    "mixed_tried_ms": tune_mix["tried"], "fp64_tried_ms": tune_f64["tried"],
                                    "note": "(chunks, residual threads, tangent CTAs/SM; 0 = default) "
                                            "picked by curvami_gb300/autotune.py on this problem"}},
        "fp64": {"value": v_f64, "ms_per_step": ms_f64, "mixed_over_fp64": ms_f64 / ms_mix,
                 "phases_ms": {k: v / max(3, args.steps // 4) for k, v in ph64_ms.items()}},
        "deterministic_mixed": {"value": world * n_gp / (ms_det * 1e-3), "ms_per_step": ms_det},
        "residual_only": {"value": world * n_gp / (ms_res * 1e-3), "ms_per_step": ms_res},
        "mixed_tensor_core_tangent": {"value": world * n_gp / (ms_tensor * 1e-3), "ms_per_step": ms_tensor,
                                      "what": "the same step with the tensor-core tangent (tcgen05, 3xTF32) for "
                                              "every cell whose node union fits one 128-row tile"},
        "error_mixed_vs_fp64": err,
        "error_vs_oracle": err_oracle,
        "phases_ms": {k: v / max(args.steps, 1) for k, v in ph_ms.items()},
        "e2e": {"value": world * n_gp / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(asm.n_dofs * 8),
                "d2h_bytes_per_step": int(asm.nnz * 8 + asm.n_dofs * 8)},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "shape_stage": shape,
        "progressive_creasing": creasing,
        "four_creases": four,
        "arc_length_path": arc,
        "batched": batched,
        "post_processing": post,
    }
    if rank == 0:
        print(json.dumps(line))
    reps.close()


# ---------------------------------------------------------------------------------
# Shape-function stage alone (1,000,000 points over a 401 x 401 jittered node grid)
# ---------------------------------------------------------------------------------

SHAPE_SEED = 1002


def reproducing_error(d, node_xy, pts, scale):
    """max over points of |scale^|a| sum_I D^a Phi_I t_I^b - a! delta_ab|, t_I = (X_I - x) /
    scale, for the quadratic monomials b and the jets a = value, x, y, xx, yy, xy (the RKPM
    reproducing conditions, GlobalRKPM.h:361-397), per derivative order 0 / 1 / 2."""
    import torch

    dev = torch.device("cuda")
    ptr = torch.from_numpy(d["ptr"]).to(dev)
    n = len(ptr) - 1
    row = torch.repeat_interleave(torch.arange(n, device=dev), ptr[1:] - ptr[:-1])
    idx = torch.from_numpy(d["idx"].astype(np.int64)).to(dev)
    X = torch.from_numpy(node_xy).to(dev)[idx]
    P = torch.from_numpy(pts).to(dev)[row]
    t = (X - P) / scale
    tx, ty = t[:, 0], t[:, 1]
    mono = [torch.ones_like(tx), tx, ty, tx * tx, tx * ty, ty * ty]
    dp = torch.from_numpy(d["dpsi"].reshape(-1, 2)).to(dev)
    ddp = torch.from_numpy(d["ddpsi"].reshape(-1, 3)).to(dev)
    jets = [torch.from_numpy(d["psi"]).to(dev), dp[:, 0] * scale, dp[:, 1] * scale,
            ddp[:, 0] * scale ** 2, ddp[:, 1] * scale ** 2, ddp[:, 2] * scale ** 2]
    expect = {(0, 0): 1.0, (1, 1): 1.0, (2, 2): 1.0, (3, 3): 2.0, (4, 5): 2.0, (5, 4): 1.0}
    worst = [0.0, 0.0, 0.0]
    for a, J in enumerate(jets):
        for b, m in enumerate(mono):
            acc = torch.zeros(n, dtype=torch.float64, device=dev).index_add_(0, row, J * m)
            acc -= expect.get((a, b), 0.0)
            order = 0 if a == 0 else (1 if a < 3 else 2)
            worst[order] = max(worst[order], float(acc.abs().max()))
    return {"order0": worst[0], "order1": worst[1], "order2": worst[2]}


def shape_stage(cg, ctx, args, with_cpu):
    from curvami_gb300 import synth

    plate, pts = synth.config_shape_points(seed=SHAPE_SEED)
    ctx.set_nodes(plate.node_xy)
    kw = dict(rho=plate.rho, order=plate.order, creases=plate.creases, rho_node=plate.rho_node,
              kernel=plate.kernel)
    steps = max(3, args.steps // 4)
    for _ in range(max(args.warmup, 3)):
        cg.shape_functions(ctx, pts, **kw)
    t0 = time.perf_counter()
    for _ in range(steps):
        sh = cg.shape_functions(ctx, pts, **kw)
    wall = (time.perf_counter() - t0) / steps
    ctx.profile(True)
    ctx.profile_read(reset=True)
    sh = cg.shape_functions(ctx, pts, **kw)
    ph, _ = ctx.profile_read(reset=True)
    ctx.profile(False)
    d = sh.download()
    nnz = int(d["ptr"][-1])
    n = np.diff(d["ptr"])
    # Progressive creasing's per-step stage A: the same set rebuilt in place for a cut that
    # moves every step (cgb_shape_rebuild: neighbour lists kept, no FRNN), alternating the
    # cut stopped at the middle of its path with the full cut; the last rebuild (full cut)
    # must reproduce the first build's bits.
    full = plate.creases[0]
    v = np.asarray(full["vertices"], np.float64)
    half = {"vertices": np.vstack([v[0], 0.5 * (v[0] + v[-1])]), "extend_start": full.get("extend_start", False),
            "extend_end": False, "is_closed": False}
    cuts = ([half], list(plate.creases))
    for c in cuts:
        sh.rebuild(c)
    ctx.synchronize()
    t0 = time.perf_counter()
    for i in range(2 * steps):
        sh.rebuild(cuts[i % 2])
    ctx.synchronize()
    wall_rb = (time.perf_counter() - t0) / (2 * steps)
    d2 = sh.download()
    rebuild_same = bool(all(np.array_equal(d[k], d2[k]) for k in ("psi", "dpsi", "ddpsi")))
    out = {
        "workload": ("1,000,000 uniform points in [0,200]^2 over 401x401 jittered nodes (+/-0.2h), quadratic "
                     "basis, cubic B-spline window, per-node support radius U[2.5h, 3.5h], one straight cut "
                     "along the node row y = 100; outputs Phi, grad Phi, Hessian Phi (FP64)"),
        "seed": SHAPE_SEED, "n_points": len(pts), "pairs": nnz, "neighbours_min_mean_max":
            [int(n.min()), float(n.mean()), int(n.max())],
        "value": len(pts) / wall, "unit": "points/s", "ms_per_build": wall * 1e3,
        "phases_ms": {k: ph[k] for k in ("frnn", "crease", "rkpm")},
        "rkpm_points_per_s": len(pts) / (ph["rkpm"] * 1e-3) if ph["rkpm"] > 0 else None,
        "reproducing_error": reproducing_error(d, plate.node_xy, pts, 1.5),
        "precision": "fp64",
        "rebuild": {"ms_per_rebuild": wall_rb * 1e3, "points_per_s": len(pts) / wall_rb,
                    "bitwise_equal_to_build": rebuild_same,
                    "what": "cgb_shape_rebuild of the same set for a moved cut (progressive creasing's "
                            "per-step stage A), alternating the half and the full cut"},
    }
    out["mixed"] = shape_stage_mixed(cg, ctx, plate, pts, kw, steps, d, cuts)
    if with_cpu:
        # The oracle's restatement of GlobalFRNN::execute + GlobalRKPM::solve (OpenMP, all
        # host threads) on the first 20,000 points, and the GPU's difference from it there.
        from oracle import Oracle

        o = Oracle(native=True)
        m = 20000
        t0 = time.perf_counter()
        ptr, idx, sdist = o.frnn(plate.node_xy, pts[:m], plate.rho, plate.rho_node)
        psi, dpsi, ddpsi, bad, rc = o.rkpm(plate.node_xy, pts[:m], ptr, idx, sdist, plate.rho, plate.order,
                                           plate.creases, plate.rho_node, plate.kernel)
        t_cpu = time.perf_counter() - t0
        e = int(ptr[-1])
        same = bool(np.array_equal(ptr, d["ptr"][: m + 1]) and np.array_equal(idx, d["idx"][:e]))

        def rel(a, b):
            return float(np.abs(a - b).max() / np.abs(b).max())

        out["cpu_baseline"] = {"value": m / t_cpu, "unit": "points/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"first {m} points (FRNN + RKPM)"}
        out["error_vs_oracle"] = {
            "neighbours_bit_exact": same,
            "psi": rel(d["psi"][:e], psi), "dpsi": rel(d["dpsi"][:e].reshape(-1), dpsi.reshape(-1)),
            "ddpsi": rel(d["ddpsi"][:e].reshape(-1), ddpsi.reshape(-1)), "sample_points": m}
        dm = out["mixed"].pop("_values")
        out["mixed"]["error_vs_oracle"] = {
            "psi": rel(dm["psi"][:e], psi), "dpsi": rel(dm["dpsi"][:e].reshape(-1), dpsi.reshape(-1)),
            "ddpsi": rel(dm["ddpsi"][:e].reshape(-1), ddpsi.reshape(-1)), "sample_points": m}
    out["mixed"].pop("_values", None)
    return out


def shape_stage_mixed(cg, ctx, plate, pts, kw, steps, d64, cuts):
    """The same 1,000,000-point build with the mixed-precision RKPM (per-neighbour sums in
    FP32 pairs on the FP32 pipe, per-point factorisation in FP64): time per build, per
    phase, per rebuild, the reproducing-condition error, and the difference from the FP64
    build of the same points (relative to each array's scale; over all points, and over
    the points whose support the cut does not reach)."""
    mkw = dict(kw, precision="mixed")
    for _ in range(3):
        cg.shape_functions(ctx, pts, **mkw)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sh = cg.shape_functions(ctx, pts, **mkw)
    wall = (time.perf_counter() - t0) / steps
    ctx.profile(True)
    ctx.profile_read(reset=True)
    sh = cg.shape_functions(ctx, pts, **mkw)
    ph, _ = ctx.profile_read(reset=True)
    ctx.profile(False)
    dm = sh.download()
    for c in cuts:
        sh.rebuild(c)
    ctx.synchronize()
    t0 = time.perf_counter()
    for i in range(2 * steps):
        sh.rebuild(cuts[i % 2])
    ctx.synchronize()
    wall_rb = (time.perf_counter() - t0) / (2 * steps)
    # Points whose support the cut y = 100 does not reach (largest radius 3.5h = 1.75).
    far_pt = np.abs(pts[:, 1] - 100.0) > 1.75 + 0.2
    far = np.repeat(far_pt, np.diff(d64["ptr"]))

    def rel(a, b, mask=None):
        if mask is not None:
            a, b = a[mask], b[mask]
        return float(np.abs(a - b).max() / np.abs(b).max())

    err = {}
    for k, m in (("psi", 1), ("dpsi", 2), ("ddpsi", 3)):
        a, b = dm[k].reshape(-1), d64[k].reshape(-1)
        err[k] = {"all": rel(a, b), "away_from_cut": rel(a, b, np.repeat(far, m))}
    return {
        "precision": "mixed (per-neighbour sums in FP32 pairs, per-point LDL^T and solves in FP64)",
        "value": len(pts) / wall, "unit": "points/s", "ms_per_build": wall * 1e3,
        "phases_ms": {k: ph[k] for k in ("frnn", "crease", "rkpm")},
        "rkpm_points_per_s": len(pts) / (ph["rkpm"] * 1e-3) if ph["rkpm"] > 0 else None,
        "reproducing_error": reproducing_error(dm, plate.node_xy, pts, 1.5),
        "error_vs_fp64_gpu": err,
        "neighbours_same_as_fp64": bool(np.array_equal(dm["idx"], d64["idx"])),
        "rebuild": {"ms_per_rebuild": wall_rb * 1e3, "points_per_s": len(pts) / wall_rb},
        "_values": dm,
    }


# ---------------------------------------------------------------------------------
# Post-processing: the kinematic state of every face Gauss point (exporter / sampler)
# ---------------------------------------------------------------------------------

def post_processing(cg, ctx, model, x_d, stream):
    """cgb_point_state_device over the 640,000 face Gauss points of the workload: per point
    the displacement sum and Kinematics::compute + Constitutive::evaluate in FP64 (18 FMA
    per neighbour), 33 doubles out. Timed with CUDA events; roofline against the FP64 FMA
    peak (measured live) and HBM."""
    import torch
    from curvami_gb300 import _lib as L

    S = model.faces
    n = S.n_gp
    out = torch.empty((n, L.POINT_STATE_COLS), dtype=torch.float64, device="cuda")
    A, B, D = (np.ascontiguousarray(M, np.float64).reshape(9) for M in (model.asm.A, model.asm.B, model.asm.D))

    def call():
        ctx.check(ctx.lib.cgb_point_state_device(ctx.h, S.h, ctx_ptr(x_d), A.ctypes.data, B.ctypes.data,
                                                 D.ctypes.data, ctx_ptr(out)))

    def ctx_ptr(t):
        return __import__("ctypes").c_void_p(t.data_ptr())

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nnz = S.nnz
    flops = 2.0 * 18 * nnz          # Psi u (3) + the 15 kinematic sums per neighbour
    bytes_ = nnz * (4 + 8 + 16 + 24 + 24) + n * (8 + 33 * 8)
    p64, _ = fma_peaks(torch.cuda.current_device())
    peaks, kind = measured_peaks()
    return {"what": "cgb_point_state_device, 640,000 face Gauss points (Exporter rows / StressSampler state)",
            "ms": ms, "points_per_s": n / (ms * 1e-3),
            "fp64_tflops": flops / (ms * 1e-3) / 1e12,
            "fp64_frac": (flops / (ms * 1e-3) / 1e12) / p64 if p64 > 0 else None,
            "algorithmic_GBps": bytes_ / (ms * 1e-3) / 1e9,
            "hbm_frac": bytes_ / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"], "peak_source": kind,
            "bytes_per_point": bytes_ / n, "flops_per_point": flops / n}


# ---------------------------------------------------------------------------------
# Four creases from the centre at 2.56 M Gauss points (one assembly, both precisions)
# ---------------------------------------------------------------------------------

FOUR_SEED = 1005


def four_creases_assembly(cg, ctx, stream):
    """401 x 401 jittered nodes, 4x4 rule (2,560,000 Gauss points), four straight creases from
    the centre with sectors 90 +/- 15 deg: two elastic hinges in the assembly, two rigid folds
    (constraint rows of the Newton driver, not assembled). Shape functions once, then the
    mixed and the FP64 assembly, each timed over a few calls, and their F difference."""
    import dataclasses

    import torch
    from curvami_gb300 import synth

    t0 = time.perf_counter()
    p = synth.four_crease_plate(401, rule=4, seed=FOUR_SEED)
    gen_s = time.perf_counter() - t0
    elastic = dataclasses.replace(p, folds=[f for f in p.folds if not f.rigid])
    ctx.set_nodes(p.node_xy)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    model = cg.PlateModel(elastic, ctx)
    ctx.synchronize()
    setup_s = time.perf_counter() - t0
    asm = model.asm
    x = synth.fourier_field(p.node_xy, np.random.default_rng(FOUR_SEED))
    x_d = torch.from_numpy(x).to("cuda")
    K_d = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
    F_d = torch.empty(asm.n_dofs, dtype=torch.float64, device="cuda")
    F64 = cg.TANGENT | cg.HINGE
    MIX = F64 | cg.MIXED

    def timed(flags, n):
        asm.assemble_device(x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), flags)
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            asm.assemble_device(x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), flags)
        e1.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    ms_mix = timed(MIX, 10)
    F_mix = F_d.cpu().numpy().copy()
    ms_f64 = timed(F64, 3)
    F_f64 = F_d.cpu().numpy()
    st = asm.stats()
    n_gp = model.faces.n_gp
    out = {"workload": "401x401 nodes (h = 0.5, jitter +/-0.1), 4x4 rule, quadratic RKPM, rho = 3.5h, four "
                       "creases from the centre (two elastic hinges Kt = 1e-3 assembled, two rigid folds as "
                       "constraint rows), seeded 8-mode Fourier displacement",
           "seed": FOUR_SEED, "sector_deg": p.meta["sector_deg"], "n_gauss_points": n_gp,
           "n_nodes": len(p.node_xy), "nnz_K": asm.nnz, "pairs": st["pairs"], "generate_s": gen_s,
           "shape_and_pattern_s": setup_s,
           "mixed": {"ms_per_assembly": ms_mix, "value": n_gp / (ms_mix * 1e-3)},
           "fp64": {"ms_per_assembly": ms_f64, "value": n_gp / (ms_f64 * 1e-3)},
           "mixed_over_fp64": ms_f64 / ms_mix,
           "F_rel_diff_mixed_vs_fp64": float(np.abs(F_mix - F_f64).max() / np.abs(F_f64).max()),
           "unit": UNIT}
    del model, asm
    return out


def arc_length_path(cg, ctx, n_side=41, target_deg=150.0, kmax=80):
    """The full arc-length path at reduced size: NonLinearSolver::KinematicArcLength restated
    (curvami_gb300/arclength.py) over the GPU's FP64 assembly with the exact hinge tangent
    (the predictor of this thin plate, t / L = 2.5e-3, needs the FP64 tangent: with the FP32
    one the run reversed its first steps). Four creases from the centre, sectors
    90 +/- 15 deg (seeded);
    creases 0 and 2 are the drivers (stiff hinges, Kt = 0.1, whose rest angle goes from 0 to
    150 deg with the deployment parameter mu), 1 and 3 passive elastic hinges (Kt = 1e-3);
    three point supports in sector 0. The drivers' load direction is the exact fold-angle
    gradient (an extension: the reference's formula drifts as the fold closes). The KKT
    system is solved on the GPU by a dense FP32 LU refined against the FP64 residual (solver
    "device_mixed", standing in for MUMPS), timed on its own line with the host's constraint
    work."""
    import math

    from curvami_gb300 import arclength as A
    from curvami_gb300 import solver as S
    from curvami_gb300 import synth

    p = synth.four_crease_plate(n_side=n_side, h=0.5, rule=4, seed=FOUR_SEED, Kt=1e-3, rho_factor=3.5)
    for k, f in enumerate(p.folds):
        f.rigid = False
        f.Kt = 1e-1 if k % 2 == 0 else 1e-3
    doms = A.sector_supports(p, 0, 1)
    ctx.set_nodes(p.node_xy)
    model = cg.PlateModel(p, ctx)
    prob = S.gpu_problem(model, points=doms, exact_hinge=True)
    drivers = [A.Driver(0, 0.0, math.radians(target_deg)), A.Driver(2, 0.0, math.radians(target_deg))]
    # ds bounded as for the 13 x 13 plate of the tests (dsmax 2), scaled with the plate's
    # displacement norm (nodes x width).
    sol = A.ArcLengthSolver(kmax=kmax, max_iters=30, dsmax=2.0 * (n_side / 13.0) ** 2, kkt="device_mixed",
                            exact_fold_gradient=True)
    t0 = time.perf_counter()
    sol.kinematic_arc_length(prob, np.zeros(prob.ns), drivers)
    wall = time.perf_counter() - t0
    last = sol.steps[-1] if sol.steps else None
    out = {
        "what": ("KinematicArcLength (plate/NonLinearSolver.h:607-812) restated, over the GPU FP64 assembly, to a "
                 f"{target_deg:.0f} deg rest angle of the drivers; the same path on the 401x401 plate is not run: its "
                 "482k-dof KKT needs a sparse direct solver (MUMPS and cuDSS are absent here)"),
        "n_side": n_side, "n_dofs": prob.ns, "n_gauss_points": model.faces.n_gp, "n_constraint_rows":
            int(len(sol.ind_rows)), "sector_deg": p.meta["sector_deg"], "seed": FOUR_SEED,
        "accepted_steps": len(sol.steps), "failed_steps": sol.failed_steps,
        "corrector_iterations": [st.iterations for st in sol.steps],
        "final_mu": last.load if last else None,
        "final_fold_angles_deg": last.angles if last else None,
        "wall_s": wall, "timing_s": dict(sol.timing), "counts": dict(sol.counts),
        "ms_per_assembly": 1e3 * sol.timing["assemble_s"] / max(sol.counts["assemblies"], 1),
        "ms_per_kkt_factorisation": 1e3 * sol.timing["kkt_s"] / max(sol.counts["kkt_factorisations"], 1),
    }
    del model, prob
    return out


# ---------------------------------------------------------------------------------
# Progressive creasing: the reference's centre-crease smoke example end to end
# ---------------------------------------------------------------------------------

SMOKE_PUBLISHED = {"E_mem": 4.006e-08, "E_ben": 9.404e-06, "E_hin": 1.594e-05, "theta_mean_deg": 0.1962}


def creasing_run(with_cpu):
    """The reference's smoke example (examples/smoke_centre_crease: 20 x 20 sheet, order-3
    RKPM at rho = 6h, crease grown from the centre in 5 steps, LineSearch at each) run by
    curvami_gb300.creasing over the GPU library: every tip move rebuilds all shape functions
    on the GPU, every Newton iteration assembles there (FP64, exact hinge tangent); the KKT
    solve is a dense FP64 LU on the GPU. Reported: wall time of the whole run, the GPU time
    per phase, the Newton iterations, and the last step against the published row."""
    import tempfile

    import curvami_gb300 as cg
    from curvami_gb300 import creasing as PC
    from curvami_gb300 import solver as S

    fx = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "smoke_centre_crease_nodes.npy")
    xy = np.load(fx) if os.path.exists(fx) else None
    tmp = tempfile.mkdtemp()
    case = PC.centre_crease_case(os.path.join(tmp, "smoke.msh"), 20, node_xy=xy)
    out = {"workload": ("examples/smoke_centre_crease of the reference: [-1,1]^2 sheet, 20x20 quads (3x3 rule, "
                        "3600 face points), cubic RKPM at rho = 6h (up to 113 neighbours), crease grown "
                        "middle_out over 10 segments (6 steps), theta0* = 0.5 deg, Kt = D, three corner "
                        "supports, LineSearch to 1e-10 / 1e-12"),
           "mesh": "gmsh node coordinates of the reference's CB_n20.msh" if xy is not None else "ideal grid",
           "published_last_step": SMOKE_PUBLISHED}
    # One untimed run first: the first dense LU and LU solve of the KKT size load their
    # library kernels (seconds), which is set-up, not the run.
    for name, mixed in (("warm-up", True), ("fp64", False), ("mixed", True)):
        ctx = cg.Context(0)
        t0 = time.perf_counter()
        model = cg.PlateModel(case.plate, ctx)
        plate = PC.GpuCreasingPlate(model, case.point_bcs, [case.spec], exact_tangent=True, mixed=mixed)
        setup = time.perf_counter() - t0
        solver = S.ContinuationSolver(kkt="device", refine_steps=1 if mixed else 0, **case.solver_args)
        ctx.profile(True)
        ctx.profile_read(reset=True)
        x = np.zeros(3 * len(case.plate.node_xy))
        t0 = time.perf_counter()
        res = PC.run(solver, plate, x, [case.line], cfg=case.config)
        wall = time.perf_counter() - t0
        ph, nl = ctx.profile_read(reset=True)
        ctx.profile(False)
        last = res.steps[-1] if res.steps else {}
        if name == "warm-up":
            del plate, model
            ctx.close()
            continue
        out[name] = {
            "setup_s": setup, "run_s": wall, "stopped": res.stopped, "steps": len(res.steps),
            "newton_iters": [r["newton_iters"] for r in res.steps],
            "assemblies": plate.problem.n_assemble, "residual_assemblies": plate.problem.n_residual,
            "last_step": {k: last.get(k) for k in SMOKE_PUBLISHED},
            "matches_published": bool(last) and all(
                abs(last[k] - v) <= 0.5 * 10 ** (np.floor(np.log10(abs(v))) - 3) + 2e-4 * abs(v)
                for k, v in SMOKE_PUBLISHED.items()),
            "gpu_ms": {"rebuild (crease + rkpm)": ph["crease"] + ph["rkpm"],
                       "assembly (face + tangent + hinge + reduce)": ph["face"] + ph["tangent"] + ph["hinge"] +
                       ph["reduce"], "copies": ph["h2d"] + ph["d2h"] + ph["zero"]},
            "gpu_launches": int(sum(nl.values())),
            "precision": "FP64 assembly" if not mixed else "FP64 residual + FP32 tangent, one FP64 refinement "
                                                            "of each Newton step",
        }
        del plate, model
        ctx.close()
    if with_cpu:
        # The oracle's restatement of the same run (OpenMP over the host threads).
        from oracle import Oracle
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests"))
        import creasing_helpers as H

        o = Oracle(native=True)
        plate = H.OracleCreasingPlate(o, case.plate, case.spec, case.point_bcs)
        x = np.zeros(3 * len(case.plate.node_xy))
        t0 = time.perf_counter()
        res = PC.run(S.ContinuationSolver(**case.solver_args), plate, x, [case.line], cfg=case.config)
        wall = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": wall, "unit": "s per run", "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": "the whole run (6 steps), oracle assembly and shape functions, sparse LU KKT",
                               "last_step": {k: res.steps[-1][k] for k in SMOKE_PUBLISHED} if res.steps else None}
    return out


# ---------------------------------------------------------------------------------
# Batched uneven plates: one assembler over all plates, one CUDA-graph launch per step
# ---------------------------------------------------------------------------------

BATCH_SEED = 1004


def batched_object(cg, ctx, n_plates, steps, warmup, reps=None, with_fp64=True):
    """Config 4 (batched uneven plates): n_plates plates with node sides U{21..161}, 1-3
    straight or arc creases each, assembled as one problem (PlateBatch); every step is one
    CUDA-graph launch of the whole assembly (the residual kernel takes 32-point units from a
    work counter and the tangent kernels stride over the cells of all plates: one global
    work list), launch shape from the autotuner. The mixed step's residual is compared with
    the FP64 assembly of the same batch."""
    import torch

    from curvami_gb300 import autotune as at
    from curvami_gb300 import synth

    t0 = time.perf_counter()
    plates, xs = synth.config_batched(n_plates, seed=BATCH_SEED)   # the same batch on every rank
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = cg.PlateBatch(plates, ctx)
    setup_s = time.perf_counter() - t0
    asm = batch.asm
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    x_d = torch.from_numpy(np.concatenate(xs)).to("cuda")
    K_d = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
    F_d = torch.empty(asm.n_dofs, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    MIX = cg.TANGENT | cg.HINGE | cg.MIXED
    F64 = cg.TANGENT | cg.HINGE
    name = torch.cuda.get_device_name(torch.cuda.current_device()).replace(" ", "_")
    tune = at.autotune(asm, x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), MIX, device_name=name)
    barrier = reps.barrier if reps else (lambda: None)
    mx = reps.max if reps else (lambda v: v)

    def timed_graph(flags, n, w):
        g = asm.graph(x_d.data_ptr(), K_d.data_ptr(), F_d.data_ptr(), flags)
        for _ in range(w):
            g.launch()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            g.launch()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        g.close()
        return mx(e0.elapsed_time(e1) / n)

    ms_mix = timed_graph(MIX, steps, warmup)
    F_mix = F_d.cpu().numpy().copy()
    K_mix = K_d.clone() if with_fp64 else None
    out = {"workload": (f"batched uneven plates: {len(plates)} independent plates, node side U{{21..161}}, 4x4 rule, "
                        "1-3 non-crossing straight or arc creases, Kt log-uniform [1e-4, 1e-1], seeded smooth "
                        "displacement per plate; all plates in one assembler, one CUDA-graph launch per step"),
           "seed": BATCH_SEED, "plates": len(plates), "n_gauss_points": batch.n_gp,
           "n_nodes": int(batch.node_offset[-1]), "nnz_K": asm.nnz,
           "sides_min_max": [min(int(p.meta["n_side"]) for p in plates), max(int(p.meta["n_side"]) for p in plates)],
           "creases": int(sum(len(p.creases) for p in plates)), "generate_s": gen_s, "setup_s": setup_s,
           "value": batch.n_gp / (ms_mix * 1e-3), "unit": UNIT, "ms_per_step": ms_mix,
           "autotune": {"tuning": list(tune["tuning"]), "cached": tune["cached"], "ms": tune["ms"]},
           "tensor_work": asm.tensor_stats()}
    # Roofline of the graph step: the hand-counted flops of every point (F_B(n), the tangent's
    # share on the FP32 pipe, F_R(n) on the FP64 pipe) over the whole step, in which the two
    # kernels overlap; against the FP32 and FP64 peaks measured live on this GPU.
    n = np.diff(batch.faces.download()["ptr"]).astype(np.float64)
    fl64 = float((121 * n + 200).sum())
    fl32 = float((181 * n * (n + 1) / 2 + 364 * n + 200).sum()) - fl64
    p64, p32 = fma_peaks(torch.cuda.current_device())
    a32 = fl32 / (ms_mix * 1e-3) / 1e12
    a64 = fl64 / (ms_mix * 1e-3) / 1e12
    out["roofline"] = {"bound": "fp32", "achieved": a32, "peak": p32, "unit": "TFLOP/s", "frac": a32 / p32,
                       "what": "the reference's hand-counted tangent flops, F_B(n) - F_R(n) per Gauss point, over "
                               "the whole graph step (the FP64 residual overlaps it)",
                       "fp64_residual": {"achieved": a64, "peak": p64, "frac": a64 / p64 if p64 > 0 else None},
                       "peak_source": "measured live on this GPU (cgb_measure_fma_peaks)",
                       "mean_neighbours": float(n.mean())}
    if with_fp64:
        ms_f64 = timed_graph(F64, max(3, steps // 4), 3)
        F_f64 = F_d.cpu().numpy()
        out["fp64"] = {"value": batch.n_gp / (ms_f64 * 1e-3), "ms_per_step": ms_f64, "mixed_over_fp64": ms_f64 / ms_mix}
        out["F_rel_diff_mixed_vs_fp64"] = float(np.abs(F_mix - F_f64).max() / np.abs(F_f64).max())
        # Per plate: each plate's block of F (its dofs) against the same plate's FP64 values.
        off = 3 * np.asarray(batch.node_offset, np.int64)
        per = [float(np.abs(F_mix[a:b] - F_f64[a:b]).max() / max(np.abs(F_f64[a:b]).max(), 1e-300))
               for a, b in zip(off[:-1], off[1:])]
        out["F_rel_inf_per_plate_max"] = max(per)
        out["K_rel_fro_mixed_vs_fp64"] = float(torch.linalg.vector_norm(K_mix - K_d) / torch.linalg.vector_norm(K_d))
        del K_mix
    del batch, asm
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    return out


def run_batched(args):
    import torch

    import curvami_gb300 as cg
    from curvami_gb300.replicas import Replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    reps = Replicas()
    ctx = cg.Context(local)
    W = max(args.warmup, 3)
    with ClockSampler(local) as clk:
        b = batched_object(cg, ctx, args.plates, args.steps, W, reps)
    line = {
        "metric": METRIC, "value": world * b["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": W, "ms_per_step": b["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64 residual + fp32-class tangent",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {k: b[k] for k in ("workload", "seed", "plates", "n_gauss_points", "n_nodes", "nnz_K",
                                     "sides_min_max", "creases", "generate_s", "setup_s")},
        "fp64": b.get("fp64"), "autotune": b["autotune"], "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))
    reps.close()


def run_shape(args):
    """The shape-function stage alone (GlobalFRNN::execute + GlobalRKPM::solve on
    1,000,000 points): builds per second in the mixed mode, with the FP64 mode beside it.
    A step is one build (FRNN, crease indicators, RKPM, guards, host set-up); the RKPM
    phase is also timed on the device by the library's event profiler."""
    import torch

    import curvami_gb300 as cg
    from curvami_gb300 import synth
    from curvami_gb300.replicas import Replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    reps = Replicas()
    plate, pts = synth.config_shape_points(n_points=args.n_points, seed=SHAPE_SEED)
    ctx = cg.Context(local)
    ctx.set_nodes(plate.node_xy)
    kw = dict(rho=plate.rho, order=plate.order, creases=plate.creases, rho_node=plate.rho_node,
              kernel=plate.kernel)
    W = max(args.warmup, 3)

    def timed(prec, steps):
        for _ in range(W):
            cg.shape_functions(ctx, pts, precision=prec, **kw)
        ctx.synchronize()
        reps.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            sh = cg.shape_functions(ctx, pts, precision=prec, **kw)
        ctx.synchronize()
        wall = reps.max((time.perf_counter() - t0) * 1e3 / steps)
        ctx.profile(True)
        ctx.profile_read(reset=True)
        cg.shape_functions(ctx, pts, precision=prec, **kw)
        ph, _ = ctx.profile_read(reset=True)
        ctx.profile(False)
        return wall, {k: ph[k] for k in ("frnn", "crease", "rkpm")}, sh

    with ClockSampler(local) as clk:
        ms_mx, ph_mx, sh = timed("mixed", args.steps)
    nnz = sh.nnz
    del sh
    ms_64, ph_64, _ = timed("fp64", max(3, args.steps // 4))
    line = {
        "metric": "shape-function evaluations (Phi, grad Phi, Hessian Phi per point) per second, mixed vs FP64 GPU",
        "value": world * len(pts) / (ms_mx * 1e-3), "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": W, "ms_per_step": ms_mx, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 pairs per neighbour, fp64 per point", "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": (f"{len(pts):,} uniform points in [0,200]^2 over 401x401 jittered nodes (+/-0.2h), "
                                "quadratic basis, cubic B-spline window, per-node support radius U[2.5h, 3.5h], one "
                                "straight cut along the node row y = 100; one build (FRNN + crease indicators + RKPM) "
                                "per step"), "seed": SHAPE_SEED, "pairs": nnz,
                   "inputs": "larger than L2 (outputs 1.7 GB per build)"},
        "phases_ms": ph_mx,
        "rkpm_points_per_s": len(pts) / (ph_mx["rkpm"] * 1e-3) if ph_mx["rkpm"] > 0 else None,
        "fp64": {"value": world * len(pts) / (ms_64 * 1e-3), "ms_per_step": ms_64, "phases_ms": ph_64,
                 "rkpm_mixed_over_fp64": ph_64["rkpm"] / ph_mx["rkpm"] if ph_mx["rkpm"] > 0 else None},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))
    reps.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "shape":
        run_shape(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
