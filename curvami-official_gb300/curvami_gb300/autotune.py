"""Autotuner for the assembly's launch shape (cgb_assembler_set_tuning).

The knobs: the number of Gauss-point chunks whose FP64 residual and FP32-class tangent
kernels overlap on two streams, the residual kernel's block size, the resident CTAs per SM
of the CUDA-core merged tangent, and which tangent forms the cells (tensor cores or CUDA
cores). The best setting depends on the problem's size and neighbour counts
(a batch of small plates wants fewer, larger chunks than one big plate). ``autotune``
times every candidate on the caller's own problem and device buffers, keeps the fastest,
and caches it in a JSON file keyed by the device, the problem's size and the flags, so a
later run with the same key skips the search.
"""
from __future__ import annotations

import itertools
import json
import os
import time

import numpy as np

DEFAULT_CANDIDATES = {
    "n_chunks": (1, 2, 4, 8, 16),
    "residual_threads": (128, 256),
    "tangent_ctas_per_sm": (0, 2),
    "tangent_kind": (0,),
}


def default_cache_path() -> str:
    base = os.environ.get("CURVAMI_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "curvami_gb300")
    return os.path.join(base, "autotune.json")


def problem_key(asm, flags: int, device_name: str) -> str:
    """Device, Gauss points (to 1 %), pairs (to 1 %), blocks and flags."""
    st = asm.stats()
    n_gp = asm.faces.n_gp

    def r(v):
        return int(round(float(v), -max(0, len(str(int(v))) - 2))) if v else 0

    return f"{device_name}|gp={r(n_gp)}|pairs={r(st['pairs'])}|blocks={r(st['blocks'])}|flags={int(flags)}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time(asm, d_x, d_K, d_F, flags, repeats):
    """Seconds per assembly in steady state: `repeats` back-to-back calls (as a Newton loop
    or the benchmark issues them, so one call's tail overlaps the next one's start) between
    two synchronisations; the best of three such runs."""
    ctx = asm.ctx
    asm.assemble_device(d_x, d_K, d_F, flags)        # warm-up (and any first-call set-up)
    ctx.synchronize()
    best = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        for _ in range(repeats):
            asm.assemble_device(d_x, d_K, d_F, flags)
        ctx.synchronize()
        best = min(best, (time.perf_counter() - t0) / repeats)
    return best


def autotune(asm, d_x: int, d_K: int | None, d_F: int, flags: int, device_name: str = "gpu",
             candidates=None, cache_path: str | None = None, repeats: int = 5, force: bool = False) -> dict:
    """Pick the fastest launch shape for this assembler and flags on the given device
    buffers (x already holding a representative state), apply it, and return
    {"tuning": (n_chunks, residual_threads, tangent_ctas_per_sm, tangent_kind), "ms": ..., "cached": bool,
    "tried": {...}}."""
    path = cache_path or default_cache_path()
    key = problem_key(asm, flags, device_name)
    cache = _load(path)
    if not force and key in cache:
        t = tuple(cache[key]["tuning"])
        asm.set_tuning(*t)
        return {"tuning": t, "ms": cache[key]["ms"], "cached": True, "key": key, "tried": {}}
    cand = candidates or DEFAULT_CANDIDATES
    tried = {}
    for t in itertools.product(cand["n_chunks"], cand["residual_threads"], cand["tangent_ctas_per_sm"],
                               cand.get("tangent_kind", (0,))):
        asm.set_tuning(*t)
        tried[t] = _time(asm, d_x, d_K, d_F, flags, repeats) * 1e3
    best = min(tried, key=tried.get)
    asm.set_tuning(*best)
    cache = _load(path)
    cache[key] = {"tuning": list(best), "ms": tried[best]}
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return {"tuning": best, "ms": tried[best], "cached": False, "key": key,
            "tried": {",".join(map(str, k)): v for k, v in tried.items()}}


def spread(result) -> float:
    """Slowest over fastest candidate of a search (1.0 for a cached result)."""
    v = np.array(list(result["tried"].values())) if result["tried"] else np.array([1.0])
    return float(v.max() / v.min())
