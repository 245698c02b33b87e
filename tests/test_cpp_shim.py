"""The C++ shim over the C ABI, compiled with g++ and run as a C++ caller would use it,
against the Python mirror on the same inputs (deterministic scatter: bitwise equal)."""
import os
import subprocess

import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "curvami-official_gb300", "curvami_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "shim_check.cpp")


def compile_shim(tmp_path):
    import __graft_entry__ as ge

    ge.build()
    exe = str(tmp_path / "shim_check")
    subprocess.check_call(["g++", "-std=c++17", "-O1", SRC, "-o", exe, f"-L{LIBDIR}", "-lcurvami_gb300",
                           f"-Wl,-rpath,{LIBDIR}"])
    return exe


def test_shim_compiles(tmp_path):
    assert os.path.exists(compile_shim(tmp_path))


@pytest.mark.gpu
def test_shim_matches_python(tmp_path):
    exe = compile_shim(tmp_path)
    p = synth.square_plate(15, 0.5, 3, jitter=0.05, seed=17, crease="row", Kt=1e-3)
    x = 0.2 * synth.fourier_field(p.node_xy, np.random.default_rng(5), lam=(3.0, 9.0))
    A, B, D = cg.abd_isotropic(p.E, p.nu, p.thickness)
    f = p.folds[0]
    arrays = [p.node_xy, p.faces.xy, p.faces.weight, p.creases[0]["vertices"], f.left.xy, f.right.xy,
              f.left.weight, f.left.tangent, x,
              np.concatenate([[p.rho, f.Kt], np.ravel(A), np.ravel(B), np.ravel(D)])]
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        for a in arrays:
            a = np.ascontiguousarray(a, np.float64).ravel()
            fh.write(np.int64(a.size).tobytes())
            fh.write(a.tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(out, "rb").read()
    vals, off = [], 0
    for dt in (np.float64, np.float64, np.int32, np.int32):
        n = int(np.frombuffer(raw[off:off + 8], np.int64)[0]); off += 8
        k = np.dtype(dt).itemsize * n
        vals.append(np.frombuffer(raw[off:off + k], dt)); off += k
    K_cpp, F_cpp, outer_cpp, inner_cpp = vals
    m = cg.PlateModel(p)
    K, F = m.asm.assemble(x, cg.TANGENT | cg.HINGE | cg.DETERMINISTIC)
    outer, inner = m.asm.pattern()
    assert np.array_equal(outer, outer_cpp) and np.array_equal(inner, inner_cpp)
    assert np.array_equal(K, K_cpp) and np.array_equal(F, F_cpp)
