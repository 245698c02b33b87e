"""The C ABI without a GPU: the library builds, loads and exports every entry point the
header declares; the host-side generator and the Python mirror hold together."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import curvami_gb300 as cg
from curvami_gb300 import _lib, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(cgb_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge

    ge.build()
    return cg.load_library()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "cgb_shape_build" in names and "cgb_assemble" in names and "cgb_assembler_create" in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_python_signatures_cover_header(lib):
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_null_handles_rejected(lib):
    # Argument checks run before any device work (no GPU needed).
    assert lib.cgb_assemble(None, None, None, None, 0) == _lib.CGB_ERR_INVALID
    assert lib.cgb_shape_size(None, None, None, None) == _lib.CGB_ERR_INVALID
    assert lib.cgb_create(0, None) == _lib.CGB_ERR_INVALID
    assert lib.cgb_last_error(None) == b"null context"


def test_quadrature_weights_and_rule():
    # 4x4 tensor rule integrates the plate area exactly and cubic monomials exactly.
    p = synth.square_plate(11, 0.5, 4, jitter=0.05, seed=1, crease=None)
    assert abs(p.faces.weight.sum() - 25.0) < 1e-12
    q, w = synth.GAUSS[4]
    assert abs((w * q ** 6).sum() - 2 / 7) < 1e-14
    p3 = synth.square_plate(11, 0.5, 3, crease=None)
    assert len(p3.faces.xy) == 100 * 9


def test_fold_points_offset_and_weights():
    p = synth.square_plate(11, 0.5, 3, crease="row", Kt=2e-3)
    f = p.folds[0]
    assert np.allclose(f.left.xy - f.right.xy, 2e-7 * np.array([-1.0, 0.0]))
    assert abs(f.left.weight.sum() - 5.0) < 1e-12  # crease length
    assert p.creases[0]["extend_start"] and p.creases[0]["extend_end"]


def test_split_on_crease():
    # A 1-point rule puts every Gauss point at a cell centre; a crease through the
    # centres splits each of those points in two half-weight twins.
    faces = synth.PointSet(np.array([[0.25, 0.25], [0.75, 0.25]]), np.array([1.0, 1.0]))
    cr = [{"vertices": np.array([[0.0, 0.25], [1.0, 0.25]])}]
    out, n = synth.split_on_creases(faces, cr)
    assert n == 2 and len(out.xy) == 4 and abs(out.weight.sum() - 2.0) < 1e-15


def test_ctypes_structs_match_the_header(tmp_path):
    """Every struct the Python mirror passes by pointer has the header's size and field
    offsets (a C program built with the host compiler prints them)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"cgb_crease": _lib.Crease, "cgb_shape_params": _lib.ShapeParams, "cgb_fold": _lib.Fold,
               "cgb_face_problem": _lib.FaceProblem, "cgb_tuning": _lib.Tuning,
               "cgb_natural_curvature": _lib.NaturalCurvature}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "curvami_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split("\n")
    got = {tuple(line.split()[:-1]): int(line.split()[-1]) for line in out if line.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
