"""Mesh input (curvami_gb300/mesh.py): the msh 4.1 reader, the quadrature, crease extraction
and the support radius, on synthetic meshes written with the module's writer, and on the
reference's example meshes when they are present (this container only)."""
import os

import numpy as np
import pytest

from curvami_gb300 import mesh, synth

# The reference tree, when present (CURVAMI_REFERENCE names its root); tests that read it
# skip otherwise.
_REF = os.environ.get("CURVAMI_REFERENCE")
REF_MESH = os.path.join(_REF, "examples", "smoke_centre_crease", "CB_n20.msh") if _REF else ""


def grid_mesh(n=9, h=0.5, crease_col=4):
    xy = synth.grid_nodes(n, n, h, 0.0, np.random.default_rng(0))
    els = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i
            els.append(mesh.Element(3, 1, (a, a + 1, a + n + 1, a + n)))
    for j in range(n - 1):                                  # crease: the middle node column
        els.append(mesh.Element(1, 5, (j * n + crease_col, (j + 1) * n + crease_col)))
    for j in range(n - 1):                                  # the edge x = 0
        els.append(mesh.Element(1, 2, (j * n, (j + 1) * n)))
    els.append(mesh.Element(15, 7, (0,)))
    return xy, els


def test_round_trip_and_quadrature(tmp_path):
    xy, els = grid_mesh()
    path = tmp_path / "grid.msh"
    mesh.write_msh41(path, xy, els)
    xy2, els2 = mesh.read_msh41(path)
    assert np.array_equal(xy2, xy) and [(e.type, e.entity_tag, e.nodes) for e in els2] == \
        [(e.type, e.entity_tag, e.nodes) for e in els]
    q = mesh.quadrature(xy2, els2, line_degree=1, face_degree=3)
    fxy, fw, _ = q["face"]
    ref = synth.quad_gauss_points(xy, 9, 9, 3)
    assert np.allclose(np.sort(fxy, axis=0), np.sort(ref.xy, axis=0), atol=1e-14)
    assert np.isclose(fw.sum(), 16.0) and np.isclose(ref.weight.sum(), 16.0)
    exy, ew, et, en, etag = q["edge"]
    assert len(exy) == 16 and np.allclose(ew, 0.5) and np.allclose(en, np.stack([-et[:, 1], et[:, 0]], 1))
    assert len(q["point"][0]) == 1 and len(q["active"]) == 81


def test_crease_extraction_and_plate(tmp_path):
    xy, els = grid_mesh()
    c = mesh.extract_curve(els, xy, [5])
    assert np.allclose(c["vertices"][:, 0], 2.0) and c["extend_start"] and c["extend_end"] and not c["is_closed"]
    path = tmp_path / "grid.msh"
    mesh.write_msh41(path, xy, els)
    p = mesh.plate_from_mesh(path, crease_tags=[5], rho=1.75)
    s = synth.square_plate(9, 0.5, 3, crease="row", rho_factor=3.5)
    assert np.array_equal(p.node_xy, s.node_xy)
    assert np.allclose(np.sort(p.faces.xy, axis=0), np.sort(s.faces.xy, axis=0), atol=1e-14)
    f, g = p.folds[0], s.folds[0]
    assert np.allclose(f.left.xy, g.left.xy, atol=1e-14) and np.allclose(f.left.weight, g.left.weight)


def test_support_radius_matches_brute_force():
    rng = np.random.default_rng(4)
    P = rng.uniform(0, 10, size=(400, 2))
    d = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    third = np.sort(d, axis=1)[:, 3]
    assert np.isclose(mesh.support_radius(P, 3), 6 * np.sort(third)[len(third) // 2])


def test_reader_rejects_bad_files(tmp_path):
    xy, els = grid_mesh(3, crease_col=1)
    good = tmp_path / "g.msh"
    mesh.write_msh41(good, xy, els)
    text = good.read_text()
    bad_type = tmp_path / "t.msh"
    bad_type.write_text(text.replace("\n2 1 3 4\n", "\n2 1 9 4\n"))
    with pytest.raises(mesh.MeshError, match="unsupported Gmsh element type 9"):
        mesh.read_msh41(bad_type)
    bad_tag = tmp_path / "n.msh"
    lines = text.split("\n")
    k = lines.index("$Elements") + 3
    lines[k] = lines[k].split()[0] + " 99 2 5 4"
    bad_tag.write_text("\n".join(lines))
    with pytest.raises(mesh.MeshError, match="undefined node tag 99"):
        mesh.read_msh41(bad_tag)


@pytest.mark.skipif(not os.path.exists(REF_MESH), reason="the reference's example meshes are not here")
def test_reference_example_mesh():
    xy, els = mesh.read_msh41(REF_MESH)
    q = mesh.quadrature(xy, els)
    assert len(q["face"][0]) > 0 and len(q["active"]) > 0
    c = mesh.extract_curve(els, xy, [5])
    assert c is not None and len(c["vertices"]) >= 2 and c["dropped"] == 0


def test_triangle_rules():
    # two triangles splitting the unit square: weights sum to the area, 1- and 3-point rules
    xy = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    els = [mesh.Element(2, 1, (0, 1, 2)), mesh.Element(2, 1, (0, 2, 3))]
    for degree, per in ((1, 1), (3, 3)):
        fxy, fw, _ = mesh.quadrature(xy, els, face_degree=degree)["face"]
        assert len(fxy) == 2 * per and np.isclose(fw.sum(), 1.0)
        # the rules integrate x exactly: int_0^1 int_0^1 x = 1/2
        assert np.isclose((fw * fxy[:, 0]).sum(), 0.5)
    fxy, fw, _ = mesh.quadrature(xy, els, face_degree=3)["face"]
    assert np.isclose((fw * fxy[:, 0] * fxy[:, 1]).sum(), 0.25)   # degree 2 exact


def test_clockwise_quad_has_positive_weights():
    xy = np.array([[0.0, 0.0], [0.0, 1.0], [1.0, 1.0], [1.0, 0.0]])   # clockwise
    fxy, fw, _ = mesh.quadrature(xy, [mesh.Element(3, 1, (0, 1, 2, 3))], face_degree=2)["face"]
    assert np.all(fw > 0) and np.isclose(fw.sum(), 1.0)
