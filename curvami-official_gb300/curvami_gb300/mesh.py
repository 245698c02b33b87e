"""Mesh input: Gmsh msh 4.1 files to Gauss points, nodes and creases.

The reference feeds the hot path from Gmsh meshes; this module restates that front end so
the same meshes drive the GPU path:

  * ``read_msh41`` = GmshReader::readMesh (core/include/curvami/GmshReader.h:32-147): the
    $Nodes and $Elements blocks of an ASCII msh 4.1 file, node tags mapped to indices in
    file order, element types 15 (point), 1 (line), 2 (triangle), 3 (quadrangle); an
    unknown type or an undefined node tag rejects the file;
  * ``quadrature`` = Quadrature::generate (core/include/curvami/Quadrature.h:60-233): one
    Gauss point per point element, a 1- or 3-point rule per line (tangent, normal = the
    tangent turned by +90 degrees), a 1- or 3-point rule per triangle, a tensor 1/2/3-point
    rule per quadrangle with |det J|; the active nodes are the nodes of face elements, in
    index order;
  * ``extract_curve`` = MeshUtils::extractCurve (MeshUtils.h:57-143): the line elements of
    the given tags walked into one polyline, closed loops detected, ends on the convex hull
    flagged for extension;
  * ``support_radius`` = MeshUtils::computeSupportRadius (MeshUtils.h:144-209): (order + 3)
    times the median distance to the third-nearest other node;
  * ``plate_from_mesh`` assembles these into a ``synth.Plate`` (faces split on the creases,
    one fold per crease tag from that tag's line Gauss points, SetupHelper.h / main.cpp).
A writer (``write_msh41``) produces files the reader accepts, for synthetic meshes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import synth

NODES_PER_TYPE = {15: 1, 1: 2, 2: 3, 3: 4}


class MeshError(ValueError):
    pass


@dataclass
class Element:
    type: int
    entity_tag: int
    nodes: tuple


def read_msh41(path):
    """(node_xy (n, 2) in file order, [Element]) of an ASCII msh 4.1 file."""
    with open(path) as f:
        lines = f.read().split("\n")
    xy, elements, tag_to_index = [], [], {}
    i = 0
    while i < len(lines):
        line = lines[i]
        if "$Nodes" in line and "$EndNodes" not in line:
            i += 1
            vals = []
            while "$EndNodes" not in lines[i]:
                vals.extend(lines[i].split())
                i += 1
            it = iter(vals)
            n_blocks, n_nodes = int(next(it)), int(next(it))
            next(it); next(it)
            for _ in range(n_blocks):
                next(it); next(it); next(it)          # entity dim, entity tag, parametric
                nb = int(next(it))
                tags = [int(next(it)) for _ in range(nb)]
                for t in tags:
                    x, y = float(next(it)), float(next(it))
                    next(it)                          # z: the plate lies in the plane
                    tag_to_index[t] = len(xy)
                    xy.append((x, y))
        elif "$Elements" in line and "$EndElements" not in line:
            i += 1
            vals = []
            while "$EndElements" not in lines[i]:
                vals.extend(lines[i].split())
                i += 1
            it = iter(vals)
            n_blocks = int(next(it))
            next(it); next(it); next(it)
            for _ in range(n_blocks):
                next(it)                              # entity dim
                etag, etype, ne = int(next(it)), int(next(it)), int(next(it))
                k = NODES_PER_TYPE.get(etype, 0)
                if k == 0:
                    raise MeshError(f"unsupported Gmsh element type {etype} in {path}; cannot determine its "
                                    "node count, aborting mesh read.")
                for _ in range(ne):
                    next(it)                          # element tag
                    idx = []
                    for _ in range(k):
                        t = int(next(it))
                        if t not in tag_to_index:
                            raise MeshError(f"element references undefined node tag {t} in {path}")
                        idx.append(tag_to_index[t])
                    elements.append(Element(etype, etag, tuple(idx)))
        i += 1
    if not xy or not elements:
        raise MeshError(f"{path} yielded {len(xy)} nodes and {len(elements)} elements; the file is empty or malformed.")
    return np.asarray(xy, np.float64), elements


def write_msh41(path, node_xy, elements):
    """An ASCII msh 4.1 file: one node block, one element block per (type, entity tag)."""
    node_xy = np.asarray(node_xy, np.float64)
    n = len(node_xy)
    groups = {}
    for el in elements:
        groups.setdefault((el.type, el.entity_tag), []).append(el)
    dims = {15: 0, 1: 1, 2: 2, 3: 2}
    with open(path, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
        f.write(f"$Nodes\n1 {n} 1 {n}\n2 1 0 {n}\n")
        f.write("".join(f"{k + 1}\n" for k in range(n)))
        f.write("".join(f"{x:.17g} {y:.17g} 0\n" for x, y in node_xy))
        f.write("$EndNodes\n")
        f.write(f"$Elements\n{len(groups)} {len(elements)} 1 {len(elements)}\n")
        tag = 1
        for (etype, etag), els in groups.items():
            f.write(f"{dims[etype]} {etag} {etype} {len(els)}\n")
            for el in els:
                f.write(f"{tag} " + " ".join(str(v + 1) for v in el.nodes) + "\n")
                tag += 1
        f.write("$EndElements\n")


def _line_rule(degree):
    if degree <= 1:
        return np.array([0.0]), np.array([2.0])
    a = math.sqrt(3.0 / 5.0)
    return np.array([-a, 0.0, a]), np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])


def _quad_rule(degree):
    if degree <= 1:
        return np.array([0.0]), np.array([2.0])
    if degree == 2:
        a = 1.0 / math.sqrt(3.0)
        return np.array([-a, a]), np.array([1.0, 1.0])
    a = math.sqrt(3.0 / 5.0)
    return np.array([-a, 0.0, a]), np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])


def _tri_rule(degree):
    if degree <= 1:
        return [(1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 1.0)]
    return [(2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 1.0 / 3.0), (1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 3.0),
            (1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0)]


def quadrature(node_xy, elements, line_degree=1, face_degree=3):
    """Gauss points of every element, in element order: {"active": raw indices of the face
    nodes (ascending), "face": (xy, weight, tag), "edge": (xy, weight, tangent, normal, tag),
    "point": (xy, weight, tag)}."""
    P = np.asarray(node_xy, np.float64)
    lp, lw = _line_rule(line_degree)
    qp, qw = _quad_rule(face_degree)
    tri = _tri_rule(face_degree)
    face, edge, point = ([], [], []), ([], [], [], [], []), ([], [], [])
    active = set()
    for el in elements:
        if el.type == 15 and len(el.nodes) == 1:
            point[0].append(P[el.nodes[0]]); point[1].append(1.0); point[2].append(el.entity_tag)
        elif el.type == 1 and len(el.nodes) == 2:
            p1, p2 = P[el.nodes[0]], P[el.nodes[1]]
            t = p2 - p1
            L = float(np.hypot(*t))
            if not L > 0.0:
                continue
            t = t / L
            nrm = np.array([-t[1], t[0]])
            for x, w in zip(lp, lw):
                edge[0].append(0.5 * (1.0 - x) * p1 + 0.5 * (1.0 + x) * p2)
                edge[1].append(0.5 * L * w); edge[2].append(t); edge[3].append(nrm); edge[4].append(el.entity_tag)
        elif el.type == 2 and len(el.nodes) == 3:
            p1, p2, p3 = P[list(el.nodes)]
            area = 0.5 * abs(p1[0] * (p2[1] - p3[1]) + p2[0] * (p3[1] - p1[1]) + p3[0] * (p1[1] - p2[1]))
            for u, v, w, wt in tri:
                face[0].append(u * p1 + v * p2 + w * p3); face[1].append(area * wt); face[2].append(el.entity_tag)
            active.update(el.nodes)
        elif el.type == 3 and len(el.nodes) == 4:
            p = P[list(el.nodes)]
            active.update(el.nodes)
            for xi, wx in zip(qp, qw):
                for eta, wy in zip(qp, qw):
                    N = 0.25 * np.array([(1 - xi) * (1 - eta), (1 + xi) * (1 - eta), (1 + xi) * (1 + eta),
                                         (1 - xi) * (1 + eta)])
                    dxi = 0.25 * np.array([-(1 - eta), (1 - eta), (1 + eta), -(1 + eta)])
                    deta = 0.25 * np.array([-(1 - xi), -(1 + xi), (1 + xi), (1 - xi)])
                    J11, J12 = dxi @ p[:, 0], dxi @ p[:, 1]
                    J21, J22 = deta @ p[:, 0], deta @ p[:, 1]
                    face[0].append(N @ p); face[1].append(abs(J11 * J22 - J12 * J21) * wx * wy)
                    face[2].append(el.entity_tag)

    return {
        "active": np.array(sorted(active), np.int64),
        "face": (np.asarray(face[0], np.float64).reshape(-1, 2), np.asarray(face[1], np.float64),
                 np.asarray(face[2], np.int64)),
        "edge": (np.asarray(edge[0], np.float64).reshape(-1, 2), np.asarray(edge[1], np.float64),
                 np.asarray(edge[2], np.float64).reshape(-1, 2), np.asarray(edge[3], np.float64).reshape(-1, 2),
                 np.asarray(edge[4], np.int64)),
        "point": (np.asarray(point[0], np.float64).reshape(-1, 2), np.asarray(point[1], np.float64),
                  np.asarray(point[2], np.int64)),
    }


def extract_curve(elements, node_xy, tags):
    """The crease polyline of the line elements whose entity tag is in `tags`; None if none."""
    tags = set(int(t) for t in tags)
    adj = {}
    for el in elements:
        if el.type == 1 and el.entity_tag in tags:
            a, b = el.nodes
            adj.setdefault(a, []).append(b)
            adj.setdefault(b, []).append(a)
    if not adj:
        return None
    keys = sorted(adj)
    start = next((k for k in keys if len(adj[k]) == 1), keys[0])
    order, prev, cur, closed = [], -1, start, False
    while True:
        order.append(cur)
        nxt = next((nb for nb in adj[cur] if nb != prev), -1)
        if nxt == -1 or nxt == start:
            closed = nxt == start
            break
        prev, cur = cur, nxt
    P = np.asarray(node_xy, np.float64)
    verts = P[order]
    if closed:
        verts = np.vstack([verts, verts[:1]])
    hull = synth.convex_hull(P)
    return {"vertices": verts, "extend_start": synth.on_hull_boundary(P[order[0]], hull),
            "extend_end": synth.on_hull_boundary(P[order[-1]], hull), "is_closed": closed,
            "dropped": len(adj) - len(order)}


def support_radius(node_xy, order):
    """(order + 3) x the median over nodes of the distance to the third-nearest other node."""
    from scipy.spatial import cKDTree

    P = np.asarray(node_xy, np.float64)
    if len(P) < 4:
        return 0.1
    d, _ = cKDTree(P).query(P, k=4)
    h = np.sort(d[:, 3])
    return (order + 3) * h[len(h) // 2]


def plate_from_mesh(path, crease_tags=(), Kt=1e-3, order=2, kernel=0, rho=None, line_degree=1, face_degree=3,
                    E=1.0, nu=0.3, thickness=0.05, theta0=0.0, cuts=None, rigid=False):
    """A synth.Plate from a msh 4.1 file (plate_from_elements of its nodes and elements)."""
    xy, elements = read_msh41(path)
    return plate_from_elements(xy, elements, crease_tags, Kt, order, kernel, rho, line_degree, face_degree, E, nu,
                               thickness, theta0, cuts, rigid, name=str(path))


def plate_from_elements(xy, elements, crease_tags=(), Kt=1e-3, order=2, kernel=0, rho=None, line_degree=1,
                        face_degree=3, E=1.0, nu=0.3, thickness=0.05, theta0=0.0, cuts=None, rigid=False,
                        name="mesh"):
    """A synth.Plate from mesh nodes and elements: the active nodes, the face Gauss points
    split on the creases, one fold per tag in `crease_tags` from that tag's line Gauss points
    (Kt, theta0 and rigid: one value for every fold or one per tag), rho from support_radius
    (order 3, as main.cpp does) unless given. The crease curves that cut the supports are
    `cuts` (lists of tags, each walked into one curve: main.cpp:171-176) or, without it, one
    curve per crease tag (main.cpp:177-184)."""
    xy = np.asarray(xy, np.float64)
    q = quadrature(xy, elements, line_degree, face_degree)
    active = q["active"]
    nodes = xy[active]
    tags = [int(t) for t in crease_tags]

    def per_tag(v, what):
        if np.ndim(v) == 0:
            return [v] * len(tags)
        if len(v) != len(tags):
            raise MeshError(f"{what}: one value per crease tag expected")
        return list(v)

    Kts, th0s, rigids = per_tag(Kt, "Kt"), per_tag(theta0, "theta0"), per_tag(rigid, "rigid")
    creases, folds = [], []
    exy, ew, et, en, etag = q["edge"]
    for tag, kt, th, rg in zip(tags, Kts, th0s, rigids):
        sel = etag == tag
        if not np.any(sel):
            raise MeshError(f"no line elements with entity tag {tag} in {name}")
        s = 1e-7
        L = synth.PointSet(exy[sel] + s * en[sel], ew[sel].copy(), et[sel].copy())
        R = synth.PointSet(exy[sel] - s * en[sel], ew[sel].copy(), et[sel].copy())
        folds.append(synth.Fold(L, R, float(kt), float(th), bool(rg)))
    for cut in (cuts if cuts is not None else [[t] for t in tags]):
        c = extract_curve(elements, xy, [int(t) for t in cut])
        if c is None:
            raise MeshError(f"no line elements with entity tags {list(cut)} in {name}")
        creases.append({k: c[k] for k in ("vertices", "extend_start", "extend_end", "is_closed")})
    fxy, fw, _ = q["face"]
    faces, nsplit = synth.split_on_creases(synth.PointSet(fxy, fw), creases)
    r = support_radius(nodes, 3) if rho is None else float(rho)
    pxy, pw, ptag = q["point"]
    points = {int(t): synth.PointSet(pxy[ptag == t], pw[ptag == t]) for t in sorted(set(ptag.tolist()))}
    edges = {int(t): (exy[etag == t], ew[etag == t], et[etag == t], en[etag == t]) for t in sorted(set(etag.tolist()))}
    return synth.Plate(name=name, node_xy=nodes, faces=faces, creases=creases, folds=folds, rho=r,
                       order=order, kernel=kernel, E=E, nu=nu, thickness=thickness,
                       meta={"mesh": name, "split": nsplit, "elements": len(elements), "edges": edges},
                       points=points)


def centre_crease_sheet(n_cells=20, half=1.0, crease_half=0.5, crease_segments=10, crease_tag=5):
    """Nodes and elements of a square sheet [-half, half]^2 of n_cells x n_cells quadrangles
    (entity 1) with a crease line (-crease_half, 0) -> (crease_half, 0) of its own nodes,
    one line element per segment (entity `crease_tag`), and point elements at the corners
    (-half, -half), (half, -half), (-half, half) with entity tags 1, 2, 4: the layout of the
    reference's centre-crease benchmark meshes (a transfinite, recombined square and a
    crease that is not embedded in it). Returns (node_xy, [Element])."""
    m = n_cells + 1
    t = np.linspace(-half, half, m)
    X, Y = np.meshgrid(t, t)                     # node (i, j) at index j * m + i
    grid = np.stack([X.ravel(), Y.ravel()], axis=1)
    c = np.stack([np.linspace(-crease_half, crease_half, crease_segments + 1),
                  np.zeros(crease_segments + 1)], axis=1)
    node_xy = np.vstack([grid, c])
    els = []
    for j in range(n_cells):
        for i in range(n_cells):
            a = j * m + i
            els.append(Element(3, 1, (a, a + 1, a + m + 1, a + m)))
    base = m * m
    for k in range(crease_segments):
        els.append(Element(1, crease_tag, (base + k, base + k + 1)))
    els.append(Element(15, 1, (0,)))
    els.append(Element(15, 2, (m - 1,)))
    els.append(Element(15, 4, ((m - 1) * m,)))
    return node_xy, els
