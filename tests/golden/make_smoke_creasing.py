"""Makes the fixtures of the progressive-creasing smoke case (run here, where the reference
tree is present; the GPU machine only reads the results):

  smoke_centre_crease_nodes.npy  the node coordinates of the reference's example mesh
      examples/smoke_centre_crease/CB_n20.msh (written by gmsh from CB_n20.geo), in the node
      order of curvami_gb300.mesh.centre_crease_sheet(). The coordinates matter beyond their
      nominal values: gmsh leaves the sheet nodes of the row y = 0 at y = +-k 2.75e-13, and
      which side of the crease a node on the crease line takes (Enrichment.h:64-67, the 1e-12
      validity distance and the sign of f) follows from those last bits. On the ideal grid the
      step energies differ by up to 6 %.
  smoke_centre_crease.json  the published last-step row (examples/smoke_centre_crease/
      README.md:14-20) and every step of the oracle's run of the same case on these nodes
      (the oracle's run reproduces the published row to its printed digits).

Usage: python tests/golden/make_smoke_creasing.py [path/to/reference]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "curvami-official_gb300"))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from curvami_gb300 import creasing as PC  # noqa: E402
from curvami_gb300 import mesh  # noqa: E402


def reference_sheet_nodes(msh_path, n_cells):
    """The node coordinates of one of the reference's centre-crease meshes (written by gmsh), in
    the node order of curvami_gb300.mesh.centre_crease_sheet(n_cells)."""
    from scipy.spatial import cKDTree

    rxy, _ = mesh.read_msh41(msh_path)
    ideal, _ = mesh.centre_crease_sheet(n_cells=n_cells, crease_segments=n_cells // 2)
    # Crease-line nodes and sheet nodes coincide in position; match each kind separately
    # (the last n_cells / 2 + 1 generator nodes are the crease line's own nodes).
    out = np.empty_like(ideal)
    n_sheet = len(ideal) - (n_cells // 2 + 1)
    used = set()
    tree = cKDTree(rxy)
    for i, p in enumerate(ideal):
        cand = tree.query_ball_point(p, 1e-9)
        cand = [c for c in cand if c not in used]
        if not cand:
            raise SystemExit(f"no reference node near {p}")
        # sheet nodes come first in the generator; gmsh lists the crease curve's nodes
        # (its end points and interior) before the surface's interior nodes, so for a
        # position shared by both take the later gmsh node for the sheet.
        c = max(cand) if i < n_sheet else min(cand)
        used.add(c)
        out[i] = rxy[c]
    return out


def main(ref_root):
    src = os.path.join(ref_root, "examples", "smoke_centre_crease", "CB_n20.msh")
    out = reference_sheet_nodes(src, 20)
    np.save(os.path.join(HERE, "smoke_centre_crease_nodes.npy"), out)

    import creasing_helpers as H
    from oracle.binding import Oracle

    o = Oracle(native=False)
    p, spec = H.smoke_plate(os.path.join("/tmp", "smoke_centre_crease_fixture.msh"))
    plate = H.OracleCreasingPlate(o, p, spec, H.point_bcs())
    x = np.zeros(3 * len(p.node_xy))
    res = PC.run(H.smoke_solver(), plate, x, [H.smoke_line(p)], cfg=H.smoke_config())
    keys = ("step", "a", "b", "newton_iters", "E_mem", "E_ben", "E_hin", "theta_mean_deg", "theta_max_deg",
            "jump_over_L", "change_over_L")
    doc = {
        "source": "examples/smoke_centre_crease (smoke.json, CB_n20.msh, README.md:14-20) of the reference",
        "published_last_step": H.GOLDEN_LAST_STEP,
        "oracle_steps": [{k: r[k] for k in keys} for r in res.steps],
        "stopped": res.stopped,
    }
    with open(os.path.join(HERE, "smoke_centre_crease.json"), "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(doc["oracle_steps"][-1]))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CURVAMI_REFERENCE")
    if not root:
        sys.exit("usage: make_smoke_creasing.py <reference root> (or set CURVAMI_REFERENCE)")
    main(root)
