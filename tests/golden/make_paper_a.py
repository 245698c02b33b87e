"""Makes the fixture of the Paper A centre-crease case (run here, where the reference tree is
present; the GPU machine only reads the result):

  paper_a_cb_n80_nodes.npy  the node coordinates of examples/paperA_centre_crease/CB_n80.msh
      (written by gmsh from CB_n80.geo: 80 x 80 cells, the crease line's 41 nodes) in the node
      order of curvami_gb300.mesh.centre_crease_sheet(80). As for the smoke case, the last bits
      of the crease-row coordinates decide on which side of the cut those nodes fall.

The run configuration (examples/paperA_centre_crease/CB_n80_t0.5_xi10.json) differs from the
smoke case's only in the mesh, the hinge stiffness (xi = 10: Kt = 10 D = 10.989...) and its
j_integral objects; tests/creasing_helpers.py restates it.

Usage: python tests/golden/make_paper_a.py [path/to/reference]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_smoke_creasing import reference_sheet_nodes  # noqa: E402


def main(ref_root):
    src = os.path.join(ref_root, "examples", "paperA_centre_crease", "CB_n80.msh")
    out = reference_sheet_nodes(src, 80)
    np.save(os.path.join(HERE, "paper_a_cb_n80_nodes.npy"), out)
    print(out.shape)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CURVAMI_REFERENCE")
    if not root:
        sys.exit("usage: make_paper_a.py <reference root> (or set CURVAMI_REFERENCE)")
    main(root)
