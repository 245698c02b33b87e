"""Makes the fixtures of the square-twist case (run here, where the reference tree is present;
the GPU machine only reads the results):

  fourvertex_st61_mesh.npz   the nodes and elements of the reference's example mesh
      examples/fourvertex/SquareTwistFiner.msh (61 x 61 background grid, four creases of
      29 segments tagged T = 6, R = 5, B = 8, L = 7, point elements tagged 1, 2, 4), as read by
      curvami_gb300.mesh.read_msh41: node_xy, and per element its type, entity tag and nodes
      (el_ptr / el_nodes);
  fourvertex_st61_trbl.json  the run configuration examples/fourvertex/
      ST-nx61nf30-TRBL-Kt5-p0.json (TargetDirectedArcLength, all four creases driven, Kt = 5),
      without its output path.

Usage: python tests/golden/make_fourvertex.py [path/to/reference]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "curvami-official_gb300"))

from curvami_gb300 import mesh  # noqa: E402


def main(ref_root):
    ex = os.path.join(ref_root, "examples", "fourvertex")
    xy, els = mesh.read_msh41(os.path.join(ex, "SquareTwistFiner.msh"))
    ptr = np.zeros(len(els) + 1, np.int64)
    ptr[1:] = np.cumsum([len(e.nodes) for e in els])
    nodes = np.fromiter((n for e in els for n in e.nodes), np.int32, count=int(ptr[-1]))
    np.savez_compressed(os.path.join(HERE, "fourvertex_st61_mesh.npz"), node_xy=xy,
                        el_type=np.array([e.type for e in els], np.int16),
                        el_tag=np.array([e.entity_tag for e in els], np.int32), el_ptr=ptr, el_nodes=nodes)
    with open(os.path.join(ex, "ST-nx61nf30-TRBL-Kt5-p0.json")) as f:
        cfg = json.load(f)
    cfg.pop("output_file", None)
    cfg["source"] = "examples/fourvertex/ST-nx61nf30-TRBL-Kt5-p0.json of the reference"
    with open(os.path.join(HERE, "fourvertex_st61_trbl.json"), "w") as f:
        json.dump(cfg, f, indent=1)
    print(len(xy), "nodes,", len(els), "elements")


def load():
    """(config dict, node_xy, [mesh.Element]) from the fixtures."""
    with open(os.path.join(HERE, "fourvertex_st61_trbl.json")) as f:
        cfg = json.load(f)
    z = np.load(os.path.join(HERE, "fourvertex_st61_mesh.npz"))
    ptr, nodes = z["el_ptr"], z["el_nodes"]
    els = [mesh.Element(int(t), int(g), tuple(int(v) for v in nodes[ptr[i]:ptr[i + 1]]))
           for i, (t, g) in enumerate(zip(z["el_type"], z["el_tag"]))]
    return cfg, z["node_xy"], els


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CURVAMI_REFERENCE")
    if not root:
        sys.exit("usage: make_fourvertex.py <reference root> (or set CURVAMI_REFERENCE)")
    main(root)
