"""Regenerate the committed mesh fixtures from the turbomodal test meshes.

Reads the reference project's own gmsh v2 test meshes (tests/test_data/*.msh in the
turbomodal tree) with this package's gmsh reader and stores nodes, TET10 connectivity
and node sets as compressed .npz files next to this script, so the tests do not need the
reference tree at run time.  Usage:  python tests/golden/make_fixtures.py <turbomodal root>
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from turbomodal_gb300.mesh import Mesh  # noqa: E402

MESHES = {"leissa_disk_sector": 24, "wedge_sector": 24, "blade_sector": 24}


def main(root: str) -> None:
    for name in MESHES:
        m = Mesh()
        m.load_from_gmsh(os.path.join(root, "tests", "test_data", name + ".msh"))
        sets = {f"set_{ns.name}": np.asarray(ns.node_ids, dtype=np.int32) for ns in m.node_sets}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), nodes=m.nodes, elements=m.elements, **sets)
        print(name, m.num_nodes(), m.num_elements(), sorted(sets))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <turbomodal source root>")
    main(sys.argv[1])
