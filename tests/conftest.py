import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def load_fixture(name: str, num_sectors: int = 24):
    """Mesh fixture converted from the reference's test_data (see tests/golden/make_fixtures.py),
    set up as the reference tests do: num_sectors, identify boundaries, match nodes."""
    from turbomodal_gb300.mesh import Mesh, NodeSet

    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = Mesh()
    m.nodes = d["nodes"]
    m.elements = d["elements"]
    m.node_sets = [NodeSet(k[4:], d[k].tolist()) for k in sorted(d.files) if k.startswith("set_")]
    m.num_sectors = num_sectors
    m.identify_cyclic_boundaries()
    m.match_boundary_nodes()
    return m


@pytest.fixture(scope="session")
def oracle():
    from oracle import orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def cfg0_mesh():
    from turbomodal_gb300.meshgen import config_mesh

    return config_mesh(0)


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
