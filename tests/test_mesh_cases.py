"""The reference's mesh test cases (tests/test_mesh.cpp) on the product's host-side sector mesh
(turbomodal_gb300.mesh.Mesh: gmsh v2 reader, cyclic boundary identification, node matching).

The wedge fixture is the reference's tests/test_data/wedge_sector.msh converted by
tests/golden/make_fixtures.py: an annular sector R = 0.05..0.15 m, 15 degrees, 0.01 m thick."""

import math

import numpy as np
import pytest

from conftest import load_fixture


@pytest.fixture(scope="module")
def wedge():
    return load_fixture("wedge_sector", 24)


def test_boundary_nodes_on_their_planes(wedge):
    """LeftBoundaryNodesAtThetaZero, RightBoundaryNodesAtThetaAlpha."""
    left = wedge.find_node_set("left_boundary").node_ids
    right = wedge.find_node_set("right_boundary").node_ids
    assert np.abs(wedge.nodes[left, 1]).max() <= 1e-10
    theta = np.arctan2(wedge.nodes[right, 1], wedge.nodes[right, 0])
    assert np.abs(theta - math.pi / 12).max() <= 1e-6


def test_matched_pairs_same_radius_same_z_unique(wedge):
    """MatchBoundaryNodes, MatchBoundaryNodesSameRadii, MatchBoundaryNodesSameZ,
    MatchBoundaryNodesUniquePairs."""
    pairs = np.asarray(wedge.matched_pairs)
    assert len(pairs) > 0
    X = wedge.nodes
    rl = np.hypot(X[pairs[:, 0], 0], X[pairs[:, 0], 1])
    rr = np.hypot(X[pairs[:, 1], 0], X[pairs[:, 1], 1])
    assert np.abs(rl - rr).max() <= 1e-8
    assert np.abs(X[pairs[:, 0], 2] - X[pairs[:, 1], 2]).max() <= 1e-10
    assert len(set(pairs[:, 0])) == len(pairs) and len(set(pairs[:, 1])) == len(pairs)


def test_boundary_errors(wedge):
    """IdentifyCyclicBoundariesThrowsWithoutGroups, MatchBoundaryNodesThrowsWithoutSectors,
    MatchBoundaryNodesThrowsWithoutIdentify."""
    from turbomodal_gb300.mesh import Mesh, NodeSet

    with pytest.raises(RuntimeError):
        Mesh().identify_cyclic_boundaries()
    m = Mesh()
    m.nodes, m.elements = wedge.nodes, wedge.elements
    m.node_sets = [NodeSet(s.name, list(s.node_ids)) for s in wedge.node_sets]
    m.identify_cyclic_boundaries()
    with pytest.raises(RuntimeError):
        m.match_boundary_nodes()          # num_sectors not set
    m2 = Mesh()
    m2.nodes, m2.elements, m2.node_sets, m2.num_sectors = wedge.nodes, wedge.elements, m.node_sets, 24
    with pytest.raises(RuntimeError):
        m2.match_boundary_nodes()         # boundaries not identified


def test_find_node_set(wedge):
    """FindNodeSetReturnsNullForMissing, FindNodeSetReturnsCorrectSet."""
    assert wedge.find_node_set("nonexistent") is None
    s = wedge.find_node_set("left_boundary")
    assert s is not None and s.name == "left_boundary" and len(s.node_ids) > 0


@pytest.mark.parametrize("header", [None, "4.1 0 8", "2.2 1 8"])
def test_loader_errors(tmp_path, header):
    """LoadThrowsForMissingFile, LoadThrowsForInvalidFormat, LoadThrowsForBinaryFormat."""
    from turbomodal_gb300.mesh import Mesh

    p = tmp_path / "m.msh"
    if header is not None:
        p.write_text("$MeshFormat\n" + header + "\n$EndMeshFormat\n")
    with pytest.raises(RuntimeError):
        Mesh().load_from_gmsh(str(p))


def test_loader_rejects_unknown_node(tmp_path):
    """An element naming a node the file does not define (src/mesh.cpp:131-134)."""
    from turbomodal_gb300.mesh import Mesh

    p = tmp_path / "m.msh"
    p.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n"
                 "$Elements\n1\n1 15 2 1 1 7\n$EndElements\n")
    with pytest.raises(RuntimeError):
        Mesh().load_from_gmsh(str(p))


def test_element_volumes_and_total_volume(oracle, wedge):
    """ElementVolumesPositive, TotalVolumeApproxCorrect: every corner tetrahedron has positive volume
    and the sector volume, from the consistent mass matrix (sum of its x-x block = rho V), is the
    annular-sector volume within 5 %."""
    from turbomodal_gb300.meshgen import Material

    X = wedge.nodes[wedge.elements[:, :4]]
    vol = np.einsum("ij,ij->i", np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), X[:, 3] - X[:, 0]) / 6
    assert np.all(vol > 0)
    rho = 7850.0
    M = oracle.OracleModel(wedge, Material(200e9, 0.3, rho)).matrix("M").tocoo()
    sel = (M.row % 3 == 0) & (M.col % 3 == 0)
    V = M.data[sel].sum() / rho
    V_ref = 0.5 * (0.15 ** 2 - 0.05 ** 2) * (math.pi / 12) * 0.01
    assert abs(V - V_ref) <= 0.05 * V_ref


def _match(mesh_factory, brute, monkeypatch):
    import turbomodal_gb300.mesh as tm

    monkeypatch.setattr(tm, "KDTREE_MIN_RIGHT", 10 ** 9 if brute else 0)
    m = mesh_factory()
    return m.matched_pairs, m.free_boundary, m.left_boundary, m.right_boundary


@pytest.mark.parametrize("case", ["wedge", "blade", "config1", "perturbed"])
def test_kdtree_matching_equals_full_scan(case, monkeypatch):
    """The k-d tree candidate search gives the pairs, the free boundary and the boundary lists of
    the reference's full scan (src/mesh.cpp:260-351), also with near-ties and with nodes moved
    beyond the tolerance."""
    from turbomodal_gb300.mesh import Mesh, NodeSet
    from turbomodal_gb300.meshgen import config_mesh

    def factory():
        if case == "wedge":
            return load_fixture("wedge_sector", 24)
        if case == "blade":
            return load_fixture("blade_sector", 24)
        base = config_mesh(1) if case == "config1" else load_fixture("leissa_disk_sector", 24)
        if case == "config1":
            return base
        # perturbed copy: right-boundary nodes moved by 0.3x / 3x the tolerance, some duplicated
        # positions (ties) added as extra right nodes
        rng = np.random.default_rng(5)
        m = Mesh()
        X = base.nodes.copy()
        right = list(base.find_node_set("right_boundary").node_ids)
        left = list(base.find_node_set("left_boundary").node_ids)
        for i, nid in enumerate(right):
            r = math.hypot(X[nid, 0], X[nid, 1])
            tol = max(1e-6, 1e-4 * r)
            X[nid] += rng.standard_normal(3) * (0.3 if i % 3 else 3.0) * tol / math.sqrt(3)
        dup = right[::7]
        X = np.vstack([X, X[dup]])
        extra = list(range(len(base.nodes), len(base.nodes) + len(dup)))
        sets = [NodeSet(s.name, list(s.node_ids)) for s in base.node_sets if s.name not in ("left_boundary",
                                                                                           "right_boundary")]
        sets += [NodeSet("left_boundary", left), NodeSet("right_boundary", right + extra)]
        m.load_from_arrays(X, base.elements, sets, 24)
        return m

    full, tree = _match(factory, True, monkeypatch), _match(factory, False, monkeypatch)
    assert full == tree and len(full[0]) > 0
    if case == "perturbed":
        assert len(full[1]) > 0          # some nodes moved beyond the tolerance stay free
