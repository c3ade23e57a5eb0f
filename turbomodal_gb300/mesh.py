"""Sector mesh: TET10 nodes/elements, node sets and cyclic boundary matching.

Mirrors the reference ``Mesh`` (include/turbomodal/mesh.hpp:40-104): the same
fields (``nodes``, ``elements``, ``node_sets``, ``left_boundary``,
``right_boundary``, ``matched_pairs``, ``free_boundary``, ``num_sectors``,
``rotation_axis``) and the same set-up steps.  The mesh is an input producer
for the modal solve; it carries no device state.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class NodeSet:
    """Named node group (include/turbomodal/mesh.hpp:10-13)."""

    name: str
    node_ids: list


_GMSH_NODE_COUNT = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 8: 3, 9: 6, 11: 10, 15: 1}
KDTREE_MIN_RIGHT = 64   # right-boundary size above which matching queries a k-d tree


class Mesh:
    """TET10 sector mesh with cyclic-symmetry boundary data."""

    def __init__(self):
        self.nodes = np.zeros((0, 3), dtype=np.float64)
        self.elements = np.zeros((0, 10), dtype=np.int32)
        self.node_sets: list[NodeSet] = []
        self.left_boundary: list[int] = []
        self.right_boundary: list[int] = []
        self.matched_pairs: list[tuple[int, int]] = []
        self.free_boundary: list[int] = []
        self.num_sectors = 0
        self.rotation_axis = 2

    # --- sizes (mesh.hpp:100-102) -------------------------------------
    def num_nodes(self) -> int:
        return int(self.nodes.shape[0])

    def num_elements(self) -> int:
        return int(self.elements.shape[0])

    def num_dof(self) -> int:
        return 3 * self.num_nodes()

    def find_node_set(self, name: str):
        """First node set with this name, else None (mesh.cpp:353-360)."""
        for ns in self.node_sets:
            if ns.name == name:
                return ns
        return None

    # --- construction --------------------------------------------------
    def load_from_arrays(self, node_coords, element_connectivity, node_sets_in,
                         num_sectors_in: int, rotation_axis_in: int = 2) -> None:
        """Set geometry and run boundary identification + matching (mesh.cpp:208-229)."""
        node_coords = np.ascontiguousarray(node_coords, dtype=np.float64)
        element_connectivity = np.ascontiguousarray(element_connectivity, dtype=np.int32)
        if node_coords.ndim != 2 or node_coords.shape[1] != 3:
            raise RuntimeError("node_coords must have 3 columns (x, y, z)")
        if element_connectivity.ndim != 2 or element_connectivity.shape[1] != 10:
            raise RuntimeError("element_connectivity must have 10 columns (TET10)")
        if rotation_axis_in < 0 or rotation_axis_in > 2:
            raise RuntimeError("rotation_axis must be 0 (X), 1 (Y), or 2 (Z)")
        self.nodes = node_coords
        self.elements = element_connectivity
        self.node_sets = [NodeSet(ns.name, list(ns.node_ids)) for ns in node_sets_in]
        self.num_sectors = int(num_sectors_in)
        self.rotation_axis = int(rotation_axis_in)
        self.identify_cyclic_boundaries()
        self.match_boundary_nodes()

    def load_from_gmsh(self, filename: str) -> None:
        """Gmsh v2 ASCII reader with the reference's TET10 node-8/9 detection (mesh.cpp:30-206)."""
        physical_names = {}
        node_list = []
        gmsh_to_local = {}
        tets = []
        node_set_map: dict[str, set] = {}
        try:
            with open(filename, "r") as fh:
                lines = [ln.rstrip("\r\n") for ln in fh]
        except OSError:
            raise RuntimeError(f"Cannot open mesh file: {filename}") from None
        i = 0
        while i < len(lines):
            line = lines[i]
            if line == "$MeshFormat":
                ver, ftype, _ = lines[i + 1].split()[:3]
                if not (2.0 <= float(ver) < 3.0):
                    raise RuntimeError(f"Unsupported Gmsh format version: {ver}. Only v2.x supported.")
                if int(ftype) != 0:
                    raise RuntimeError("Only ASCII Gmsh files supported (file-type must be 0).")
                i += 3
                continue
            if line == "$PhysicalNames":
                cnt = int(lines[i + 1])
                for k in range(cnt):
                    parts = lines[i + 2 + k].split()
                    dim, tag, name = int(parts[0]), int(parts[1]), parts[2].strip('"')
                    physical_names[tag] = (dim, name)
                i += 3 + cnt
                continue
            if line == "$Nodes":
                cnt = int(lines[i + 1])
                for k in range(cnt):
                    parts = lines[i + 2 + k].split()
                    gmsh_to_local[int(parts[0])] = len(node_list)
                    node_list.append([float(parts[1]), float(parts[2]), float(parts[3])])
                i += 3 + cnt
                continue
            if line == "$Elements":
                cnt = int(lines[i + 1])
                for k in range(cnt):
                    parts = [int(p) for p in lines[i + 2 + k].split()]
                    etype, ntags = parts[1], parts[2]
                    tags = parts[3:3 + ntags]
                    phys = tags[0] if ntags > 0 else -1
                    nn = _GMSH_NODE_COUNT.get(etype, -1)
                    if nn < 0:
                        raise RuntimeError(f"Unknown Gmsh element type: {etype}")
                    enodes = []
                    for g in parts[3 + ntags:3 + ntags + nn]:
                        if g not in gmsh_to_local:
                            raise RuntimeError(f"Element references unknown node ID: {g}")
                        enodes.append(gmsh_to_local[g])
                    if etype == 11:
                        p = np.asarray(node_list, dtype=np.float64)
                        mid13 = 0.5 * (p[enodes[1]] + p[enodes[3]])
                        mid23 = 0.5 * (p[enodes[2]] + p[enodes[3]])
                        d13 = float(np.sum((p[enodes[8]] - mid13) ** 2))
                        d23 = float(np.sum((p[enodes[8]] - mid23) ** 2))
                        if d23 < d13:
                            enodes[8], enodes[9] = enodes[9], enodes[8]
                        tets.append(enodes)
                    if phys > 0 and phys in physical_names:
                        node_set_map.setdefault(physical_names[phys][1], set()).update(enodes)
                i += 3 + cnt
                continue
            i += 1
        self.nodes = np.asarray(node_list, dtype=np.float64).reshape(-1, 3)
        self.elements = np.asarray(tets, dtype=np.int32).reshape(-1, 10)
        self.node_sets = [NodeSet(name, sorted(ids)) for name, ids in sorted(node_set_map.items())]

    def identify_cyclic_boundaries(self) -> None:
        """Read left/right/free node sets (mesh.cpp:231-258)."""
        left = self.find_node_set("left_boundary")
        right = self.find_node_set("right_boundary")
        if left is None or right is None:
            raise RuntimeError("Mesh must have physical groups named 'left_boundary' and "
                               "'right_boundary' for cyclic symmetry.")
        self.left_boundary = list(left.node_ids)
        self.right_boundary = list(right.node_ids)
        free = self.find_node_set("free_boundary")
        self.free_boundary = list(free.node_ids) if free is not None else []

    def match_boundary_nodes(self) -> None:
        """Greedy nearest-partner matching of left and rotated-back right nodes (mesh.cpp:260-351).

        Left nodes are visited in order; each takes the closest unused right node
        (first index wins ties, as the reference's strict ``<``).  Pairs farther
        apart than max(1e-6, 1e-4 * r_left) leave both nodes on the free boundary.
        The reference scans every right node per left node, O(L R); above 64 right
        nodes the candidates come from a k-d tree ball query with the same result.
        """
        if self.num_sectors <= 0:
            raise RuntimeError("num_sectors must be set before matching boundary nodes.")
        if not self.left_boundary or not self.right_boundary:
            raise RuntimeError("Call identify_cyclic_boundaries() before match_boundary_nodes().")
        alpha = 2.0 * math.pi / self.num_sectors
        cos_a, sin_a = math.cos(-alpha), math.sin(-alpha)
        c1, c2, cax = {0: (1, 2, 0), 1: (0, 2, 1)}.get(self.rotation_axis, (0, 1, 2))
        right = np.asarray(self.right_boundary, dtype=np.int64)
        r1 = self.nodes[right, c1]
        r2 = self.nodes[right, c2]
        rax = self.nodes[right, cax]
        r1_rot = cos_a * r1 - sin_a * r2
        r2_rot = sin_a * r1 + cos_a * r2
        used = np.zeros(len(right), dtype=bool)
        # Only right nodes within the tolerance can be accepted, so the closest unused node is
        # taken from a ball query (k-d tree) instead of a scan of every right node: the pair,
        # or the rejection, is the one the full scan gives (same distance formula, first index
        # on ties).
        tree = None
        if len(right) > KDTREE_MIN_RIGHT:
            from scipy.spatial import cKDTree
            tree = cKDTree(np.column_stack([r1_rot, r2_rot, rax]))
        new_left, new_right, free_left, pairs = [], [], [], []
        for left_id in self.left_boundary:
            l1 = self.nodes[left_id, c1]
            l2 = self.nodes[left_id, c2]
            lax = self.nodes[left_id, cax]
            r_ref = math.sqrt(l1 * l1 + l2 * l2)
            tol = max(1e-6, 1e-4 * r_ref)
            cand = (np.arange(len(right)) if tree is None else
                    np.sort(np.asarray(tree.query_ball_point([l1, l2, lax], tol * (1.0 + 1e-9) + 1e-300),
                                       dtype=np.int64)))
            cand = cand[~used[cand]]
            best = -1
            if len(cand):
                d1 = l1 - r1_rot[cand]
                d2 = l2 - r2_rot[cand]
                dax = lax - rax[cand]
                dist = np.sqrt(d1 * d1 + d2 * d2 + dax * dax)
                q = int(np.argmin(dist))
                if dist[q] <= tol:
                    best = int(cand[q])
            if best < 0:
                free_left.append(int(left_id))
                continue
            used[best] = True
            new_left.append(int(left_id))
            new_right.append(int(right[best]))
            pairs.append((int(left_id), int(right[best])))
        free_right = [int(right[j]) for j in range(len(right)) if not used[j]]
        self.left_boundary = new_left
        self.right_boundary = new_right
        self.matched_pairs = pairs
        self.free_boundary = sorted(set(self.free_boundary) | set(free_left) | set(free_right))
