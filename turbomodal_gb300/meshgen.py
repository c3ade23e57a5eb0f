"""Seeded synthetic TET10 sector meshes: annular hub sector plus optional twisted blade.

The reference generates its test sectors with gmsh (tests/test_data/generate_blade_sector.py)
or with a pure-Python structured hex -> 6-tet split (tests/test_data/generate_test_mesh.py).
gmsh is not available here, so this module builds the same kind of sector directly:

* hub: structured (nr x nt x nz) hex grid in (r, theta, z) over r in [r_in, r_out],
  theta in [0, 2*pi/num_sectors], z in [-t/2, t/2]; each hex is split into 6 tets along
  its main diagonal (Kuhn split, face diagonals consistent between neighbours) and promoted
  to TET10 with straight-edge midside nodes, so the node set is the full quadratic lattice
  (2nr+1)(2nt+1)(2nz+1);
* strictly interior corner nodes get seeded uniform jitter of +-jitter x the local cell
  size in each parametric direction, so the cyclic faces stay planar and match exactly;
* blade (optional): a (ns x nc x nb) hex block whose root layer is a (nc x nb) patch of
  the hub rim (shared nodes, so the mesh is conforming).  Chord runs circumferentially,
  thickness axially; chord and thickness blend linearly from the patch size at the root
  to the nominal size at the tip, and the section twists linearly from 0 to ``twist_deg``.

Node sets: ``left_boundary`` (theta = 0), ``right_boundary`` (theta = sector angle) and
``hub_constraint`` (bore r = r_in), the names the reference requires
(src/mesh.cpp:236-243, src/cyclic_solver.cpp:94).
"""

from __future__ import annotations

import itertools
import math
from dataclasses import dataclass

import numpy as np

from .mesh import Mesh, NodeSet

# TET10 edge order: 4(0-1), 5(1-2), 6(0-2), 7(0-3), 8(1-3), 9(2-3)  (src/element.cpp:71-85)
_EDGES = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))


@dataclass(frozen=True)
class Material:
    """Isotropic linear-elastic material (include/turbomodal/material.hpp)."""

    E: float
    nu: float
    rho: float
    T_ref: float = 293.15
    E_slope: float = 0.0

    def __post_init__(self):
        if self.E <= 0.0:
            raise ValueError("Young's modulus E must be positive")
        if self.nu <= 0.0 or self.nu >= 0.5:
            raise ValueError("Poisson's ratio nu must be in (0, 0.5)")
        if self.rho <= 0.0:
            raise ValueError("Density rho must be positive")

    def at_temperature(self, T: float) -> "Material":
        """Linear E(T) (src/material.cpp:33-38)."""
        E_adj = self.E + self.E_slope * (T - self.T_ref)
        if E_adj <= 0.0:
            raise RuntimeError("Temperature-adjusted E is non-positive")
        return Material(E_adj, self.nu, self.rho, self.T_ref, self.E_slope)


STEEL = Material(200e9, 0.3, 7800.0)
TITANIUM = Material(114e9, 0.34, 4430.0)


def _kuhn_tets():
    """Six tets of the unit cube as monotone vertex paths 000 -> 111, positively oriented."""
    tets = []
    for perm in itertools.permutations(range(3)):
        v = [np.zeros(3, dtype=np.int64)]
        for ax in perm:
            nxt = v[-1].copy()
            nxt[ax] += 1
            v.append(nxt)
        a, b, c = v[1] - v[0], v[2] - v[0], v[3] - v[0]
        if np.dot(a, np.cross(b, c)) < 0:
            v[1], v[2] = v[2], v[1]
        tets.append([tuple(x) for x in v])
    return tets


_KUHN = _kuhn_tets()


def _lattice_tets(cells, lat_id):
    """TET10 connectivity for a block of hex cells on a quadratic lattice.

    ``cells`` is (m, 3) lower-corner cell indices; ``lat_id(I, J, K)`` maps quadratic
    lattice indices (arrays) to node ids.  Midside nodes sit at the lattice point
    between their edge's two corners.
    """
    out = np.empty((len(cells) * 6, 10), dtype=np.int64)
    base = 2 * np.asarray(cells, dtype=np.int64)
    for t, verts in enumerate(_KUHN):
        corners = [base + 2 * np.asarray(vv, dtype=np.int64) for vv in verts]
        conn = [lat_id(c[:, 0], c[:, 1], c[:, 2]) for c in corners]
        for (a, b) in _EDGES:
            mid = (corners[a] + corners[b]) // 2
            conn.append(lat_id(mid[:, 0], mid[:, 1], mid[:, 2]))
        out[t::6] = np.stack(conn, axis=1)
    return out


def _fill_midsides(pos, shape):
    """Set every odd-index lattice point to the midpoint of its edge's two corners.

    Corner points (all indices even) must already be set.  On a Kuhn-split lattice the
    edge through an odd point runs from the point minus 1 to the point plus 1 in each
    odd coordinate.
    """
    n0, n1, n2 = shape
    I, J, K = np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij")
    odd = (I % 2 == 1) | (J % 2 == 1) | (K % 2 == 1)
    oi, oj, ok = I[odd], J[odd], K[odd]
    lo = (oi - (oi % 2), oj - (oj % 2), ok - (ok % 2))
    hi = (oi + (oi % 2), oj + (oj % 2), ok + (ok % 2))
    p = pos.reshape(n0, n1, n2, 3)
    p[oi, oj, ok] = 0.5 * (p[lo] + p[hi])
    return p.reshape(-1, 3)


def sector_mesh(nr: int, nt: int, nz: int, *, r_in: float = 0.10, r_out: float = 0.30,
                thickness: float = 0.01, num_sectors: int = 36, jitter: float = 0.02,
                seed: int = 0, blade: dict | None = None) -> Mesh:
    """Build a hub sector (optionally with one blade) and run cyclic boundary matching."""
    alpha = 2.0 * math.pi / num_sectors
    rng = np.random.default_rng(seed)
    L0, L1, L2 = 2 * nr + 1, 2 * nt + 1, 2 * nz + 1
    I, J, K = np.meshgrid(np.arange(L0), np.arange(L1), np.arange(L2), indexing="ij")
    r = r_in + (r_out - r_in) * I / (2 * nr)
    th = alpha * J / (2 * nt)
    z = -0.5 * thickness + thickness * K / (2 * nz)
    corner = (I % 2 == 0) & (J % 2 == 0) & (K % 2 == 0)
    interior = corner & (I > 0) & (I < L0 - 1) & (J > 0) & (J < L1 - 1) & (K > 0) & (K < L2 - 1)
    nint = int(interior.sum())
    if jitter > 0 and nint:
        dr = (r_out - r_in) / nr
        dth = alpha / nt
        dz = thickness / nz
        u = rng.uniform(-jitter, jitter, size=(nint, 3))
        r = r.astype(np.float64).copy()
        th = th.astype(np.float64).copy()
        z = z.astype(np.float64).copy()
        r[interior] += u[:, 0] * dr
        th[interior] += u[:, 1] * dth
        z[interior] += u[:, 2] * dz
    pos = np.stack([r * np.cos(th), r * np.sin(th), z], axis=-1).reshape(-1, 3)
    pos = _fill_midsides(pos, (L0, L1, L2))
    # Exact cyclic faces: the right face is the left face rotated by alpha.
    p4 = pos.reshape(L0, L1, L2, 3)
    left = p4[:, 0, :, :].copy()
    ca, sa = math.cos(alpha), math.sin(alpha)
    p4[:, -1, :, 0] = ca * left[..., 0] - sa * left[..., 1]
    p4[:, -1, :, 1] = sa * left[..., 0] + ca * left[..., 1]
    p4[:, -1, :, 2] = left[..., 2]
    pos = p4.reshape(-1, 3)

    def hub_id(a, b, c):
        return (a * L1 + b) * L2 + c

    cells = np.array(list(itertools.product(range(nr), range(nt), range(nz))), dtype=np.int64)
    elems = [_lattice_tets(cells, hub_id)]
    nodes = [pos]
    n_hub = pos.shape[0]

    if blade is not None:
        ns, nc, nb = blade["ns"], blade["nc"], blade["nb"]
        span, chord, bthick = blade["span"], blade["chord"], blade["thick"]
        twist = math.radians(blade.get("twist_deg", 30.0))
        if nc > nt or nb > nz:
            raise ValueError("blade root patch must fit on the hub rim grid")
        j0 = 2 * ((nt - nc) // 2)
        k0 = 2 * ((nz - nb) // 2)
        B0, B1, B2 = 2 * ns + 1, 2 * nc + 1, 2 * nb + 1
        S, C, T = np.meshgrid(np.arange(B0), np.arange(B1), np.arange(B2), indexing="ij")
        rim = p4[L0 - 1]                       # (L1, L2, 3) rim lattice
        th_rim = np.arctan2(rim[..., 1], rim[..., 0])
        th_c = 0.5 * (th_rim[j0, 0] + th_rim[j0 + 2 * nc, 0])
        z_c = 0.5 * (rim[0, k0, 2] + rim[0, k0 + 2 * nb, 2])
        th_root = th_rim[j0 + C, k0 + T]
        z_root = rim[j0 + C, k0 + T, 2]
        u_root = r_out * (th_root - th_c)
        w_root = z_root - z_c
        root_chord = r_out * (th_rim[j0 + 2 * nc, 0] - th_rim[j0, 0])
        root_thick = rim[0, k0 + 2 * nb, 2] - rim[0, k0, 2]
        s = S / (2 * ns)
        u = u_root * (1.0 + (chord / root_chord - 1.0) * s)
        w = w_root * (1.0 + (bthick / root_thick - 1.0) * s)
        phi = twist * s
        u2 = u * np.cos(phi) - w * np.sin(phi)
        w2 = u * np.sin(phi) + w * np.cos(phi)
        rb = r_out + span * s
        thb = th_c + u2 / rb
        bpos = np.stack([rb * np.cos(thb), rb * np.sin(thb), z_c + w2], axis=-1)
        bpos = _fill_midsides(bpos.reshape(-1, 3), (B0, B1, B2)).reshape(B0, B1, B2, 3)
        # Layer S=0 is the hub rim; the blade owns layers S >= 1.
        own = bpos[1:].reshape(-1, 3)

        def blade_id(a, b, c):
            a = np.asarray(a)
            out = n_hub + ((a - 1) * B1 + b) * B2 + c
            root = hub_id(L0 - 1, j0 + b, k0 + c)
            return np.where(a == 0, root, out)

        bcells = np.array(list(itertools.product(range(ns), range(nc), range(nb))), dtype=np.int64)
        elems.append(_lattice_tets(bcells, blade_id))
        nodes.append(own)

    all_nodes = np.concatenate(nodes, axis=0)
    all_elems = np.concatenate(elems, axis=0).astype(np.int32)
    hub_ids = np.arange(n_hub).reshape(L0, L1, L2)
    node_sets = [
        NodeSet("hub_constraint", sorted(hub_ids[0].ravel().tolist())),
        NodeSet("left_boundary", sorted(hub_ids[:, 0, :].ravel().tolist())),
        NodeSet("right_boundary", sorted(hub_ids[:, -1, :].ravel().tolist())),
    ]
    mesh = Mesh()
    mesh.load_from_arrays(all_nodes, all_elems, node_sets, num_sectors, 2)
    return mesh


# Workload definitions: the synthetic meshes of the five benchmark configurations.
CONFIG_MESHES = {
    0: dict(nr=12, nt=8, nz=2, num_sectors=36, jitter=0.02, seed=0, blade=None),
    1: dict(nr=40, nt=24, nz=6, num_sectors=36, jitter=0.02, seed=1,
            blade=dict(ns=30, nc=10, nb=2, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0)),
    4: dict(nr=80, nt=48, nz=12, num_sectors=36, jitter=0.02, seed=4,
            blade=dict(ns=60, nc=20, nb=4, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0)),
}
CONFIG_MATERIAL = {0: STEEL, 1: TITANIUM, 4: TITANIUM}


def config_mesh(cfg: int, **overrides) -> Mesh:
    params = dict(CONFIG_MESHES[cfg])
    params.update(overrides)
    return sector_mesh(**params)


def scaled_mesh(target_nodes: int, num_sectors: int, seed: int, with_blade: bool = True) -> Mesh:
    """Config-0/1-style sector scaled to about ``target_nodes`` nodes (request-stream meshes)."""
    base_nodes = 57897 if with_blade else 2125
    f = (target_nodes / base_nodes) ** (1.0 / 3.0)
    if with_blade:
        nr, nt, nz = max(4, round(40 * f)), max(4, round(24 * f)), max(2, round(6 * f))
        ns, nc, nb = max(2, round(30 * f)), max(2, min(nt, round(10 * f))), max(1, min(nz, round(2 * f)))
        blade = dict(ns=ns, nc=nc, nb=nb, span=0.12, chord=0.05, thick=0.004, twist_deg=30.0)
    else:
        nr, nt, nz = max(2, round(12 * f)), max(2, round(8 * f)), max(1, round(2 * f))
        blade = None
    return sector_mesh(nr, nt, nz, num_sectors=num_sectors, jitter=0.02, seed=seed, blade=blade)
