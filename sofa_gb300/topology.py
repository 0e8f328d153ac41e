"""Mesh topology helpers for the tetrahedral FEM path.

These build the inputs the reference scenes describe with
``RegularGridTopology`` + ``Hexa2TetraTopologicalMapping`` + ``BoxROI`` and the
synthetic beams of the benchmark workloads:

* ``regular_grid`` -- node positions and hexahedra in the reference's grid
  numbering, ``index = nx*(ny*k + j) + i`` (Sofa/Component/Topology/Container/
  Grid/src/sofa/component/topology/container/grid/GridTopology.cpp:352-356) and
  hexahedron corner order (same file, :391-398).
* ``hexa_to_tetra6`` -- the reference's 6-tetrahedra split of each hexahedron
  (Sofa/Component/Topology/Mapping/src/sofa/component/topology/mapping/
  Hexa2TetraTopologicalMapping.cpp:104-199), including its optional swapping of
  corners by grid parity.
* ``hexa_to_tetra5`` -- a 5-tetrahedra split with the diagonal choice
  alternating by cell parity (i+j+k) so neighbouring cells share face
  diagonals. The reference has no 5-tet split; this one is defined here for
  the synthetic beams and every tetrahedron is emitted with positive volume.
* ``box_roi`` -- indices of nodes inside an axis-aligned box, inclusive, like
  BoxROI's point test.
* ``beam`` -- the synthetic cantilever beam: grid, interior jitter, 5-tet
  split, fixed z=0 end.

Everything is numpy on the host; it runs once per mesh at set-up.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# Hexahedron edge pairs along each axis, in the reference's corner numbering
# (Sofa/framework/Geometry/src/sofa/geometry/Hexahedron.h:67-88).
_X_EDGES = ((0, 1), (4, 5), (3, 2), (7, 6))
_Y_EDGES = ((4, 7), (5, 6), (1, 2), (0, 3))
_Z_EDGES = ((4, 0), (5, 1), (6, 2), (7, 3))

# Per-hexahedron tetra patterns of Hexa2TetraTopologicalMapping
# (Hexa2TetraTopologicalMapping.cpp:186-190).
_TET6_PLAIN = ((0, 5, 1, 6), (0, 1, 3, 6), (1, 3, 6, 2), (6, 3, 0, 7), (6, 7, 0, 5), (7, 5, 4, 0))
_TET6_SWAPPED = ((0, 5, 6, 1), (0, 1, 6, 3), (1, 3, 2, 6), (6, 3, 7, 0), (6, 7, 5, 0), (7, 5, 0, 4))

# 5-tet split: four corner tetrahedra cut off alternate corners plus the
# central one. Even cells cut corners 1,3,4,6; odd cells cut 0,2,5,7. The
# vertex order gives every tetrahedron of an undistorted cell a positive
# volume (a jitter below a quarter of the spacing cannot flip one).
_TET5_EVEN = ((1, 0, 5, 2), (3, 0, 2, 7), (4, 0, 7, 5), (6, 2, 5, 7), (0, 2, 7, 5))
_TET5_ODD = ((0, 1, 3, 4), (2, 1, 6, 3), (5, 1, 4, 6), (7, 3, 6, 4), (1, 3, 4, 6))


def grid_index(n, i, j, k):
    """GridTopology::getIndex: nx*(ny*k + j) + i."""
    return n[0] * (n[1] * k + j) + i


def regular_grid(n, pmin, pmax):
    """Positions (N,3) float64 and hexahedra (H,8) int32 of a regular grid.

    ``n`` = (nx, ny, nz) nodes per axis; positions are p0 + dx*i + dy*j + dz*k
    with dx = (max-min)_x/(nx-1) (RegularGridTopology.cpp:165-168).
    """
    nx, ny, nz = (int(v) for v in n)
    pmin = np.asarray(pmin, dtype=np.float64)
    pmax = np.asarray(pmax, dtype=np.float64)
    d = np.where(np.array([nx, ny, nz]) > 1, (pmax - pmin) / np.maximum(np.array([nx, ny, nz]) - 1, 1), 0.0)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pos = np.empty((nx * ny * nz, 3), dtype=np.float64)
    pos[:, 0] = pmin[0] + d[0] * i.ravel()
    pos[:, 1] = pmin[1] + d[1] * j.ravel()
    pos[:, 2] = pmin[2] + d[2] * k.ravel()
    hexa = grid_hexahedra((nx, ny, nz))
    return pos, hexa


def grid_hexahedra(n):
    """Hexahedra in GridTopology order (z outer, then y, then x)."""
    nx, ny, nz = (int(v) for v in n)
    if min(nx, ny, nz) < 2:
        return np.zeros((0, 8), dtype=np.int32)
    z, y, x = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()

    def p(a, b, c):
        return nx * (ny * c + b) + a

    hexa = np.stack(
        [p(x, y, z), p(x + 1, y, z), p(x + 1, y + 1, z), p(x, y + 1, z),
         p(x, y, z + 1), p(x + 1, y, z + 1), p(x + 1, y + 1, z + 1), p(x, y + 1, z + 1)],
        axis=1,
    )
    return hexa.astype(np.int32)


def hexa_to_tetra6(hexa, n_cells=None, swapping=False):
    """Hexa2TetraTopologicalMapping: 6 tetrahedra per hexahedron.

    ``n_cells`` = (cx, cy) cells along x and y when the hexahedra come from a
    grid (used only by ``swapping``, as in the reference).
    """
    hexa = np.asarray(hexa, dtype=np.int64)
    cx, cy = (2, 1) if n_cells is None else (int(n_cells[0]), int(n_cells[1]))
    out = np.empty((hexa.shape[0] * 6, 4), dtype=np.int32)
    for h in range(hexa.shape[0]):
        c = list(hexa[h])
        swapped = False
        if swapping:
            if not ((h % cx) & 1):
                for a, b in _X_EDGES:
                    c[a], c[b] = c[b], c[a]
                swapped = not swapped
            if ((h // cx) % cy) & 1:
                for a, b in _Y_EDGES:
                    c[a], c[b] = c[b], c[a]
                swapped = not swapped
            if (h // (cx * cy)) & 1:
                for a, b in _Z_EDGES:
                    c[a], c[b] = c[b], c[a]
                swapped = not swapped
        pattern = _TET6_SWAPPED if swapped else _TET6_PLAIN
        for t, ids in enumerate(pattern):
            out[6 * h + t] = [c[ids[0]], c[ids[1]], c[ids[2]], c[ids[3]]]
    return out


def hexa_to_tetra5(hexa, n_nodes_per_axis, positions=None):
    """5 tetrahedra per grid cell, diagonals alternating with (i+j+k) parity.

    The patterns are positively oriented on undistorted cells; with
    ``positions`` given, any tetrahedron that still has a negative volume
    (a strongly distorted grid) gets vertices 2 and 3 swapped.
    """
    nx, ny, nz = (int(v) for v in n_nodes_per_axis)
    hexa = np.asarray(hexa, dtype=np.int64)
    cx, cy = nx - 1, ny - 1
    h = np.arange(hexa.shape[0])
    i, j, k = h % cx, (h // cx) % cy, h // (cx * cy)
    odd = ((i + j + k) & 1).astype(bool)
    even_t = np.array(_TET5_EVEN)
    odd_t = np.array(_TET5_ODD)
    tets = np.where(odd[:, None, None], hexa[:, odd_t], hexa[:, even_t])  # (H,5,4)
    tets = tets.reshape(-1, 4)
    if positions is not None:
        tets = orient_positive(tets, positions)
    return tets.astype(np.int32)


def beam_dims(n_nodes, aspect):
    """Grid of a square-section beam with about ``n_nodes`` nodes and
    length/width ratio ``aspect`` (z : x)."""
    nx = max(2, int(round((n_nodes / aspect) ** (1.0 / 3.0))))
    nz = max(2, int(round(n_nodes / (nx * nx))))
    return (nx, nx, nz)


def signed_volumes(tets, positions):
    p = np.asarray(positions, dtype=np.float64)
    t = np.asarray(tets, dtype=np.int64)
    a = p[t[:, 1]] - p[t[:, 0]]
    b = p[t[:, 2]] - p[t[:, 0]]
    c = p[t[:, 3]] - p[t[:, 0]]
    return np.einsum("ij,ij->i", np.cross(a, b), c) / 6.0


def orient_positive(tets, positions):
    t = np.array(tets, dtype=np.int64, copy=True)
    neg = signed_volumes(t, positions) < 0
    t[neg, 2], t[neg, 3] = t[neg, 3].copy(), t[neg, 2].copy()
    return t


def box_roi(positions, box):
    """Indices of nodes with min <= p <= max on every axis (inclusive)."""
    p = np.asarray(positions)
    lo = np.asarray(box[:3], dtype=np.float64)
    hi = np.asarray(box[3:], dtype=np.float64)
    inside = np.all((p >= lo) & (p <= hi), axis=1)
    return np.nonzero(inside)[0].astype(np.int32)


@dataclass
class BeamMesh:
    """A tetrahedral beam: rest positions, tetrahedra and the fixed z=0 end."""

    positions: np.ndarray  # (N,3) float64
    tetrahedra: np.ndarray  # (E,4) int32
    fixed: np.ndarray  # (F,) int32
    n: tuple  # nodes per axis

    @property
    def n_nodes(self):
        return int(self.positions.shape[0])

    @property
    def n_tets(self):
        return int(self.tetrahedra.shape[0])


def beam(n, spacing=0.5, jitter=0.05, seed=0, split=5):
    """Cantilever beam on an (nx,ny,nz) node grid.

    Interior nodes (not on the grid's outer faces) are moved by
    U(-jitter*spacing, +jitter*spacing) per coordinate from ``seed``. Cells are
    split into 5 tetrahedra (``split=5``) or by the reference's 6-tet mapping
    (``split=6``). Nodes with z = 0 are fixed.
    """
    nx, ny, nz = (int(v) for v in n)
    pos, hexa = regular_grid((nx, ny, nz), (0.0, 0.0, 0.0),
                             ((nx - 1) * spacing, (ny - 1) * spacing, (nz - 1) * spacing))
    if jitter > 0:
        rng = np.random.default_rng(seed)
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        interior = (i > 0) & (i < nx - 1) & (j > 0) & (j < ny - 1) & (k > 0) & (k < nz - 1)
        delta = rng.uniform(-jitter * spacing, jitter * spacing, size=pos.shape)
        pos = pos + np.where(interior[:, None], delta, 0.0)
    if split == 5:
        tets = hexa_to_tetra5(hexa, (nx, ny, nz), pos if jitter > 0.2 else None)
    elif split == 6:
        tets = hexa_to_tetra6(hexa, (nx - 1, ny - 1))
    else:
        raise ValueError("split must be 5 or 6")
    fixed = np.nonzero(np.abs(pos[:, 2]) <= 1e-12)[0].astype(np.int32)
    return BeamMesh(pos, tets, fixed, (nx, ny, nz))


@dataclass
class InclusionBeam:
    """A beam with a stiff spherical inclusion and a tip load."""

    mesh: BeamMesh
    young: np.ndarray  # (E,) per-element Young's modulus
    tip_force: np.ndarray  # (N,3) constant external force on the tip nodes
    traction: float


def inclusion_beam(n, spacing=0.5, jitter=0.05, seed=0, young_out=1e3, young_in=1e6, radius_frac=0.25,
                   traction_max=10.0):
    """Cantilever beam with a sphere of radius radius_frac * width at
    mid-length whose elements (by centroid) have young_in, the others
    young_out; a tip traction of magnitude U[0, traction_max] (seeded) along
    -y over the free end face, applied as equal forces on its nodes."""
    m = beam(n, spacing, jitter, seed, split=5)
    nx, ny, nz = m.n
    width = (nx - 1) * spacing
    centre = np.array([width / 2, (ny - 1) * spacing / 2, (nz - 1) * spacing / 2])
    cen = m.positions[m.tetrahedra].mean(axis=1)
    inside = np.linalg.norm(cen - centre, axis=1) <= radius_frac * width
    young = np.where(inside, young_in, young_out).astype(np.float64)
    rng = np.random.default_rng(seed + 7)
    t = float(rng.uniform(0.0, traction_max))
    zmax = m.positions[:, 2].max()
    tip = np.nonzero(np.abs(m.positions[:, 2] - zmax) <= 1e-12)[0]
    area = width * (ny - 1) * spacing
    f = np.zeros_like(m.positions)
    f[tip, 1] = -t * area / len(tip)
    return InclusionBeam(m, young, f, t)
