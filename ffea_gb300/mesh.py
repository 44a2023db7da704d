"""Synthetic blob meshes with FFEA's 10-node element layout.

A cube grid of ``n^3`` cells is split into 6 tetrahedra per cell along the
main diagonal (the Freudenthal / Kuhn split), optionally cut to a sphere by
keeping the tetrahedra whose centroid lies inside it, and its linear nodes are
jittered by N(0, (jitter * cell)^2) from a seed.  Every element then gets its
six edge-midpoint ("secondary") nodes, numbered after all linear nodes, in the
local order FFEA uses: n4..n9 = mid(0,1), mid(0,2), mid(0,3), mid(1,2),
mid(1,3), mid(2,3) (src/tetra_element_linear.cpp:567-591).

Stokes radii follow ffeatools' default (FFEA_convert_from_volumetric_mesh.py:
149-156 and FFEA_stokes.py default()): only linear nodes get a radius, equal
to the largest bounding-box extent divided by the number of linear nodes.
"""
from __future__ import annotations

import dataclasses
import itertools

import numpy as np

from .params import material_si_to_meso, nm, stokes_drag, SimulationParams

# corner offsets for the 6 tetrahedra of a unit cube, one per axis permutation
_PERMS = list(itertools.permutations(range(3)))
_EYE = np.eye(3, dtype=np.int64)
_TET_OFFSETS = np.array(
    [[np.zeros(3, np.int64), _EYE[p[0]], _EYE[p[0]] + _EYE[p[1]], np.ones(3, np.int64)] for p in _PERMS],
    dtype=np.int64)  # (6, 4, 3)
_EDGES = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]], dtype=np.int64)


@dataclasses.dataclass
class Mesh:
    """One blob's mesh in meso units."""

    pos: np.ndarray          # (N_t, 3) float64: linear nodes first, then secondary
    topology: np.ndarray     # (E, 10) int32
    num_linear: int
    stokes_radius: np.ndarray  # (N_t,) float64
    cell: float              # grid spacing (meso)

    @property
    def num_nodes(self) -> int:
        return len(self.pos)

    @property
    def num_elements(self) -> int:
        return len(self.topology)


def _orient(verts, tets):
    """Swap nodes 2 and 3 of negatively oriented tetrahedra."""
    a, b, c, d = (verts[tets[:, i]] for i in range(4))
    det = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    neg = det < 0
    t = tets.copy()
    t[neg, 2], t[neg, 3] = tets[neg, 3], tets[neg, 2]
    return t


def grid_mesh(n_cells: int, cell: float, radius_cells: float | None = None, jitter: float = 0.05,
              seed: int = 0, center_cells=None) -> Mesh:
    """Freudenthal-split cube grid, optionally cut to a sphere.

    ``radius_cells``: sphere radius in cells (None keeps the whole cube);
    ``center_cells``: sphere centre in cells (default: the cube centre).
    """
    n = int(n_cells)
    idx = np.arange(n, dtype=np.int64)
    cells = np.stack(np.meshgrid(idx, idx, idx, indexing="ij"), axis=-1).reshape(-1, 3)  # (C,3)
    corners = cells[:, None, None, :] + _TET_OFFSETS[None]  # (C,6,4,3)
    corners = corners.reshape(-1, 4, 3)
    if radius_cells is not None:
        c = np.full(3, n / 2.0) if center_cells is None else np.asarray(center_cells, dtype=np.float64)
        cent = corners.mean(axis=1) - c
        keep = np.einsum("ij,ij->i", cent, cent) < float(radius_cells) ** 2
        corners = corners[keep]
    m = n + 1
    flat = (corners[..., 0] * m + corners[..., 1]) * m + corners[..., 2]  # (E,4)
    used, inv = np.unique(flat.ravel(), return_inverse=True)
    tets = inv.reshape(-1, 4).astype(np.int64)
    gi = np.stack([used // (m * m), (used // m) % m, used % m], axis=-1).astype(np.float64)
    verts = gi * cell
    tets = _orient(verts, tets)
    rng = np.random.default_rng(seed)
    verts = verts + rng.normal(0.0, jitter * cell, size=verts.shape)
    N = len(verts)
    # secondary (edge-midpoint) nodes
    ea = tets[:, _EDGES[:, 0]]
    eb = tets[:, _EDGES[:, 1]]
    lo, hi = np.minimum(ea, eb), np.maximum(ea, eb)
    key = lo * N + hi
    ukey, einv = np.unique(key.ravel(), return_inverse=True)
    mid_ids = N + einv.reshape(-1, 6)
    elo, ehi = ukey // N, ukey % N
    mids = 0.5 * (verts[elo] + verts[ehi])
    pos = np.concatenate([verts, mids], axis=0)
    topo = np.concatenate([tets, mid_ids], axis=1).astype(np.int32)
    ext = verts.max(axis=0) - verts.min(axis=0)
    radius = np.zeros(len(pos))
    radius[:N] = float(ext.max()) / N
    return Mesh(pos=pos, topology=topo, num_linear=N, stokes_radius=radius, cell=cell)


def sphere_mesh(radius_nm: float, cell_nm: float = 1.25, jitter: float = 0.05, seed: int = 0) -> Mesh:
    """A cut sphere of the given radius on a grid with the given cell size."""
    r_cells = radius_nm / cell_nm
    n = int(np.ceil(2 * r_cells))
    return grid_mesh(n, nm(cell_nm), radius_cells=r_cells, jitter=jitter, seed=seed)


def cube_mesh(n_cells: int, cell_nm: float = 1.25, jitter: float = 0.05, seed: int = 0) -> Mesh:
    return grid_mesh(n_cells, nm(cell_nm), radius_cells=None, jitter=jitter, seed=seed)


@dataclasses.dataclass
class BlobSpec:
    """Everything one blob of the update needs, in meso units."""

    mesh: Mesh
    material: np.ndarray   # (E, 5): rho, A, B, G, E
    drag: np.ndarray       # (N_t,) 6 pi eta r
    pinned: np.ndarray     # (P,) int32
    params: SimulationParams

    @property
    def num_linear(self):
        return self.mesh.num_linear


def make_blob(mesh: Mesh, params: SimulationParams, density=1.5e3, shear_visc=1e-3, bulk_visc=1e-3,
              shear_mod=3.7e8, bulk_mod=1.1e9, pinned=None) -> BlobSpec:
    """Uniform SI material (converted like Blob::load_material_params) and drag."""
    E = mesh.num_elements
    mat = material_si_to_meso(np.full(E, density), np.full(E, shear_visc), np.full(E, bulk_visc),
                              np.full(E, shear_mod), np.full(E, bulk_mod))
    drag = stokes_drag(mesh.stokes_radius, params.stokes_visc, params.calc_stokes)
    pins = np.zeros(0, np.int32) if pinned is None else np.asarray(pinned, dtype=np.int32)
    return BlobSpec(mesh=mesh, material=mat, drag=drag, pinned=pins, params=params)


__all__ = ["Mesh", "grid_mesh", "sphere_mesh", "cube_mesh", "BlobSpec", "make_blob"]
