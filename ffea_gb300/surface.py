"""Surface-surface Lennard-Jones interactions on the GPU (ffea_gpu_ssint_*).

The host-side mirror of FFEA's VdW_solver for "vdw_type = lennard-jones"
(include/VdW_solver.h:36-127, src/VdW_solver.cpp:124-210): created once from
the surface faces of every blob, then called once per step with the node
positions, like VdW_solver::solve.  The node forces it returns are what
Blob::aggregate_forces_and_solve adds from the faces (src/Blob.cpp:3841-3851);
pass them to the blob update with ffea_gpu_set_external_forces.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class SsintDesc(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32), ("num_faces", ctypes.c_int32),
        ("faces", ctypes.POINTER(ctypes.c_int32)), ("face_blob", ctypes.POINTER(ctypes.c_int32)),
        ("face_type", ctypes.POINTER(ctypes.c_int32)), ("num_types", ctypes.c_int32),
        ("emin", ctypes.POINTER(ctypes.c_double)), ("rmin", ctypes.POINTER(ctypes.c_double)),
        ("num_blobs", ctypes.c_int32), ("cell_size", ctypes.c_double),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("inc_self", ctypes.c_int32),
    ]


class LJSurfaceSolver:
    """VdW_solver (lennard-jones) over all blobs' surface faces.

    num_nodes: nodes of all blobs in one numbering; faces (F, 3) corner node
    indices in FFEA's pool order; face_blob, face_type (F,), type -1 inactive;
    emin, rmin (T, T) in meso units; grid (nx, ny, nz) cells of size
    cell_size (ssint_cutoff); inc_self as inc_self_ssint."""

    def __init__(self, num_nodes, faces, face_blob, face_type, emin, rmin, num_blobs, cell_size, grid,
                 inc_self=0):
        L = _lib.lib()
        self._keep = [np.ascontiguousarray(faces, np.int32), np.ascontiguousarray(face_blob, np.int32),
                      np.ascontiguousarray(face_type, np.int32), np.ascontiguousarray(emin, np.float64),
                      np.ascontiguousarray(rmin, np.float64)]
        f, b, t, e, r = self._keep
        if e.ndim != 2 or e.shape[0] != e.shape[1] or r.shape != e.shape:
            raise ValueError("emin and rmin must be square (num_types, num_types) arrays")
        d = SsintDesc(int(num_nodes), len(b), _lib.ptr(f, _lib._ip), _lib.ptr(b, _lib._ip), _lib.ptr(t, _lib._ip),
                      e.shape[0], _lib.ptr(e), _lib.ptr(r), int(num_blobs), float(cell_size),
                      int(grid[0]), int(grid[1]), int(grid[2]), int(inc_self))
        h = ctypes.c_void_p()
        _lib.check(L.ffea_gpu_ssint_create(ctypes.byref(d), ctypes.byref(h)), "ffea_gpu_ssint_create")
        self._h = h
        self.num_nodes = int(num_nodes)
        self.num_blobs = int(num_blobs)

    def forces(self, pos):
        """One solve: returns (node forces (N, 3), energy (B, B), interacting pairs)."""
        pos = np.ascontiguousarray(pos, np.float64)
        if pos.shape != (self.num_nodes, 3):
            raise ValueError(f"pos must have shape ({self.num_nodes}, 3)")
        force = np.zeros((self.num_nodes, 3))
        energy = np.zeros((self.num_blobs, self.num_blobs))
        pairs = ctypes.c_int64(0)
        _lib.check(_lib.lib().ffea_gpu_ssint_forces(self._h, _lib.ptr(pos), _lib.ptr(force), _lib.ptr(energy),
                                                    ctypes.byref(pairs)), "ffea_gpu_ssint_forces")
        return force, energy, int(pairs.value)

    def forces_device(self, pos_ptr: int, force_ptr: int, energy_ptr: int) -> None:
        """Enqueue a solve on device arrays (raw pointers) on the solver's stream."""
        _lib.check(_lib.lib().ffea_gpu_ssint_forces_device(self._h, pos_ptr, force_ptr, energy_ptr),
                   "ffea_gpu_ssint_forces_device")

    def synchronize(self) -> int:
        pairs = ctypes.c_int64(0)
        _lib.check(_lib.lib().ffea_gpu_ssint_synchronize(self._h, ctypes.byref(pairs)), "ffea_gpu_ssint_synchronize")
        return int(pairs.value)

    @property
    def stream(self) -> int:
        return _lib.lib().ffea_gpu_ssint_stream(self._h) or 0

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().ffea_gpu_ssint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def surface_faces(verts, tets):
    """Outward surface triangles of a tetrahedral mesh: faces of exactly one
    tetrahedron, ordered so that (n1 - n0) x (n2 - n0) points away from the
    tetrahedron's fourth corner (FFEA's .surf convention)."""
    tets = np.asarray(tets)[:, :4]
    verts = np.asarray(verts, np.float64)
    loc = np.array([[1, 2, 3, 0], [0, 2, 3, 1], [0, 1, 3, 2], [0, 1, 2, 3]])
    tri = tets[:, loc[:, :3]].reshape(-1, 3)
    opp = tets[:, loc[:, 3]].reshape(-1)
    key = np.sort(tri, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    once = cnt[inv.reshape(-1)] == 1
    tri, opp = tri[once], opp[once]
    a = verts[tri[:, 1]] - verts[tri[:, 0]]
    b = verts[tri[:, 2]] - verts[tri[:, 0]]
    n = np.cross(a, b)
    flip = np.einsum("ij,ij->i", n, verts[opp] - verts[tri[:, 0]]) > 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    return tri.astype(np.int32)
