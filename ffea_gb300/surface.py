"""Surface-surface interactions on the GPU (ffea_gpu_ssint_*).

The host-side mirror of FFEA's VdW_solver and its steric variants
(include/VdW_solver.h:36-127, src/VdW_solver.cpp:124-210; Steric_solver,
LJSteric_solver, GenSoftSSINT_solver) for ssint_type lennard-jones, steric,
ljsteric and gensoft: created once from the surface faces of every blob, then
called once per step with the node positions, like VdW_solver::solve.  The node forces it returns are what
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
        ("ssint_type", ctypes.c_int32), ("face_apex", ctypes.POINTER(ctypes.c_int32)),
        ("steric_factor", ctypes.c_double), ("steric_dr", ctypes.c_double),
        ("k0", ctypes.POINTER(ctypes.c_double)),
    ]


# SimulationParams::ssint_type
SSINT_LJ, SSINT_STERIC, SSINT_LJSTERIC, SSINT_GENSOFT = 0, 1, 2, 3
SSINT_TYPES = {"lennard-jones": SSINT_LJ, "steric": SSINT_STERIC, "ljsteric": SSINT_LJSTERIC,
               "gensoft": SSINT_GENSOFT}


class SurfaceSolver:
    """VdW_solver (or a steric variant) over all blobs' surface faces.

    num_nodes: nodes of all blobs in one numbering; faces (F, 3) corner node
    indices in FFEA's pool order; face_blob, face_type (F,), type -1 inactive;
    emin, rmin (T, T) in meso units; grid (nx, ny, nz) cells of size
    cell_size (ssint_cutoff); inc_self as inc_self_ssint.  The steric types
    (ssint_type SSINT_STERIC, SSINT_LJSTERIC, SSINT_GENSOFT) also take
    face_apex (F,), the fourth node of each face's element (Face::n[3]),
    steric_factor and steric_dr (SimulationParams), and gensoft k0 (T, T) in
    meso units.  sticky_wall: the xz walls of sticky_wall_xz; periodic blob
    corrections (force_pbc) are set per pass with set_pbc."""

    def __init__(self, num_nodes, faces, face_blob, face_type, emin, rmin, num_blobs, cell_size, grid,
                 inc_self=0, ssint_type=SSINT_LJ, face_apex=None, steric_factor=1.0, steric_dr=5e-3, k0=None,
                 sticky_wall=False):
        L = _lib.lib()
        self._keep = [np.ascontiguousarray(faces, np.int32), np.ascontiguousarray(face_blob, np.int32),
                      np.ascontiguousarray(face_type, np.int32), np.ascontiguousarray(emin, np.float64),
                      np.ascontiguousarray(rmin, np.float64)]
        f, b, t, e, r = self._keep
        if e.ndim != 2 or e.shape[0] != e.shape[1] or r.shape != e.shape:
            raise ValueError("emin and rmin must be square (num_types, num_types) arrays")
        apex = None if face_apex is None else np.ascontiguousarray(face_apex, np.int32)
        kk = None if k0 is None else np.ascontiguousarray(k0, np.float64)
        if kk is not None and kk.shape != e.shape:
            raise ValueError("k0 must be a (num_types, num_types) array")
        self._keep += [apex, kk]
        d = SsintDesc(int(num_nodes), len(b), _lib.ptr(f, _lib._ip), _lib.ptr(b, _lib._ip), _lib.ptr(t, _lib._ip),
                      e.shape[0], _lib.ptr(e), _lib.ptr(r), int(num_blobs), float(cell_size),
                      int(grid[0]), int(grid[1]), int(grid[2]), int(inc_self), int(ssint_type),
                      _lib.ptr(apex, _lib._ip), float(steric_factor), float(steric_dr), _lib.ptr(kk))
        h = ctypes.c_void_p()
        _lib.check(L.ffea_gpu_ssint_create(ctypes.byref(d), ctypes.byref(h)), "ffea_gpu_ssint_create")
        self._h = h
        self.num_nodes = int(num_nodes)
        self.num_blobs = int(num_blobs)
        self.box = float(cell_size) * np.asarray(grid[:3], np.float64)
        if sticky_wall:
            _lib.check(L.ffea_gpu_ssint_set_sticky_wall(h, 1), "ffea_gpu_ssint_set_sticky_wall")

    def set_pbc(self, blob_corr=None):
        """Periodic blob corrections (num_blobs, num_blobs, 3) for the next
        passes, as World::calc_blob_corr_matrix makes them (blob_corr()
        below); None turns them off."""
        if blob_corr is None:
            _lib.check(_lib.lib().ffea_gpu_ssint_set_pbc(self._h, None), "ffea_gpu_ssint_set_pbc")
            return
        bc = np.ascontiguousarray(blob_corr, np.float64)
        if bc.shape != (self.num_blobs, self.num_blobs, 3):
            raise ValueError(f"blob_corr must have shape ({self.num_blobs}, {self.num_blobs}, 3)")
        _lib.check(_lib.lib().ffea_gpu_ssint_set_pbc(self._h, _lib.ptr(bc)), "ffea_gpu_ssint_set_pbc")

    def blob_corr(self, centroids):
        """World::calc_blob_corr_matrix for blob centroids (num_blobs, 3) in this grid's box."""
        c = np.ascontiguousarray(centroids, np.float64).reshape(-1, 3)
        out = np.zeros((len(c), len(c), 3))
        _lib.check(_lib.lib().ffea_gpu_ssint_blob_corr(len(c), _lib.ptr(c), _lib.ptr(self.box), _lib.ptr(out)),
                   "ffea_gpu_ssint_blob_corr")
        return out

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


# the name of the Lennard-Jones-only solver, kept for its callers
LJSurfaceSolver = SurfaceSolver


def surface_faces(verts, tets, with_apex=False):
    """Outward surface triangles of a tetrahedral mesh: faces of exactly one
    tetrahedron, ordered so that (n1 - n0) x (n2 - n0) points away from the
    tetrahedron's fourth corner (FFEA's .surf convention).  with_apex: also
    return that fourth corner per face (Face::n[3], for the steric types)."""
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
    if with_apex:
        return tri.astype(np.int32), opp.astype(np.int32)
    return tri.astype(np.int32)
