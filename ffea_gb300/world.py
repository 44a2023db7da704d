"""Python side of the GB300 blob update, shaped like FFEA's own interface.

``World`` holds one or many blobs in one device handle and runs the
per-timestep update the way ``World::run`` drives ``Blob::update_internal_forces``
and ``Blob::update_positions`` (src/World.cpp:2024-2043).  ``Blob`` is a view
of one of them with the getters a caller of FFEA's Blob uses.
``NoMassCGSolver`` / ``ConjugateGradientSolver`` mirror the Solver plugin
(include/Solver.h:30-55): init, solve (rhs in, solution out) and apply_matrix.

Errors map to ``FfeaGpuError`` -- the analogue of FFEA_ERROR -- with the
library's message.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from . import _lib as L
from .params import PRECISION_MIXED, SOLVER_MASS, SOLVER_NOMASS, SimulationParams

RNG_PER_BLOB = 0
RNG_SHARED = 1

# ffea_gpu_measurements' values per blob (FFEA_GPU_MEAS_* order)
MEASUREMENT_COLUMNS = ("kinetic", "strain", "centroid_x", "centroid_y", "centroid_z", "rmsd", "com_x", "com_y",
                       "com_z", "angmom_x", "angmom_y", "angmom_z")


def measurement_dict(row) -> dict:
    """One blob's measurement row as {"kinetic", "strain", "centroid" (3),
    "rmsd", "com" (3), "angmom" (3)}."""
    row = np.asarray(row, dtype=float)
    return {"kinetic": float(row[0]), "strain": float(row[1]), "centroid": row[2:5].copy(), "rmsd": float(row[5]),
            "com": row[6:9].copy(), "angmom": row[9:12].copy()}


class _Keep:
    """Owns the numpy arrays a Mesh struct points into until creation returns."""

    def __init__(self):
        self.arrays = []

    def arr(self, a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        self.arrays.append(a)
        return a


def _mesh_struct(keep: _Keep, pos, topology, material, drag=None, pinned=None, vel=None) -> L.Mesh:
    pos = keep.arr(np.asarray(pos).reshape(-1, 3), np.float64)
    topo = keep.arr(np.asarray(topology).reshape(-1, 10), np.int32)
    mat = keep.arr(np.asarray(material).reshape(-1, 5), np.float64)
    drag = keep.arr(drag, np.float64)
    vel = keep.arr(None if vel is None else np.asarray(vel).reshape(-1, 3), np.float64)
    pins = keep.arr(np.zeros(0, np.int32) if pinned is None else pinned, np.int32)
    if len(mat) != len(topo):
        raise ValueError("material needs one row (rho, A, B, G, E) per element")
    if drag is not None and len(drag) != len(pos):
        raise ValueError("stokes_drag needs one value per node")
    return L.Mesh(len(pos), len(topo), L.ptr(pos), L.ptr(vel), L.ptr(topo, L._ip), L.ptr(mat), L.ptr(drag),
                  len(pins), L.ptr(pins, L._ip))


PRECOND_JACOBI, PRECOND_TWO_LEVEL, PRECOND_LEARNED = 0, 1, 2


def _params_struct(p: SimulationParams, true_residual: int = 0, preconditioner: int = PRECOND_JACOBI) -> L.Params:
    return L.Params(p.dt, p.kT, p.epsilon2, p.max_iterations_cg, p.calc_noise, p.calc_stokes, p.solver, p.precision,
                    p.rng_seed, true_residual, preconditioner)


class World:
    """A batch of blobs on the current CUDA device.

    ``blobs``: sequence of objects with ``mesh`` (pos, topology), ``material``,
    ``drag``, ``pinned`` and ``params`` attributes (ffea_gb300.mesh.BlobSpec), or
    dicts with those keys.
    """

    def __init__(self, blobs: Sequence, rng_mode: int = RNG_PER_BLOB, true_residual: bool = False,
                 graph: bool = True, velocities: Sequence | None = None, preconditioner: int = PRECOND_JACOBI):
        keep = _Keep()
        meshes, params = [], []
        self.num_nodes = []
        self.num_elements = []
        self.solvers = []
        self.params = []
        for i, b in enumerate(blobs):
            get = (lambda k: b[k]) if isinstance(b, dict) else (lambda k: getattr(b, k))
            mesh = get("mesh")
            pos = mesh.pos if hasattr(mesh, "pos") else mesh["pos"]
            topo = mesh.topology if hasattr(mesh, "topology") else mesh["topology"]
            vel = None if velocities is None else velocities[i]
            meshes.append(_mesh_struct(keep, pos, topo, get("material"), get("drag"), get("pinned"), vel))
            p = get("params")
            params.append(_params_struct(p, int(true_residual), int(preconditioner)))
            self.num_nodes.append(len(np.asarray(pos).reshape(-1, 3)))
            self.num_elements.append(len(np.asarray(topo).reshape(-1, 10)))
            self.solvers.append(p.solver)
            self.params.append(p)
        n = len(meshes)
        if n == 0:
            raise ValueError("World needs at least one blob")
        marr = (L.Mesh * n)(*meshes)
        parr = (L.Params * n)(*params)
        h = ctypes.c_void_p()
        L.check(L.lib().ffea_gpu_create_batch(n, marr, parr, int(rng_mode), ctypes.byref(h)), "ffea_gpu_create_batch")
        self._h = h
        self.num_blobs = n
        self.rng_mode = int(rng_mode)
        L.lib().ffea_gpu_set_graph_mode(self._h, 1 if graph else 0)

    @classmethod
    def from_script(cls, path: str, precision: int = PRECISION_MIXED, preconditioner: int = PRECOND_JACOBI,
                    true_residual: bool = True, graph: bool = True) -> "World":
        """Every blob of an FFEA script (.ffea) in one handle, read by the
        library's C++ front end (ffea_gpu_script_load / _create)."""
        from .script import Script
        with Script(path) as sc:
            h = ctypes.c_void_p()
            L.check(L.lib().ffea_gpu_script_create(sc.handle, int(precision), int(preconditioner),
                                                   int(true_residual), ctypes.byref(h)), "ffea_gpu_script_create")
            w = cls.__new__(cls)
            w._h = h
            w.num_blobs = sc.num_blobs
            w.rng_mode = RNG_SHARED
            w.num_nodes, w.num_elements, w.solvers, w.params = [], [], [], []
            for i in range(sc.num_blobs):
                b = sc.blob(i)
                w.num_nodes.append(len(b["pos"]))
                w.num_elements.append(len(b["topology"]))
                w.params.append(sc.simulation_params(i, precision))
                w.solvers.append(w.params[-1].solver)
        L.lib().ffea_gpu_set_graph_mode(w._h, 1 if graph else 0)
        return w

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            L.lib().ffea_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- stepping
    def run(self, num_steps: int = 1) -> None:
        """num_steps x (update_internal_forces + update_positions) for every blob."""
        L.check(L.lib().ffea_gpu_step(self._h, int(num_steps)), "ffea_gpu_step")

    def run_async(self, num_steps: int = 1) -> None:
        """Enqueue steps on the handle's stream without waiting (graph mode)."""
        L.check(L.lib().ffea_gpu_step_async(self._h, int(num_steps)), "ffea_gpu_step_async")

    def synchronize(self) -> None:
        L.check(L.lib().ffea_gpu_synchronize(self._h), "ffea_gpu_synchronize")

    def cg_loop_count(self) -> int:
        return int(L.lib().ffea_gpu_cg_loop_count(self._h))

    def diag_spmv(self, variant: int, reps: int = 50) -> float:
        """Microseconds per standalone SpMV of the current matrix (variant 0..3)."""
        us = ctypes.c_double()
        L.check(L.lib().ffea_gpu_diag_spmv(self._h, int(variant), int(reps), ctypes.byref(us)), "diag_spmv")
        return us.value

    def coarse(self, blob: int = 0):
        """(A_c, X) of a blob's two-level coarse space as float32 arrays (n x n),
        or None when the handle has none."""
        n = ctypes.c_int32()
        L.check(L.lib().ffea_gpu_diag_coarse(self._h, int(blob), ctypes.byref(n), None, None), "diag_coarse")
        if n.value == 0:
            return None
        a = np.zeros((n.value, n.value), np.float32)
        x = np.zeros((n.value, n.value), np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        L.check(L.lib().ffea_gpu_diag_coarse(self._h, int(blob), ctypes.byref(n), a.ctypes.data_as(fp),
                                             x.ctypes.data_as(fp)), "diag_coarse")
        return a, x

    def coarse_half(self, blob: int = 0):
        """(Xh, s) of a blob's FP16 coarse inverse as read by the memory-resident
        solve: Xh float16 (n x n rounded up to 8 columns, zero padded) holding
        X_ij / (s_i s_j), s float32 (n), or None when the handle keeps none."""
        n, w = ctypes.c_int32(), ctypes.c_int32()
        L.check(L.lib().ffea_gpu_diag_coarse_half(self._h, int(blob), ctypes.byref(n), ctypes.byref(w), None, None),
                "diag_coarse_half")
        if n.value == 0:
            return None
        xh = np.zeros((n.value, w.value), np.uint16)
        sv = np.zeros(n.value, np.float32)
        L.check(L.lib().ffea_gpu_diag_coarse_half(self._h, int(blob), ctypes.byref(n), ctypes.byref(w),
                                                  xh.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                                  sv.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                "diag_coarse_half")
        return xh.view(np.float16), sv

    def set_timing(self, on: bool):
        L.check(L.lib().ffea_gpu_set_timing(self._h, 1 if on else 0))

    def phase_times(self) -> np.ndarray:
        out = np.zeros(5)
        L.check(L.lib().ffea_gpu_phase_times(self._h, L.ptr(out)))
        return out

    KERNEL_TIMES = ("noise", "elements", "assemble", "coarse", "nodes", "cg", "euler")

    def kernel_times(self) -> dict:
        """Milliseconds per kernel over the last timed run() (set_timing(True))."""
        out = np.zeros(len(self.KERNEL_TIMES))
        L.check(L.lib().ffea_gpu_kernel_times(self._h, L.ptr(out)))
        return dict(zip(self.KERNEL_TIMES, out.tolist()))

    def sizes(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        L.check(L.lib().ffea_gpu_sizes(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def stream(self) -> int:
        return L.lib().ffea_gpu_stream(self._h) or 0

    def preconditioner(self) -> int:
        """The preconditioner the solves use (PRECOND_*), after fall-backs."""
        return int(L.lib().ffea_gpu_preconditioner(self._h))

    def set_smoother_weights(self, blob: int, omega) -> None:
        """Per-node Jacobi weights of the learned preconditioner (blob node order)."""
        w = np.ascontiguousarray(omega, dtype=np.float32)
        L.check(L.lib().ffea_gpu_set_smoother_weights(self._h, int(blob), w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                "ffea_gpu_set_smoother_weights")

    def measurements(self) -> np.ndarray:
        """Blob::make_measurements of every blob, one row per blob, columns
        MEASUREMENT_COLUMNS (meso units); one pass over the batch."""
        out = np.zeros((self.num_blobs, len(MEASUREMENT_COLUMNS)))
        L.check(L.lib().ffea_gpu_measurements(self.handle, 0, self.num_blobs, L.ptr(out)), "ffea_gpu_measurements")
        return out

    def blob(self, i: int) -> "Blob":
        return Blob(self, i)


class Blob:
    """One blob of a World (the getters of FFEA's Blob)."""

    def __init__(self, world: World, index: int):
        if not 0 <= index < world.num_blobs:
            raise IndexError(index)
        self.world = world
        self.index = index
        self.n = world.num_nodes[index]
        self.e = world.num_elements[index]

    def get_nodes(self, out=None):
        """(pos, vel, force), each (num_nodes, 3) float64 in the blob's node
        order; `out` = three such C-contiguous arrays to fill instead."""
        if out is None:
            out = (np.empty((self.n, 3)), np.empty((self.n, 3)), np.empty((self.n, 3)))
        for a in out:
            if a.dtype != np.float64 or a.shape != (self.n, 3) or not a.flags.c_contiguous:
                raise ValueError("get_nodes: out arrays must be C-contiguous float64 of shape (num_nodes, 3)")
        pos, vel, force = out
        L.check(L.lib().ffea_gpu_get_nodes(self.world.handle, self.index, L.ptr(pos), L.ptr(vel), L.ptr(force)))
        return pos, vel, force

    def set_nodes(self, pos=None, vel=None):
        pos = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        L.check(L.lib().ffea_gpu_set_nodes(self.world.handle, self.index, L.ptr(pos), L.ptr(vel)))

    def set_external_forces(self, nodes=None, forces=None):
        """External forces (FFEA's springs / ctforces) on nodes of this blob,
        kept for every following step; no arguments clears them."""
        nodes = np.ascontiguousarray([] if nodes is None else nodes, dtype=np.int32).reshape(-1)
        forces = np.ascontiguousarray(np.zeros((0, 3)) if forces is None else forces, dtype=np.float64).reshape(-1, 3)
        if len(nodes) != len(forces):
            raise ValueError("set_external_forces: one force (3 components) per node")
        L.check(L.lib().ffea_gpu_set_external_forces(self.world.handle, self.index, len(nodes),
                                                     L.ptr(nodes, L._ip) if len(nodes) else None,
                                                     L.ptr(forces) if len(nodes) else None),
                "ffea_gpu_set_external_forces")

    def rng_state(self) -> np.ndarray:
        st = np.zeros(6, np.uint64)
        L.check(L.lib().ffea_gpu_get_rng_state(self.world.handle, self.index, L.ptr(st, L._u64p)))
        return st

    def set_rng_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.uint64)
        L.check(L.lib().ffea_gpu_set_rng_state(self.world.handle, self.index, L.ptr(st, L._u64p)))

    def energies(self):
        s, k = ctypes.c_double(), ctypes.c_double()
        L.check(L.lib().ffea_gpu_energies(self.world.handle, self.index, ctypes.byref(s), ctypes.byref(k)))
        return s.value, k.value

    def measurements(self) -> dict:
        """Blob::make_measurements at the current state (meso units): kinetic
        and strain energy, centroid, RMSD from the creation positions, centre
        of mass and angular momentum."""
        out = np.zeros(len(MEASUREMENT_COLUMNS))
        L.check(L.lib().ffea_gpu_measurements(self.world.handle, self.index, 1, L.ptr(out)), "ffea_gpu_measurements")
        return measurement_dict(out)

    def status(self):
        inv, it, fb = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        rr = ctypes.c_double()
        L.check(L.lib().ffea_gpu_status(self.world.handle, self.index, ctypes.byref(inv), ctypes.byref(it),
                                        ctypes.byref(rr), ctypes.byref(fb)))
        return {"inverted": inv.value, "cg_iters": it.value, "true_relres": rr.value, "fail_bits": fb.value}

    def rhs(self) -> np.ndarray:
        out = np.zeros((self.n, 3))
        L.check(L.lib().ffea_gpu_get_rhs(self.world.handle, self.index, L.ptr(out)))
        return out

    def element_forces(self) -> np.ndarray:
        out = np.zeros((self.e, 4, 3))
        L.check(L.lib().ffea_gpu_get_element_forces(self.world.handle, self.index, L.ptr(out)))
        return out


class _GpuSolver:
    """Solver plugin mirror (include/Solver.h:30-55) backed by a one-blob World."""

    kind = SOLVER_NOMASS

    def __init__(self):
        self.world = None

    def init(self, pos, topology, material, params: SimulationParams, drag=None, pinned=None):
        p = SimulationParams(**{**params.__dict__, "solver": self.kind})
        self.world = World([{"mesh": {"pos": pos, "topology": topology}, "material": material, "drag": drag,
                             "pinned": pinned, "params": p}], graph=False)
        self.n = len(np.asarray(pos).reshape(-1, 3))
        return 0

    def solve(self, x, pos=None):
        """x: (N_t, 3) rhs on entry, solution on return (in place)."""
        xx = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        pp = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        L.check(L.lib().ffea_gpu_solver_solve(self.world.handle, 0, L.ptr(pp), L.ptr(xx)), "solve")
        if isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous:
            x.reshape(-1, 3)[:] = xx
        return xx

    def apply_matrix(self, v):
        vin = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        out = np.zeros_like(vin)
        L.check(L.lib().ffea_gpu_solver_apply(self.world.handle, 0, L.ptr(vin), L.ptr(out)), "apply_matrix")
        return out


class NoMassCGSolver(_GpuSolver):
    kind = SOLVER_NOMASS


class ConjugateGradientSolver(_GpuSolver):
    kind = SOLVER_MASS


def rng_draws(state, offset: int, count: int) -> np.ndarray:
    """RngStream::RandU01 draws number offset .. offset+count-1 of a stream, on the GPU."""
    st = np.ascontiguousarray(state, dtype=np.uint64)
    out = np.zeros(int(count), np.float64)
    L.check(L.lib().ffea_gpu_rng_draws(L.ptr(st, L._u64p), ctypes.c_uint64(int(offset)), int(count), L.ptr(out)),
            "ffea_gpu_rng_draws")
    return out


def ffea_seed(rng_seed: int) -> np.ndarray:
    out = np.zeros(6, np.uint64)
    L.check(L.lib().ffea_gpu_ffea_seed(int(rng_seed), L.ptr(out, L._u64p)))
    return out


def kernel_launches() -> int:
    return int(L.lib().ffea_gpu_kernel_launches())


__all__ = ["World", "Blob", "NoMassCGSolver", "ConjugateGradientSolver", "rng_draws", "ffea_seed",
           "kernel_launches", "RNG_PER_BLOB", "RNG_SHARED", "PRECISION_MIXED", "SOLVER_MASS", "SOLVER_NOMASS"]
