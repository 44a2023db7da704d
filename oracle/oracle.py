"""ctypes bindings for the CPU oracle (oracle/liboracle.so) and, where it was
built, the reference objects (oracle/_ref/libffea_ref.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / --impl reference legs use this module to check and time the
CPU algorithm.  The product (ffea_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
FAST_SO = os.path.join(HERE, "liboracle_fast.so")
FAST_FLAGS = "-O3 -ffast-math -fopenmp (FFEA's GNU release flags without -march=native)"
REF_SO = os.path.join(HERE, "_ref", "libffea_ref.so")
REF_KAT = os.path.join(HERE, "_ref", "test_rngstream")
SOURCE_RECORD = os.path.join(HERE, "_ref", "SOURCE")


def reference_src():
    """The FFEA source tree: FFEA_REFERENCE_SRC, else the tree the reference
    objects in oracle/_ref were built from (recorded there by `make ref`);
    None when neither is known or the tree is absent."""
    path = os.environ.get("FFEA_REFERENCE_SRC")
    if not path and os.path.exists(SOURCE_RECORD):
        with open(SOURCE_RECORD) as fh:
            path = fh.read().strip()
    return path if path and os.path.isdir(os.path.join(path, "src")) else None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def build(ref: bool | None = None, quiet: bool = True, source: str | None = None) -> None:
    """Compile the oracle, and the reference objects from the FFEA sources at
    `source` (default reference_src()) when they are present."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "port", "fast"], check=True, stdout=out)
    src = source or reference_src()
    if ref is None:
        ref = src is not None
    if ref and src:
        subprocess.run(["make", "-C", HERE, "-j8", "ref", f"REF={src}"], check=True, stdout=out)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _declare(lib, prefix):
    f = getattr(lib, prefix + "_blob_create")
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip, _dp, _dp, ctypes.c_int, _ip, _dp, _ip]
    for name, res, args in [
        ("_blob_destroy", None, [ctypes.c_void_p]),
        ("_blob_seed", None, [ctypes.c_void_p, ctypes.c_int]),
        ("_blob_step", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
        ("_blob_get_nodes", None, [ctypes.c_void_p, _dp, _dp, _dp]),
        ("_blob_get_rhs", None, [ctypes.c_void_p, _dp]),
        ("_blob_get_element_forces", None, [ctypes.c_void_p, _dp]),
        ("_blob_last_inversions", ctypes.c_int, [ctypes.c_void_p]),
    ]:
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args


_port = None
_ref = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        lib = ctypes.CDLL(PORT_SO)
        _declare(lib, "orc")
        lib.orc_blob_set_rng_state.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p]
        lib.orc_blob_get_rng_state.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p]
        lib.orc_blob_set_nodes.argtypes = [ctypes.c_void_p, _dp, _dp]
        lib.orc_blob_set_external_forces.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp]
        lib.orc_blob_last_cg_iters.restype = ctypes.c_int
        lib.orc_blob_last_cg_iters.argtypes = [ctypes.c_void_p]
        lib.orc_blob_energies.argtypes = [ctypes.c_void_p, _dp, _dp]
        lib.orc_blob_measurements.argtypes = [ctypes.c_void_p, _dp]
        lib.orc_blob_apply_nomass.argtypes = [ctypes.c_void_p, _dp, _dp]
        lib.orc_rng_draws.argtypes = [_u64p, ctypes.c_int64, _dp]
        lib.orc_rng_jump.argtypes = [_u64p, ctypes.c_uint64]
        lib.orc_rng_fingerprint.argtypes = [_u64p, ctypes.c_int64, _dp, _u64p]
        lib.orc_rng_package_kat.restype = ctypes.c_double
        lib.orc_ffea_seed.argtypes = [ctypes.c_int, _u64p]
        lib.orc_ffea_thread_stream.argtypes = [_u64p, ctypes.c_int, _u64p]
        lib.orc_num_threads_available.restype = ctypes.c_int
        lib.orc_blob_set_parallel.restype = ctypes.c_int
        lib.orc_blob_set_parallel.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _port = lib
    return _port


_fast = None


def fast_lib():
    """The oracle built with FFEA's release flags (timed CPU baseline only)."""
    global _fast
    if _fast is None:
        if not os.path.exists(FAST_SO):
            build(ref=False)
        lib = ctypes.CDLL(FAST_SO)
        _declare(lib, "orc")
        lib.orc_blob_last_cg_iters.restype = ctypes.c_int
        lib.orc_blob_last_cg_iters.argtypes = [ctypes.c_void_p]
        lib.orc_blob_set_parallel.restype = ctypes.c_int
        lib.orc_blob_set_parallel.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _fast = lib
    return _fast


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_SO)
        _declare(lib, "ref")
        lib.ref_blob_set_rng_state.argtypes = [ctypes.c_void_p, _u64p]
        lib.ref_blob_get_rng_state.argtypes = [ctypes.c_void_p, _u64p]
        lib.ref_ffea_seed.argtypes = [ctypes.c_int, _u64p]
        lib.ref_rng_draws.argtypes = [_u64p, ctypes.c_int64, _dp]
        lib.ref_rng_advance.argtypes = [_u64p, ctypes.c_long, ctypes.c_long, _u64p]
        _ref = lib
    return _ref


# ---------------------------------------------------------------- RNG helpers
def ffea_seed(rng_seed: int) -> np.ndarray:
    out = np.zeros(6, np.uint64)
    port_lib().orc_ffea_seed(int(rng_seed), _ptr(out, _u64p))
    return out


def thread_stream(six, k: int) -> np.ndarray:
    six = np.ascontiguousarray(six, dtype=np.uint64)
    out = np.zeros(6, np.uint64)
    port_lib().orc_ffea_thread_stream(_ptr(six, _u64p), int(k), _ptr(out, _u64p))
    return out


def rng_draws(state, n: int):
    """(draws, state after) from a 6-word MRG32k3a state."""
    st = np.ascontiguousarray(state, dtype=np.uint64).copy()
    out = np.zeros(int(n), np.float64)
    port_lib().orc_rng_draws(_ptr(st, _u64p), int(n), _ptr(out, _dp))
    return out, st


def rng_jump(state, n: int) -> np.ndarray:
    st = np.ascontiguousarray(state, dtype=np.uint64).copy()
    port_lib().orc_rng_jump(_ptr(st, _u64p), ctypes.c_uint64(int(n)))
    return st


def rng_fingerprint(state, n: int):
    """(sequential sum, FNV-style hash) of n draws from a state."""
    st = np.ascontiguousarray(state, dtype=np.uint64)
    s = ctypes.c_double()
    h = ctypes.c_uint64()
    port_lib().orc_rng_fingerprint(_ptr(st, _u64p), int(n), ctypes.byref(s), ctypes.byref(h))
    return s.value, h.value


def rng_package_kat() -> float:
    return port_lib().orc_rng_package_kat()


# ---------------------------------------------------------------- blobs
class OracleBlob:
    """One blob stepped by the oracle ("port") or by the reference objects ("ref")."""

    def __init__(self, pos, topology, material, drag, pinned, dt, kT, epsilon2, max_iterations_cg=1000,
                 calc_noise=1, calc_stokes=1, solver=0, num_threads=1, impl="port"):
        self.impl = impl
        self.lib = {"port": port_lib, "fast": fast_lib, "ref": ref_lib}[impl]()
        self.pfx = "ref" if impl == "ref" else "orc"
        self.pos0 = np.ascontiguousarray(pos, dtype=np.float64)
        self.topo = np.ascontiguousarray(topology, dtype=np.int32)
        self.mat = np.ascontiguousarray(material, dtype=np.float64)
        self.drag = np.ascontiguousarray(drag, dtype=np.float64)
        self.pinned = np.ascontiguousarray(pinned if pinned is not None else np.zeros(0), dtype=np.int32)
        self.n = len(self.pos0)
        self.e = len(self.topo)
        fp = np.array([dt, kT, epsilon2], np.float64)
        ip = np.array([max_iterations_cg, calc_noise, calc_stokes, solver, num_threads], np.int32)
        self.h = getattr(self.lib, self.pfx + "_blob_create")(
            self.n, self.e, _ptr(self.pos0, _dp), _ptr(self.topo, _ip), _ptr(self.mat, _dp),
            _ptr(self.drag, _dp), len(self.pinned), _ptr(self.pinned, _ip), _ptr(fp, _dp), _ptr(ip, _ip))
        if not self.h:
            raise RuntimeError("oracle blob creation failed")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            getattr(self.lib, self.pfx + "_blob_destroy")(h)
            self.h = None

    def seed(self, rng_seed: int):
        getattr(self.lib, self.pfx + "_blob_seed")(self.h, int(rng_seed))

    def set_rng_state(self, st, thread: int = 0):
        st = np.ascontiguousarray(st, dtype=np.uint64)
        if self.pfx == "orc":
            self.lib.orc_blob_set_rng_state(self.h, thread, _ptr(st, _u64p))
        else:
            self.lib.ref_blob_set_rng_state(self.h, _ptr(st, _u64p))

    def rng_state(self, thread: int = 0) -> np.ndarray:
        st = np.zeros(6, np.uint64)
        if self.pfx == "orc":
            self.lib.orc_blob_get_rng_state(self.h, thread, _ptr(st, _u64p))
        else:
            self.lib.ref_blob_get_rng_state(self.h, _ptr(st, _u64p))
        return st

    def step(self, nsteps: int = 1) -> int:
        return getattr(self.lib, self.pfx + "_blob_step")(self.h, int(nsteps))

    def nodes(self):
        pos = np.zeros((self.n, 3)); vel = np.zeros((self.n, 3)); frc = np.zeros((self.n, 3))
        getattr(self.lib, self.pfx + "_blob_get_nodes")(self.h, _ptr(pos, _dp), _ptr(vel, _dp), _ptr(frc, _dp))
        return pos, vel, frc

    def set_nodes(self, pos=None, vel=None):
        pos = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        self.lib.orc_blob_set_nodes(self.h, _ptr(pos, _dp), _ptr(vel, _dp))

    def set_external_forces(self, nodes=None, forces=None):
        nodes = np.ascontiguousarray([] if nodes is None else nodes, dtype=np.int32).reshape(-1)
        forces = np.ascontiguousarray(np.zeros((0, 3)) if forces is None else forces, dtype=np.float64).reshape(-1)
        self.lib.orc_blob_set_external_forces(self.h, len(nodes), _ptr(nodes, _ip), _ptr(forces, _dp))

    def rhs(self):
        out = np.zeros((self.n, 3))
        getattr(self.lib, self.pfx + "_blob_get_rhs")(self.h, _ptr(out, _dp))
        return out

    def element_forces(self):
        out = np.zeros((self.e, 4, 3))
        getattr(self.lib, self.pfx + "_blob_get_element_forces")(self.h, _ptr(out, _dp))
        return out

    def last_inversions(self) -> int:
        return getattr(self.lib, self.pfx + "_blob_last_inversions")(self.h)

    def last_cg_iters(self) -> int:
        return self.lib.orc_blob_last_cg_iters(self.h)

    def set_parallel(self, threads: int):
        """Spread one single-stream blob's step over `threads` host threads with
        every draw in its serial position (orc_blob_set_parallel): element
        forces, the matrix and each SpMV stay bit-identical to one thread; only
        the NoMass CG dot products round in another order."""
        if self.pfx != "orc":
            raise NotImplementedError("the parallel single-stream mode is the C oracle's")
        if self.lib.orc_blob_set_parallel(self.h, int(threads)) != 0:
            raise ValueError("the parallel single-stream mode needs a blob with one RNG stream")

    def energies(self):
        s = ctypes.c_double(); k = ctypes.c_double()
        self.lib.orc_blob_energies(self.h, ctypes.byref(s), ctypes.byref(k))
        return s.value, k.value

    def measurements(self) -> np.ndarray:
        """Blob::make_measurements at the current state in ffea_gpu_measurements'
        order: kinetic, strain, centroid (3), RMSD, centre of mass (3),
        angular momentum (3)."""
        if self.pfx != "orc":
            raise NotImplementedError("measurements are restated by the C oracle only")
        strain, kinetic = self.energies()
        rest = np.zeros(10)
        self.lib.orc_blob_measurements(self.h, _ptr(rest, _dp))
        return np.concatenate([[kinetic, strain], rest])

    def apply_nomass(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        out = np.zeros_like(x)
        self.lib.orc_blob_apply_nomass(self.h, _ptr(x, _dp), _ptr(out, _dp))
        return out.reshape(-1, 3)


def blob_from_spec(spec, impl="port", num_threads=1, epsilon2=None, seed=True, parallel=0):
    """OracleBlob from an ffea_gb300.mesh.BlobSpec-like object.  parallel > 1
    turns on the parallel single-stream mode with that many threads."""
    p = spec.params
    b = OracleBlob(spec.mesh.pos, spec.mesh.topology, spec.material, spec.drag, spec.pinned, p.dt, p.kT,
                   p.epsilon2 if epsilon2 is None else epsilon2, p.max_iterations_cg, p.calc_noise,
                   p.calc_stokes, p.solver, num_threads, impl)
    if seed:
        b.seed(p.rng_seed)
    if parallel > 1:
        b.set_parallel(parallel)
    return b


# ---------------------------------------------------------------- surface interactions
def ssint_lj(pos, faces, face_blob, face_type, emin, rmin, num_blobs, h, grid, inc_self=0):
    """FFEA's surface-surface Lennard-Jones pass (oracle/ssint_oracle.c, which
    cites src/VdW_solver.cpp).  pos: (N, 3) FP64; faces: (F, 3) node indices;
    emin, rmin: (T, T) in meso units; grid: (nx, ny, nz) cells of size h.
    Returns (node_force (N, 3), energy (num_blobs, num_blobs), interacting pairs)."""
    lib = port_lib()
    fn = lib.oracle_ssint_lj
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _ip, _ip, ctypes.c_int, _dp, _dp, ctypes.c_int,
                   ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp,
                   ctypes.POINTER(ctypes.c_longlong)]
    pos = np.ascontiguousarray(pos, np.float64)
    faces = np.ascontiguousarray(faces, np.int32)
    face_blob = np.ascontiguousarray(face_blob, np.int32)
    face_type = np.ascontiguousarray(face_type, np.int32)
    emin = np.ascontiguousarray(emin, np.float64)
    rmin = np.ascontiguousarray(rmin, np.float64)
    force = np.zeros((len(pos), 3))
    energy = np.zeros((num_blobs, num_blobs))
    pairs = ctypes.c_longlong(0)
    rc = fn(len(pos), _ptr(pos, _dp), len(faces), _ptr(faces, _ip), _ptr(face_blob, _ip), _ptr(face_type, _ip),
            emin.shape[0], _ptr(emin, _dp), _ptr(rmin, _dp), num_blobs, float(h), int(grid[0]), int(grid[1]),
            int(grid[2]), int(inc_self), _ptr(force, _dp), _ptr(energy, _dp), ctypes.byref(pairs))
    if rc != 0:
        raise ValueError("a face centroid lies outside the interaction grid")
    return force, energy, int(pairs.value)


def ssint(pos, faces, face_blob, face_type, emin, rmin, num_blobs, h, grid, inc_self=0, ssint_type=0,
          face_apex=None, steric_factor=1.0, steric_dr=5e-3, k0=None, blob_corr=None, sticky_wall=False):
    """FFEA's surface-surface pass for any ssint type (oracle/ssint_oracle.c
    with oracle/steric_oracle.c): 0 lennard-jones, 1 steric, 2 ljsteric,
    3 gensoft; blob_corr (B, B, 3) the periodic corrections (force_pbc),
    sticky_wall the xz walls.  Returns (node_force (N, 3), energy (B, B),
    interacting pairs)."""
    lib = port_lib()
    fn = lib.oracle_ssint
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _ip, _ip, _ip, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int,
                   ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_double, ctypes.c_double, _dp, ctypes.c_int, _dp, _dp, ctypes.POINTER(ctypes.c_longlong)]
    bc = None if blob_corr is None else np.ascontiguousarray(blob_corr, np.float64).reshape(-1)
    pos = np.ascontiguousarray(pos, np.float64)
    faces = np.ascontiguousarray(faces, np.int32)
    apex = None if face_apex is None else np.ascontiguousarray(face_apex, np.int32)
    face_blob = np.ascontiguousarray(face_blob, np.int32)
    face_type = np.ascontiguousarray(face_type, np.int32)
    emin = np.ascontiguousarray(emin, np.float64)
    rmin = np.ascontiguousarray(rmin, np.float64)
    kk = None if k0 is None else np.ascontiguousarray(k0, np.float64)
    force = np.zeros((len(pos), 3))
    energy = np.zeros((num_blobs, num_blobs))
    pairs = ctypes.c_longlong(0)
    rc = fn(len(pos), _ptr(pos, _dp), len(faces), _ptr(faces, _ip), _ptr(apex, _ip), _ptr(face_blob, _ip),
            _ptr(face_type, _ip), emin.shape[0], _ptr(emin, _dp), _ptr(rmin, _dp), _ptr(kk, _dp), num_blobs,
            float(h), int(grid[0]), int(grid[1]), int(grid[2]), int(inc_self), int(ssint_type),
            float(steric_factor), float(steric_dr), _ptr(bc, _dp), int(bool(sticky_wall)), _ptr(force, _dp),
            _ptr(energy, _dp), ctypes.byref(pairs))
    if rc == -2:
        raise ValueError("the sticky wall needs at least two rows of cells in y")
    if rc != 0:
        raise ValueError("a face centroid lies outside the interaction grid")
    return force, energy, int(pairs.value)


def blob_corr(centroids, box):
    """World::calc_blob_corr_matrix: (B, B, 3) periodic corrections of blob centroids (B, 3) in a box (3)."""
    lib = port_lib()
    lib.oracle_blob_corr.restype = None
    lib.oracle_blob_corr.argtypes = [ctypes.c_int, _dp, _dp, _dp]
    c = np.ascontiguousarray(centroids, np.float64).reshape(-1, 3)
    b = np.ascontiguousarray(box, np.float64).reshape(3)
    out = np.zeros((len(c), len(c), 3))
    lib.oracle_blob_corr(len(c), _ptr(c, _dp), _ptr(b, _dp), _ptr(out, _dp))
    return out


def steric_overlap(A, B):
    """(volume, FFEA's centre) of the overlap of tetrahedra A and B (4 x 3 each)."""
    lib = port_lib()
    lib.steric_overlap.restype = ctypes.c_double
    lib.steric_overlap.argtypes = [_dp, _dp, _dp]
    A = np.ascontiguousarray(A, np.float64)
    B = np.ascontiguousarray(B, np.float64)
    cm = np.zeros(3)
    v = lib.steric_overlap(_ptr(A, _dp), _ptr(B, _dp), _ptr(cm, _dp))
    return v, cm


def steric_pair(A, B, dr, k=1.0):
    """One steric pair (oracle/steric_oracle.c): None without overlap, else
    (k V, forces on A's 4 nodes, forces on B's)."""
    lib = port_lib()
    lib.steric_pair.restype = ctypes.c_int
    lib.steric_pair.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]
    A = np.ascontiguousarray(A, np.float64)
    B = np.ascontiguousarray(B, np.float64)
    vol = np.zeros(1)
    f1 = np.zeros((4, 3))
    f2 = np.zeros((4, 3))
    if not lib.steric_pair(_ptr(A, _dp), _ptr(B, _dp), float(dr), float(k), _ptr(vol, _dp), _ptr(f1, _dp),
                           _ptr(f2, _dp)):
        return None
    return float(vol[0]), f1, f2
