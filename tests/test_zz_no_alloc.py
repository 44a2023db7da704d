"""The allocation-free energy entry point (ffea_gpu_energies_noalloc).

It serves callers that cannot allocate device memory where they measure --
for instance a host code's own time-step loop, where a cudaMalloc would
synchronise the device and fragment the memory pool the host manages.  Its
scratch is a static device array inside the library.  This test calls it
through the C ABI twice in a row and checks both results against the
allocating entry point ffea_gpu_energies, to 1e-9 relative (FP64 on both
sides; they differ only in the order of a few FP64 operations), and that the
two calls agree exactly: for the mass solver (kinetic term on) on a small
mesh of a few tiles, for the NoMass solver (velocity NULL, kinetic 0) on the
10 nm sphere (12,996 elements, 102 tiles of 128, so the last CTA sums many
partials), and for the mass solver on an 8 nm sphere.  It lives in its own
file so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("radius,mass", [(3.0, True), (10.0, False), (8.0, True)])
def test_energies_noalloc_matches_energies(gpulib, radius, mass):
    import torch

    from ffea_gb300 import params as P
    from ffea_gb300.world import World
    from tests.helpers import spec

    solver = P.SOLVER_MASS if mass else P.SOLVER_NOMASS
    s = spec(radius_nm=radius, solver=solver, precision=P.PRECISION_FP64)
    rest = s.mesh.pos.copy()
    with World([s]) as w:
        w.run(4)
        strain_ref, kin_ref = w.blob(0).energies()
        pos, vel, _ = w.blob(0).get_nodes()
    assert strain_ref != 0.0
    assert (kin_ref > 0.0) if mass else (kin_ref == 0.0)
    if not mass:
        assert s.mesh.num_elements > 100 * 128, "the NoMass case is meant to span more than 100 tiles"

    dev = torch.device("cuda", torch.cuda.current_device())
    t_pos = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
    t_vel = torch.from_numpy(np.ascontiguousarray(vel)).to(dev) if mass else None
    t_rest = torch.from_numpy(np.ascontiguousarray(rest)).to(dev)
    t_topo = torch.from_numpy(np.ascontiguousarray(s.mesh.topology, dtype=np.int32)).to(dev)
    t_mat = torch.from_numpy(np.ascontiguousarray(s.material)).to(dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)

    fn = gpulib.ffea_gpu_energies_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    stream = torch.cuda.current_stream(dev).cuda_stream
    results = []
    for _ in range(2):
        out.fill_(-1.0)
        rc = fn(t_pos.data_ptr(), None if t_vel is None else t_vel.data_ptr(), t_topo.data_ptr(),
                t_rest.data_ptr(), t_mat.data_ptr(), s.mesh.num_elements, solver, out.data_ptr(),
                ctypes.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        results.append(out.cpu().numpy().copy())
    for r in results:
        assert _rel(r[0], strain_ref) < 1e-9, (r[0], strain_ref)
        if mass:
            assert _rel(r[1], kin_ref) < 1e-9, (r[1], kin_ref)
        else:
            assert r[1] == 0.0
    assert np.array_equal(results[0], results[1])


def test_energies_noalloc_rejects_oversized_mesh(gpulib):
    fn = gpulib.ffea_gpu_energies_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = fn(dummy, None, dummy, dummy, dummy, 2_097_153, 0, dummy, None)
    assert rc == -1
    from ffea_gb300 import _lib as L
    assert "exceeds the maximum" in L.last_error()
