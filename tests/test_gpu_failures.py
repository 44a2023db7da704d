"""Failure detection without a GPU fault (GPU).

FFEA stops with an error when an element inverts (Blob::update_internal_forces,
src/Blob.cpp:677-685) or a solve does not converge
(src/NoMassCGSolver.cpp:191-196).  Here the failing blob stops at the
failing step, the step call returns an error, and the other blobs of a
batch carry on.  The solve's grid barriers give up after a bounded wait
and report a time-out instead of hanging; the self-test makes a wait run
out on purpose (a target no arrival reaches) and checks the report.
"""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import spec

pytestmark = pytest.mark.gpu

FAIL_INVERSION, FAIL_CG, FAIL_TIMEOUT = 1, 2, 8


def _world(specs, **kw):
    from ffea_gb300.world import World
    return World(specs, **kw)


def test_cg_non_convergence_stops_only_that_blob(gpulib):
    from ffea_gb300._lib import FfeaGpuError
    bad = spec(radius_nm=4.0, precision=P.PRECISION_MIXED, epsilon=1e-12, max_iter=2, rng_seed=5)
    good = spec(radius_nm=3.0, seed=2, precision=P.PRECISION_MIXED, epsilon=1e-6, rng_seed=6)
    with _world([bad, good]) as w:
        with pytest.raises(FfeaGpuError):
            w.run(1)
        st = w.blob(0).status()
        assert st["fail_bits"] & FAIL_CG, st
        assert w.blob(1).status()["fail_bits"] == 0
        frozen = w.blob(0).get_nodes()[0].copy()
        before = w.blob(1).get_nodes()[0].copy()
        with pytest.raises(FfeaGpuError):
            w.run(1)
        assert np.array_equal(w.blob(0).get_nodes()[0], frozen)
        assert not np.array_equal(w.blob(1).get_nodes()[0], before)


@pytest.mark.parametrize("precision", [P.PRECISION_FP64, P.PRECISION_MIXED])
def test_element_inversion_is_reported(gpulib, precision):
    from ffea_gb300._lib import FfeaGpuError
    s = spec(radius_nm=3.0, precision=precision, epsilon=1e-6)
    with _world([s]) as w:
        w.run(1)
        pos, vel, _ = w.blob(0).get_nodes()
        t = s.mesh.topology[0, :4]
        # push corner 0 of element 0 through the plane of the other three
        c = pos[t[1:]].mean(axis=0)
        pos = pos.copy()
        pos[t[0]] = c + (c - pos[t[0]])
        w.blob(0).set_nodes(pos, vel)
        with pytest.raises(FfeaGpuError, match="invert"):
            w.run(1)
        st = w.blob(0).status()
        assert st["fail_bits"] & FAIL_INVERSION and st["inverted"] >= 1, st


def test_barrier_timeout_is_reported_without_hanging(gpulib):
    import ctypes
    from ffea_gb300 import _lib as L
    for ctas in (1, 4):
        out = ctypes.c_int32(-1)
        L.check(L.lib().ffea_gpu_selftest_barrier_timeout(ctas, 2000, ctypes.byref(out)))
        assert out.value == ctas
    # the context is still usable afterwards
    s = spec(radius_nm=3.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with _world([s]) as w:
        w.run(2)
        assert w.blob(0).status()["fail_bits"] == 0
