"""Accuracy of the CG reductions in mixed precision, at the size of the
single-blob throughput workload (the 40 nm sphere, 146,737 corner nodes).

The solver forms each dot product as FP32 sums of the row products within a
warp, combined in double-float (TwoSum) across warps and segments.  Here the
sums r.u, w.u and r.r of the solver's last reduction (ffea_gpu_diag_cg_vectors)
are checked against an FP64 recomputation from the FP32 vectors the solver
holds in memory (each product of two FP32 values is exact in FP64):

  |sum_gpu - sum_fp64| <= 1e-6 * sum |terms|

The warp sums of 32 rows x 3 components carry about log2(96) FP32
roundings of the partial magnitudes (~4e-7 relative), the double-float
stage adds nothing at this level.  r.r and r.u (u = M r, M SPD) are also
checked to 1e-6 relative.  The memory-resident solve keeps the vectors in
memory; its reductions are bit-identical to the register-resident solve's
(tests/test_gpu_parity.py::test_register_and_memory_cg_state_agree).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vectors(w, blob=0):
    from ffea_gb300 import _lib as L
    rows = ctypes.c_int32()
    L.check(L.lib().ffea_gpu_diag_cg_vectors(w._h, blob, ctypes.byref(rows), None, None, None, None), "diag")
    r, u, wv = (np.zeros(3 * rows.value, np.float32) for _ in range(3))
    sums = np.zeros(3)
    L.check(L.lib().ffea_gpu_diag_cg_vectors(w._h, blob, ctypes.byref(rows), r.ctypes.data, u.ctypes.data,
                                             wv.ctypes.data, sums.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
            "diag")
    return r.astype(np.float64), u.astype(np.float64), wv.astype(np.float64), sums


@pytest.mark.parametrize("arm", ["jacobi", "learned"])
def test_cg_dot_products_against_fp64_sphere40(gpulib, monkeypatch, arm):
    from ffea_gb300 import learned
    from ffea_gb300.workloads import build_specs
    from ffea_gb300.world import PRECOND_JACOBI, PRECOND_LEARNED, World
    specs = build_specs("sphere40", 0, "mixed", epsilon=1e-6)
    monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", "1")
    pc = PRECOND_LEARNED if arm == "learned" else PRECOND_JACOBI
    with World(specs, preconditioner=pc) as w:
        monkeypatch.delenv("FFEA_GPU_CG_MEMORY_STATE")
        if arm == "learned":
            learned.apply(w, learned.load())
        for step in range(2):
            w.run(1)
            assert w.blob(0).status()["fail_bits"] == 0
            r, u, wv, sums = _vectors(w)
            assert np.abs(r).max() > 0, "the solver's vectors are not in memory"
            for name, a, b, k in (("r.u", r, u, 0), ("w.u", wv, u, 1), ("r.r", r, r, 2)):
                exact = float(np.dot(a, b))
                mag = float(np.dot(np.abs(a), np.abs(b)))
                err = abs(sums[k] - exact)
                assert err <= 1e-6 * mag, (arm, step, name, sums[k], exact, mag)
                if name != "w.u":
                    assert err <= 1e-6 * abs(exact), (arm, step, name, sums[k], exact)
