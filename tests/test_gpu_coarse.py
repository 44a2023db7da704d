"""The two-level preconditioner's dense coarse inverse, built with the
library's own FP32 product kernel (ffea_gpu_diag_sgemm; Newton-Schulz
X <- 2X - X A_c X in coarse.cu).

  - the product kernel against torch's FP32 matmul on sizes around its tile
    edges (1, 5, 63-65, 127-129, 300, 913) and in batches, with and without
    the 2X-style term, to 1e-5 of the product's scale;
  - the converged inverse after creation against numpy's FP64 inverse of the
    same A_c, within what FP32 arithmetic allows for its condition number,
    and symmetric, for a single blob (register-resident solve), a blob with
    an odd number of segments (n not a multiple of 4) and a batch of
    replicas (the batched update).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,batch", [(1, 1), (5, 3), (63, 2), (64, 1), (65, 2), (127, 1), (128, 3), (129, 1),
                                     (300, 2), (913, 1), (120, 256)])
@pytest.mark.parametrize("with_d", [False, True])
def test_sgemm_matches_torch(gpulib, n, batch, with_d):
    import torch
    g = torch.Generator(device="cuda").manual_seed(n * 7 + batch)
    a = torch.randn(batch, n, n, device="cuda", generator=g)
    b = torch.randn(batch, n, n, device="cuda", generator=g)
    d = torch.randn(batch, n, n, device="cuda", generator=g) if with_d else None
    c = torch.full((batch, n, n), float("nan"), device="cuda")
    alpha, beta = (-1.0, 2.0) if with_d else (1.0, 0.0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = gpulib.ffea_gpu_diag_sgemm(a.data_ptr(), b.data_ptr(), None if d is None else d.data_ptr(), c.data_ptr(),
                                    n, batch, ctypes.c_float(alpha), ctypes.c_float(beta), ctypes.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    ref = alpha * torch.matmul(a.double(), b.double())
    if with_d:
        ref = ref + beta * d.double()
    err = (c.double() - ref).abs().max().item()
    scale = np.sqrt(n) * 4.0 + (2.0 * 4.0 if with_d else 0.0)
    assert err <= 1e-5 * scale, (err, scale)


def test_sgemm_rejects_bad_arguments(gpulib):
    rc = gpulib.ffea_gpu_diag_sgemm(None, None, None, None, 4, 1, ctypes.c_float(1.0), ctypes.c_float(0.0), None)
    assert rc == -1


def _check_inverse(a, x):
    a64, x64 = a.astype(np.float64), x.astype(np.float64)
    assert np.array_equal(x, x.T), "X must be exactly symmetric"
    assert np.abs(a64 - a64.T).max() <= 1e-5 * np.abs(a64).max(), "A_c should be symmetric"
    inv = np.linalg.inv(a64)
    kappa = np.linalg.cond(a64)
    err = np.linalg.norm(x64 - inv) / np.linalg.norm(inv)
    bound = max(1e-4, 200 * kappa * np.finfo(np.float32).eps)
    assert err <= bound, (err, bound, kappa)
    assert np.linalg.eigvalsh(x64).min() > 0, "X must be positive definite"


@pytest.mark.parametrize("radius,replicas", [(8.0, 1), (12.0, 1), (5.0, 6)])
def test_coarse_inverse_after_create(gpulib, radius, replicas):
    from ffea_gb300 import params as P
    from ffea_gb300.world import PRECOND_TWO_LEVEL, World
    from tests.helpers import spec
    specs = [spec(radius_nm=radius, precision=P.PRECISION_MIXED, epsilon=1e-6, rng_seed=50 + i)
             for i in range(replicas)]
    with World(specs, preconditioner=PRECOND_TWO_LEVEL) as w:
        assert w.preconditioner() == PRECOND_TWO_LEVEL
        sizes = set()
        for i in range(replicas):
            a, x = w.coarse(i)
            sizes.add(a.shape[0])
            _check_inverse(a, x)
        w.run(12)  # one refresh of the inverse for the moved mesh (every 10 steps)
        a, x = w.coarse(0)
        _check_inverse(a, x)
    assert len(sizes) == 1


def _check_half(x, xh, s):
    """xh, s against the FP16 rounding of X_ij / (s_i s_j), s_i = sqrt(X_ii)
    in FP32 (1 where X_ii is not positive), bit for bit, padding zero."""
    n = x.shape[0]
    d = np.diag(x)
    s_ref = np.where((d > 0) & np.isfinite(d), np.sqrt(d), np.float32(1.0)).astype(np.float32)
    assert np.array_equal(s.view(np.uint32), s_ref.view(np.uint32))
    ref = (x / (s_ref[:, None] * s_ref[None, :])).astype(np.float16)
    assert xh.shape == (n, (n + 7) // 8 * 8)
    assert np.array_equal(xh[:, :n].view(np.uint16), ref.view(np.uint16))
    assert not xh[:, n:].view(np.uint16).any()
    # unit diagonal up to the rounding of s_i^2, and S Xh S symmetric and
    # positive definite as X (so the preconditioner stays SPD)
    assert np.allclose(np.diag(xh[:, :n]).astype(np.float64), 1.0, atol=2e-3)
    assert np.array_equal(xh[:, :n], xh[:, :n].T)
    assert np.linalg.eigvalsh(xh[:, :n].astype(np.float64)).min() > 0


@pytest.mark.parametrize("radius,max_ctas", [(8.0, "2"), (12.0, "3")])
def test_memory_resident_half_inverse(gpulib, monkeypatch, radius, max_ctas):
    """The memory-resident solve reads the coarse inverse from an FP16 copy
    scaled to unit diagonal (k_coarse_half): after creation and after a
    refresh it is the IEEE rounding of the current FP32 inverse, row by row;
    the register-resident solve keeps no such copy."""
    from ffea_gb300 import params as P
    from ffea_gb300.world import PRECOND_TWO_LEVEL, World
    from tests.helpers import spec
    s = spec(radius_nm=radius, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with World([s], preconditioner=PRECOND_TWO_LEVEL) as w:
        assert w.coarse_half(0) is None
    monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", "1")
    monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", max_ctas)
    with World([s], preconditioner=PRECOND_TWO_LEVEL) as w:
        assert w.preconditioner() == PRECOND_TWO_LEVEL
        for _ in range(2):
            _, x = w.coarse(0)
            xh, sv = w.coarse_half(0)
            _check_half(x, xh, sv)
            w.run(12)  # moves the mesh and refreshes the inverse
            assert w.blob(0).status()["fail_bits"] == 0
