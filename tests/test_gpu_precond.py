"""The two-level and learned preconditioners of the NoMass solve (GPU).

They change how fast the CG iteration converges, not what it converges to:
every solve still stops on the reference's test sum r^2 / sum f^2 < eps^2
(src/NoMassCGSolver.cpp:180-189), and with the FP64 true-residual check on,
every accepted solution has |b - A x| / |b| < eps.  Tolerances as in
test_gpu_parity: mixed precision <= 1e-5 relative per step over 100 steps.
"""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import rel, spec

pytestmark = pytest.mark.gpu

JACOBI, TWO_LEVEL, LEARNED = 0, 1, 2


def _world(specs, **kw):
    from ffea_gb300.world import World
    return World(specs, **kw)


def test_two_level_is_used_and_meets_the_true_residual(gpulib):
    s = spec(radius_nm=8.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with _world([s], true_residual=True, preconditioner=TWO_LEVEL) as w:
        assert w.preconditioner() == TWO_LEVEL
        for _ in range(3):
            w.run(1)
            st = w.blob(0).status()
            assert st["fail_bits"] == 0, st
            assert st["true_relres"] < 1e-6, st


def test_two_level_needs_fewer_iterations(gpulib):
    s = spec(radius_nm=12.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    iters = {}
    for pc in (JACOBI, TWO_LEVEL):
        with _world([s], true_residual=True, preconditioner=pc) as w:
            w.run(2)
            st = w.blob(0).status()
            assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, (pc, st)
            iters[pc] = st["cg_iters"]
    assert iters[TWO_LEVEL] < 0.8 * iters[JACOBI], iters


def test_two_level_matches_oracle_100_steps(gpulib, oracle):
    s = spec(radius_nm=5.0, precision=P.PRECISION_MIXED)
    ref = oracle.blob_from_spec(s)
    worst_v = worst_f = 0.0
    with _world([s], preconditioner=TWO_LEVEL) as w:
        assert w.preconditioner() == TWO_LEVEL
        b = w.blob(0)
        for _ in range(100):
            w.run(1)
            assert ref.step(1) == 0
            _, vel, _ = b.get_nodes()
            _, rvel, _ = ref.nodes()
            worst_v = max(worst_v, rel(vel, rvel))
            worst_f = max(worst_f, rel(b.rhs(), ref.rhs()))
            assert b.status()["fail_bits"] == 0
    assert worst_v <= 1e-5, worst_v
    assert worst_f <= 1e-5, worst_f


def test_two_level_is_deterministic_in_and_out_of_graphs(gpulib):
    s = spec(radius_nm=8.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    outs = []
    for graph in (True, True, False):
        with _world([s], graph=graph, preconditioner=TWO_LEVEL) as w:
            w.run(4)
            outs.append(w.blob(0).get_nodes())
    for o in outs[1:]:
        for a, c in zip(outs[0], o):
            assert np.array_equal(a, c)


def test_smoother_weights(gpulib):
    from ffea_gb300._lib import FfeaGpuError
    s = spec(radius_nm=8.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    n = s.mesh.num_nodes
    with _world([s], true_residual=True, preconditioner=TWO_LEVEL) as w:
        w.run(2)
        ref = w.blob(0).get_nodes()
    with _world([s], true_residual=True, preconditioner=LEARNED) as w:
        assert w.preconditioner() == LEARNED
        w.set_smoother_weights(0, np.ones(n, np.float32))
        w.run(2)
        for a, c in zip(w.blob(0).get_nodes(), ref):
            assert np.array_equal(a, c)
        w.set_smoother_weights(0, np.full(n, 0.7, np.float32))
        w.run(2)
        st = w.blob(0).status()
        assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, st
        for bad in (0.0, 2.5, np.nan):
            with pytest.raises(FfeaGpuError, match="smoother weight"):
                w.set_smoother_weights(0, np.full(n, bad, np.float32))


@pytest.mark.parametrize("case", ["fp64", "mass"])
def test_falls_back_to_jacobi(gpulib, case):
    if case == "fp64":
        s = spec(radius_nm=4.0, precision=P.PRECISION_FP64)
    else:
        s = spec(radius_nm=4.0, precision=P.PRECISION_MIXED, solver=P.SOLVER_MASS)
    with _world([s], preconditioner=TWO_LEVEL) as w:
        assert w.preconditioner() == JACOBI
        w.run(2)
        assert w.blob(0).status()["fail_bits"] == 0


def test_handles_with_different_plans_coexist(gpulib):
    """The CG kernel's shared-memory plan depends on the mesh; handles with
    different plans must be able to step in any order."""
    a = spec(radius_nm=5.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    b = spec(radius_nm=9.0, seed=2, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with _world([a], preconditioner=TWO_LEVEL) as wa, _world([b], preconditioner=JACOBI) as wb:
        for _ in range(2):
            wa.run(1)
            wb.run(1)
        assert wa.blob(0).status()["fail_bits"] == 0
        assert wb.blob(0).status()["fail_bits"] == 0


# ---------------------------------------------------------------- memory-resident solve
# Batches with more CG segments than SMs (large blobs, ensembles), with more
# than CG_THREADS coarse dofs per blob, or reduced by the last-arriving CTA
# (many blobs) run the two-level preconditioner in the memory-resident CG
# kernel.  FFEA_GPU_CG_MAX_CTAS caps the grid to put several segments on one
# CTA at test sizes; FFEA_GPU_CG_MEMORY_STATE forces that kernel.


@pytest.mark.parametrize("max_ctas", ["1", "2"])
def test_memory_resident_two_level_matches_oracle(gpulib, oracle, monkeypatch, max_ctas):
    """Two segments on one CTA, or one each, with the row state in memory."""
    monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", "1")
    monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", max_ctas)
    s = spec(radius_nm=9.0, precision=P.PRECISION_MIXED)
    ref = oracle.blob_from_spec(s)
    worst_v = worst_f = 0.0
    with _world([s], preconditioner=TWO_LEVEL) as w:
        assert w.preconditioner() == TWO_LEVEL
        b = w.blob(0)
        for _ in range(30):
            w.run(1)
            assert ref.step(1) == 0
            _, vel, _ = b.get_nodes()
            _, rvel, _ = ref.nodes()
            worst_v = max(worst_v, rel(vel, rvel))
            worst_f = max(worst_f, rel(b.rhs(), ref.rhs()))
            assert b.status()["fail_bits"] == 0
    assert worst_v <= 1e-5, worst_v
    assert worst_f <= 1e-5, worst_f


def test_memory_resident_two_level_needs_fewer_iterations(gpulib, monkeypatch):
    monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", "1")
    monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", "2")
    s = spec(radius_nm=12.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    iters = {}
    for pc in (JACOBI, TWO_LEVEL):
        with _world([s], true_residual=True, preconditioner=pc) as w:
            assert w.preconditioner() == pc
            w.run(2)
            st = w.blob(0).status()
            assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, (pc, st)
            iters[pc] = st["cg_iters"]
    # four aggregates only: a small gain, as in the register-resident test
    assert iters[TWO_LEVEL] < 0.8 * iters[JACOBI], iters


@pytest.mark.parametrize("num_blobs", [3, 9])
def test_memory_resident_two_level_local_and_last_arriver_agree(gpulib, monkeypatch, num_blobs):
    """Uneven blobs in one batch, several segments per CTA: the redundant
    per-CTA reduction and the last-arriver reduction sum the same partials in
    the same order and apply the same coarse corrections, so the iterates are
    bit-identical, and every solve meets the true residual."""
    monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", "1")
    monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", "2")
    specs = [spec(radius_nm=3.0 + 0.75 * i, seed=i, rng_seed=70 + i, precision=P.PRECISION_MIXED, epsilon=1e-6)
             for i in range(num_blobs)]
    outs = []
    for last in ("0", "1"):
        monkeypatch.setenv("FFEA_GPU_CG_LAST_ARRIVER", last)
        with _world(specs, true_residual=True, preconditioner=TWO_LEVEL) as w:
            assert w.preconditioner() == TWO_LEVEL
            w.run(3)
            outs.append([w.blob(i).get_nodes() for i in range(num_blobs)])
            for i in range(num_blobs):
                st = w.blob(i).status()
                assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, (i, st)
    for i in range(num_blobs):
        for a, c in zip(outs[0][i], outs[1][i]):
            assert np.array_equal(a, c), i


def test_two_level_beyond_one_cta_per_segment(gpulib):
    """A blob with more CG segments than SMs (over 1024 coarse dofs): the
    memory-resident kernel carries the coarse space, every solve meets the
    true residual, and the iterations drop against Jacobi."""
    s = spec(radius_nm=46.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    iters = {}
    for pc in (JACOBI, TWO_LEVEL):
        with _world([s], true_residual=True, preconditioner=pc) as w:
            assert w.preconditioner() == pc
            w.run(2)
            st = w.blob(0).status()
            assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, (pc, st)
            iters[pc] = st["cg_iters"]
    assert iters[TWO_LEVEL] < 0.6 * iters[JACOBI], iters


@pytest.mark.parametrize("pc", [TWO_LEVEL, LEARNED])
def test_two_level_on_a_tiny_blob(gpulib, pc):
    """A blob of a few slices (130 corner nodes): every segment, which is
    also an aggregate of the coarse space, keeps enough rows for its six
    rigid modes to be independent, so the solve converges (an aggregate of
    two nodes made the coarse matrix singular)."""
    from ffea_gb300 import learned
    s = spec(radius_nm=3.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with _world([s], true_residual=True, preconditioner=pc) as w:
        assert w.preconditioner() == pc
        if pc == LEARNED:
            learned.apply(w, learned.load())
        for _ in range(3):
            w.run(1)
            st = w.blob(0).status()
            assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, st
