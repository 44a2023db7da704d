"""GPU blob update vs the CPU oracle (FFEA's algorithm restated), through the C ABI.

Tolerances:
  - RNG draws: bit-exact.
  - FP64 precision mode: positions to 1e-10 absolute (meso), velocities and
    rhs to 1e-9 relative (2-norm) -- the remaining differences are CG
    round-off with both sides solving to epsilon 1e-12.
  - mixed FP32/FP64 mode: per-step velocity and force error <= 1e-5 relative
    (2-norm) over the first 100 steps, the parity bar of the mixed path.
"""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import rel, spec

pytestmark = pytest.mark.gpu


def _world(specs, **kw):
    from ffea_gb300.world import World
    return World(specs, **kw)


def test_rng_draws_bit_exact(gpulib, oracle):
    from ffea_gb300.world import rng_draws
    st = oracle.ffea_seed(44)
    ref, _ = oracle.rng_draws(st, 5000)
    got = rng_draws(st, 0, 5000)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    # arbitrary offsets via jump-ahead, including beyond 2^32
    for off in (1, 255, 256, 65537, 7 * 823968 + 5, 2**31 + 3, 2**32 + 17, 3 * 2**32 + 1):
        jumped = oracle.rng_jump(st, off)
        ref, _ = oracle.rng_draws(jumped, 64)
        got = rng_draws(st, off, 64)
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), off


@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS])
def test_fp64_matches_oracle_10_steps(gpulib, oracle, solver):
    s = spec(radius_nm=3.0, solver=solver)
    ref = oracle.blob_from_spec(s)
    with _world([s]) as w:
        b = w.blob(0)
        for step in range(10):
            w.run(1)
            assert ref.step(1) == 0
            pos, vel, force = b.get_nodes()
            rpos, rvel, rforce = ref.nodes()
            assert np.array_equal(b.rng_state(), ref.rng_state()), step
            assert rel(b.rhs(), ref.rhs()) < 1e-9, step
            assert rel(vel, rvel) < 1e-9, step
            assert np.abs(pos - rpos).max() < 1e-10, step


def test_fp64_pinned_nodes(gpulib, oracle):
    s = spec(radius_nm=3.0, pinned=[0, 3, 10, 11])
    ref = oracle.blob_from_spec(s)
    with _world([s]) as w:
        w.run(5)
        assert ref.step(5) == 0
        pos, vel, _ = w.blob(0).get_nodes()
        rpos, rvel, _ = ref.nodes()
        assert np.abs(vel[[0, 3, 10, 11]]).max() == 0.0
        assert rel(vel, rvel) < 1e-9
        assert np.abs(pos - rpos).max() < 1e-10


def test_secondary_drag_folding(gpulib, oracle):
    """Stokes radii on every node (as in hand-made .stokes files): the midpoint
    nodes' noise is folded onto the corners like Blob::linearise_force."""
    s = spec(radius_nm=3.0)
    s.drag = s.drag.copy()
    s.drag[s.mesh.num_linear:] = 0.5 * s.drag[0]
    ref = oracle.blob_from_spec(s)
    with _world([s]) as w:
        w.run(3)
        assert ref.step(3) == 0
        _, vel, _ = w.blob(0).get_nodes()
        _, rvel, _ = ref.nodes()
        assert rel(vel, rvel) < 1e-9


@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS])
def test_mixed_precision_100_steps(gpulib, oracle, solver):
    s = spec(radius_nm=4.0, solver=solver, precision=P.PRECISION_MIXED)
    ref = oracle.blob_from_spec(s)
    worst_v = worst_f = 0.0
    with _world([s]) as w:
        b = w.blob(0)
        for step in range(100):
            w.run(1)
            assert ref.step(1) == 0
            _, vel, _ = b.get_nodes()
            _, rvel, _ = ref.nodes()
            worst_v = max(worst_v, rel(vel, rvel))
            worst_f = max(worst_f, rel(b.rhs(), ref.rhs()))
    assert worst_v <= 1e-5, worst_v
    assert worst_f <= 1e-5, worst_f


def test_batch_equals_independent_blobs(gpulib):
    specs = [spec(radius_nm=r, seed=i, rng_seed=100 + i, precision=P.PRECISION_MIXED) for i, r in enumerate((2.5, 4.0, 3.0))]
    with _world(specs) as w:
        w.run(4)
        batch = [w.blob(i).get_nodes() for i in range(3)]
    for i, s in enumerate(specs):
        with _world([s]) as w1:
            w1.run(4)
            single = w1.blob(0).get_nodes()
        for a, c in zip(batch[i], single):
            assert np.array_equal(a, c), i


def test_deterministic_and_graph_equals_host_loop(gpulib):
    s = spec(radius_nm=4.0, precision=P.PRECISION_MIXED)
    outs = []
    for graph in (True, True, False):
        with _world([s], graph=graph) as w:
            w.run(5)
            outs.append(w.blob(0).get_nodes())
    for o in outs[1:]:
        for a, c in zip(outs[0], o):
            assert np.array_equal(a, c)


def test_register_and_memory_cg_state_agree(gpulib, monkeypatch):
    """The persistent solver keeps per-row CG state in registers when every
    node tile has a CTA; the memory-resident variant (used for larger meshes)
    must give the same iterates."""
    s = spec(radius_nm=4.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    outs = []
    for mem in ("0", "1"):
        monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", mem)
        with _world([s], true_residual=True) as w:
            w.run(3)
            outs.append(w.blob(0).get_nodes())
            st = w.blob(0).status()
            assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6
    for a, c in zip(outs[0], outs[1]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("precision", [P.PRECISION_MIXED, P.PRECISION_FP64])
def test_shared_memory_matrix_copy_is_exact(gpulib, monkeypatch, precision):
    """Matrix slots read from the per-solve shared-memory copy enter the SpMV
    in the same order as slots read from global memory: identical iterates
    with the copy on or off."""
    s = spec(radius_nm=8.0, precision=precision, epsilon=1e-6 if precision == P.PRECISION_MIXED else 1e-12)
    outs = []
    for slots in ("0", "64"):
        monkeypatch.setenv("FFEA_GPU_CG_SMEM_SLOTS", slots)
        with _world([s]) as w:
            w.run(3)
            outs.append(w.blob(0).get_nodes())
            assert w.blob(0).status()["fail_bits"] == 0
    for a, c in zip(outs[0], outs[1]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("max_ctas", ["1", "3"])
def test_several_segments_per_cta_match_oracle(gpulib, oracle, monkeypatch, max_ctas):
    """A grid capped below the segment count runs the memory-resident CG
    variant with several segments per CTA (the layout of batches too large
    for one segment per CTA); FP64 results must still follow the oracle."""
    monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", max_ctas)
    s = spec(radius_nm=8.0)
    ref = oracle.blob_from_spec(s)
    with _world([s]) as w:
        b = w.blob(0)
        for step in range(4):
            w.run(1)
            assert ref.step(1) == 0
            pos, vel, _ = b.get_nodes()
            rpos, rvel, _ = ref.nodes()
            assert b.status()["fail_bits"] == 0
            assert rel(vel, rvel) < 1e-9, step
            assert np.abs(pos - rpos).max() < 1e-10, step


@pytest.mark.parametrize("num_blobs", [1, 9])
def test_local_and_last_arriver_reduction_agree(gpulib, monkeypatch, num_blobs):
    """The CG sums are reduced either redundantly by every CTA (few tiles and
    blobs) or once by the last CTA at a barrier; both sum the same partials
    in the same order (a CTA per blob below 8 blobs, a warp per blob from 8),
    so the iterates must be bit-identical."""
    specs = [spec(radius_nm=2.5 + 0.25 * i, seed=i, rng_seed=60 + i, precision=P.PRECISION_MIXED, epsilon=1e-6)
             for i in range(num_blobs)]
    outs = []
    for last in ("0", "1"):
        monkeypatch.setenv("FFEA_GPU_CG_LAST_ARRIVER", last)
        with _world(specs, true_residual=True) as w:
            w.run(3)
            outs.append([w.blob(i).get_nodes() for i in range(num_blobs)])
            for i in range(num_blobs):
                st = w.blob(i).status()
                assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, (i, st)
    for i in range(num_blobs):
        for a, c in zip(outs[0][i], outs[1][i]):
            assert np.array_equal(a, c), i


def test_true_residual_confirms_convergence(gpulib, oracle):
    s = spec(radius_nm=4.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with _world([s], true_residual=True) as w:
        for _ in range(5):
            w.run(1)
            st = w.blob(0).status()
            assert st["fail_bits"] == 0
            assert st["true_relres"] < 1e-6, st


@pytest.mark.parametrize("pinned", [None, [0, 7]])
def test_lumped_mass_solver_matches_oracle(gpulib, oracle, pinned):
    """<solver = masslumped>: x = M_lumped^-1 f with no CG (MassLumpedSolver,
    src/MassLumpedSolver.cpp:40-89), then the mass-path Euler update; FP64
    tolerances as above, and no CG iterations are reported."""
    from ffea_gb300.world import World
    s = spec(radius_nm=4.0, solver=P.SOLVER_LUMPED, pinned=pinned)
    ref = oracle.blob_from_spec(s)
    with World([s]) as w:
        b = w.blob(0)
        for step in range(10):
            w.run(1)
            assert ref.step(1) == 0
            pos, vel, _ = b.get_nodes()
            rpos, rvel, _ = ref.nodes()
            assert rel(b.rhs(), ref.rhs()) < 1e-9, step
            assert rel(vel, rvel) < 1e-9, step
            assert np.abs(pos - rpos).max() < 1e-10, step
            assert b.status()["cg_iters"] == 0
        ks, kk = b.energies()
        rs, rk = ref.energies()
        assert abs(ks - rs) <= 1e-9 * abs(rs) and abs(kk - rk) <= 1e-9 * abs(rk), (ks, rs, kk, rk)


def test_node_io_pinned_and_device_buffers_agree(gpulib):
    """get_nodes / set_nodes with pinned host arrays (staged copies) and with
    device arrays (used in place): the values are those of the path with
    pageable arrays, bit for bit."""
    import ctypes

    import torch

    from ffea_gb300 import _lib as L
    from ffea_gb300.world import World
    s = spec(radius_nm=4.0, solver=P.SOLVER_MASS, precision=P.PRECISION_MIXED, epsilon=1e-6)
    n = s.mesh.num_nodes
    with World([s]) as w:
        b = w.blob(0)
        w.run(3)
        ref = b.get_nodes()
        pinned = tuple(torch.empty((n, 3), dtype=torch.float64, pin_memory=True) for _ in range(3))
        b.get_nodes(out=tuple(t.numpy() for t in pinned))
        for a, c in zip(ref, pinned):
            assert np.array_equal(a, c.numpy())
        dev = tuple(torch.empty((n, 3), dtype=torch.float64, device="cuda") for _ in range(3))
        dp = [ctypes.cast(t.data_ptr(), L._dp) for t in dev]
        L.check(L.lib().ffea_gpu_get_nodes(w.handle, 0, *dp))
        torch.cuda.synchronize()
        for a, c in zip(ref, dev):
            assert np.array_equal(a, c.cpu().numpy())
        # set from pinned (shifted positions, scaled velocities), read back staged
        pos2 = torch.from_numpy(ref[0] + 0.01).pin_memory()
        vel2 = torch.from_numpy(ref[1] * 0.5).pin_memory()
        b.set_nodes(pos2.numpy(), vel2.numpy())
        got = b.get_nodes()
        corner = np.zeros(n, bool)
        corner[s.mesh.topology[:, :4]] = True
        assert np.array_equal(got[0][corner], ref[0][corner] + 0.01)
        assert np.array_equal(got[1][corner], ref[1][corner] * 0.5)
        # and from device arrays
        pos3 = torch.from_numpy(ref[0]).cuda()
        L.check(L.lib().ffea_gpu_set_nodes(w.handle, 0, ctypes.cast(pos3.data_ptr(), L._dp), None))
        assert np.array_equal(b.get_nodes()[0][corner], ref[0][corner])
        w.run(2)
        assert b.status()["fail_bits"] == 0


@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS])
def test_all_pinned_blob(gpulib, oracle, solver):
    """Every node pinned: no element step and no element draws, as in the
    reference (src/Blob.cpp:643-645); the RNG stream advances by the node
    draws alone, bit for bit with the oracle.  Nothing moves.  (FFEA's
    NoMassCGSolver turns the all-zero rhs into NaN positions, 0 / 0 before
    its stopping test; the GPU solve stops on the zero rhs, as FFEA's own
    residual2 treats sum f^2 = 0 as converged, and returns x = 0.)"""
    from ffea_gb300.world import World
    s0 = spec(radius_nm=3.0)
    s = spec(radius_nm=3.0, solver=solver, pinned=list(range(s0.mesh.num_nodes)))
    ref = oracle.blob_from_spec(s)
    with World([s]) as w:
        pos0, _, _ = w.blob(0).get_nodes()
        w.run(5)
        assert ref.step(5) == 0
        b = w.blob(0)
        assert np.array_equal(b.rng_state(), ref.rng_state())
        pos, vel, _ = b.get_nodes()
        assert np.array_equal(pos, pos0) and not vel.any()
        if solver == P.SOLVER_MASS:
            assert np.array_equal(pos, ref.nodes()[0])
        assert b.status()["fail_bits"] == 0


@pytest.mark.parametrize("rng_mode", ["per_blob", "shared"])
def test_rng_state_set_on_a_running_handle_replays(gpulib, oracle, rng_mode):
    """The noise kernel keeps each run's start state for the next step (one
    advance per step instead of a jump).  Setting a blob's RNG state on a
    handle that has already stepped must drop those kept states: rewinding
    the RNG state and the nodes to an earlier step replays the same steps bit
    for bit, and the draws stay the oracle's (compared through the stream
    state after every step)."""
    from ffea_gb300.world import RNG_PER_BLOB, RNG_SHARED, World
    specs = [spec(radius_nm=3.0, seed=1, rng_seed=7), spec(radius_nm=2.5, seed=2, rng_seed=9)]
    mode = RNG_PER_BLOB if rng_mode == "per_blob" else RNG_SHARED
    with World(specs, rng_mode=mode) as w:
        w.run(2)
        saved = [(w.blob(i).rng_state(), w.blob(i).get_nodes()) for i in range(2)]
        w.run(3)
        first = [(w.blob(i).rng_state(), w.blob(i).get_nodes()[0]) for i in range(2)]
        for i, (st, (pos, vel, _)) in enumerate(saved):
            w.blob(i).set_rng_state(st)
            w.blob(i).set_nodes(pos, vel)
        w.run(3)
        for i in range(2):
            st, pos = first[i]
            assert np.array_equal(w.blob(i).rng_state(), st), i
            assert np.array_equal(w.blob(i).get_nodes()[0], pos), i
    if mode == RNG_PER_BLOB:
        # a fresh handle seeded from the saved state agrees with the oracle
        ref = oracle.blob_from_spec(specs[0])
        assert ref.step(5) == 0
        assert np.array_equal(first[0][0], ref.rng_state())
