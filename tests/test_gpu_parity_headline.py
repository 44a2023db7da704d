"""The measured path against the oracle at the measured workloads' sizes.

Every test steps the GPU blobs and the oracle's FP64 restatement of FFEA's
step (src/Blob.cpp:638-764, 3826-3969; src/NoMassCGSolver.cpp:165-197) side
by side from the same state and compares each step:
  - the RNG stream state: bit-exact;
  - the rhs handed to the solver (force) and the velocity (the solution):
    relative 2-norm error <= 1e-5 per step for the mixed FP32/FP64 path,
    <= 1e-9 for FP64.
Both sides solve to epsilon 1e-12 (the mixed path down to its FP32 floor),
so the comparison measures the path's arithmetic, not two different
stopping points.  The GPU arms are the measured ones: the learned two-level
preconditioner with the committed network weights, the two-level
preconditioner at smoother weight 1, and plain Jacobi-PCG (FFEA's own
method).  The oracle runs single-stream on all host cores
(orc_blob_set_parallel), bit-identical draws to a one-thread run.
"""
import os

import numpy as np
import pytest

from ffea_gb300 import params as P
from ffea_gb300.workloads import build_specs
from tests.helpers import rel

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)
MIXED_BAR = 1e-5
FP64_BAR = 1e-9


def _arm_world(specs, arm, memory_state=None, monkeypatch=None):
    from ffea_gb300 import learned
    from ffea_gb300.world import PRECOND_JACOBI, PRECOND_LEARNED, PRECOND_TWO_LEVEL, World
    pc = {"learned": PRECOND_LEARNED, "two-level": PRECOND_TWO_LEVEL, "jacobi": PRECOND_JACOBI}[arm]
    if monkeypatch is not None and memory_state is not None:
        monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", memory_state)
    w = World(list(specs), preconditioner=pc)
    if monkeypatch is not None:
        monkeypatch.delenv("FFEA_GPU_CG_MEMORY_STATE", raising=False)
    if specs[0].params.precision == P.PRECISION_MIXED:
        assert w.preconditioner() == pc, f"{arm} preconditioner not in use"
    if arm == "learned":
        learned.apply(w, learned.load())
    return w


def _lockstep(specs, arms, steps, oracle, monkeypatch=None):
    """Step every arm's world and one oracle blob per spec together; return
    {arm: (worst velocity error, worst force error)} over blobs and steps."""
    refs = [oracle.blob_from_spec(s, parallel=THREADS) for s in specs]
    worlds = {name: _arm_world(specs, arm, mem, monkeypatch) for name, (arm, mem) in arms.items()}
    worst = {name: [0.0, 0.0] for name in worlds}
    try:
        for step in range(steps):
            for w in worlds.values():
                w.run(1)
            for i, r in enumerate(refs):
                assert r.step(1) == 0, f"oracle step failed (blob {i}, step {step})"
                _, rvel, _ = r.nodes()
                rrhs = r.rhs()
                rst = r.rng_state()
                for name, w in worlds.items():
                    b = w.blob(i)
                    assert np.array_equal(b.rng_state(), rst), (name, i, step)
                    _, vel, _ = b.get_nodes()
                    worst[name][0] = max(worst[name][0], rel(vel, rvel))
                    worst[name][1] = max(worst[name][1], rel(b.rhs(), rrhs))
    finally:
        for w in worlds.values():
            w.close()
    return worst


def _assert_bar(worst, bar):
    for name, (v, f) in worst.items():
        assert v <= bar and f <= bar, f"{name}: velocity {v:.3e}, force {f:.3e} (bar {bar:g})"


ARMS3 = {"learned": ("learned", None), "two-level": ("two-level", None), "jacobi": ("jacobi", None)}


def test_sphere10_nomass_100_steps(gpulib, oracle):
    """The 16^3-cell, 10 nm sphere (2,771 corner nodes), 100 steps."""
    specs = build_specs("sphere10", 0, "mixed", epsilon=1e-12)
    worst = _lockstep(specs, ARMS3, 100, oracle)
    _assert_bar(worst, MIXED_BAR)


@pytest.mark.parametrize("precision,bar", [("fp64", FP64_BAR), ("mixed", MIXED_BAR)])
def test_sphere10_mass_solver_100_steps(gpulib, oracle, precision, bar):
    """The 10 nm sphere with the mass-matrix CG solver (FFEA's <solver = CG>),
    100 steps, in FP64 and in mixed precision."""
    specs = build_specs("sphere10", 0, precision, epsilon=1e-12)
    for s in specs:
        s.params.solver = P.SOLVER_MASS
    worst = _lockstep(specs, {"jacobi": ("jacobi", None)}, 100, oracle)
    _assert_bar(worst, bar)


def test_sphere40_20_steps(gpulib, oracle):
    """The 64^3-cell, 40 nm sphere (146,737 corner nodes, 823,968 elements):
    the single-blob workload of the throughput line, 20 steps, every arm."""
    specs = build_specs("sphere40", 0, "mixed", epsilon=1e-12)
    worst = _lockstep(specs, ARMS3, 20, oracle)
    _assert_bar(worst, MIXED_BAR)


def test_ensemble64_slice_20_steps(gpulib, oracle, monkeypatch):
    """Blobs 0-3 of the 64-blob ensemble (radii 8.6, 9.3, 27.2, 6.1 nm, moduli
    x 0.53 / 1.75 / 0.65 / 1.18) in one batch, 20 steps: the register-resident
    solve and the memory-resident one the full ensemble runs, with the learned
    preconditioner, and plain Jacobi."""
    specs = build_specs("ensemble64", 0, "mixed", epsilon=1e-12, blobs=[0, 1, 2, 3])
    arms = {"learned": ("learned", "0"), "learned-memory": ("learned", "1"), "jacobi-memory": ("jacobi", "1")}
    worst = _lockstep(specs, arms, 20, oracle, monkeypatch)
    _assert_bar(worst, MIXED_BAR)
