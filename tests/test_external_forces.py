"""External forces on the rhs (FFEA's springs / ctforces): the oracle's fold
onto corner nodes on the CPU, and the GPU step against the oracle.

FFEA adds interaction and constant forces to Blob::force after the per-step
zeroing and before the element loop (src/World.cpp:1907, src/Blob.cpp:647,
2094-2162); Blob::linearise_force then moves half of a secondary node's force
onto each end of its edge (src/Blob.cpp:1066-1085) and pinned nodes keep
none (:3907-3919).  Tolerances as in test_gpu_parity."""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import rel, spec


def _forces(s, rng, count=12):
    """A few corner and edge-midpoint nodes (one repeated) with forces of the
    size of a blob's elastic forces (meso units)."""
    topo = s.mesh.topology
    corners = np.unique(topo[:, :4])
    mids = np.unique(topo[:, 4:])
    nodes = np.concatenate([rng.choice(corners, count // 2, replace=False),
                            rng.choice(mids, count // 2, replace=False)])
    nodes = np.append(nodes, nodes[0]).astype(np.int32)
    forces = rng.normal(0.0, 50.0, size=(len(nodes), 3))
    return nodes, forces


def test_oracle_folds_external_forces_onto_corners(oracle):
    """At rest with noise and drag off, the rhs of the first step is the
    external force folded by linearise_force: corners keep theirs, each end of
    an edge gets half of its midpoint's."""
    s = spec(radius_nm=3.0, calc_noise=0, calc_stokes=0)
    b = oracle.blob_from_spec(s)
    nodes, forces = _forces(s, np.random.default_rng(0))
    b.set_external_forces(nodes, forces)
    b.step(1)
    got = b.rhs()
    want = np.zeros((s.mesh.num_nodes, 3))
    ext = np.zeros_like(want)
    np.add.at(ext, nodes, forces)
    topo = s.mesh.topology
    is_corner = np.zeros(s.mesh.num_nodes, bool)
    is_corner[topo[:, :4]] = True
    want[is_corner] = ext[is_corner]
    mid = {4: (0, 1), 5: (0, 2), 6: (0, 3), 7: (1, 2), 8: (1, 3), 9: (2, 3)}
    seen = set()
    for e in range(len(topo)):
        for j, (a, c) in mid.items():
            m = topo[e, j]
            if m in seen:
                continue
            seen.add(m)
            want[topo[e, a]] += 0.5 * ext[m]
            want[topo[e, c]] += 0.5 * ext[m]
    assert np.allclose(got, want, rtol=1e-12, atol=1e-9 * np.abs(want).max())
    # cleared: the rhs is zero again (the blob is at rest)
    b.set_external_forces()
    b.step(1)
    assert np.abs(b.rhs()).max() < 1e-6 * np.abs(want).max()


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS])
def test_gpu_external_forces_match_oracle_fp64(gpulib, oracle, solver):
    from ffea_gb300.world import World
    s = spec(radius_nm=4.0, solver=solver, pinned=[0, 5])
    ref = oracle.blob_from_spec(s)
    nodes, forces = _forces(s, np.random.default_rng(1))
    with World([s]) as w:
        b = w.blob(0)
        for step in range(6):
            if step == 0:
                b.set_external_forces(nodes, forces)
                ref.set_external_forces(nodes, forces)
            if step == 4:  # cleared
                b.set_external_forces()
                ref.set_external_forces()
            w.run(1)
            assert ref.step(1) == 0
            pos, vel, _ = b.get_nodes()
            rpos, rvel, _ = ref.nodes()
            assert rel(b.rhs(), ref.rhs()) < 1e-9, step
            assert rel(vel, rvel) < 1e-9, step
            assert np.abs(pos - rpos).max() < 1e-10, step


@pytest.mark.gpu
def test_gpu_external_forces_mixed_precision_two_level(gpulib, oracle):
    from ffea_gb300.world import World
    s = spec(radius_nm=6.0, precision=P.PRECISION_MIXED)
    ref = oracle.blob_from_spec(s)
    nodes, forces = _forces(s, np.random.default_rng(2), count=40)
    worst = 0.0
    with World([s], preconditioner=1) as w:
        b = w.blob(0)
        b.set_external_forces(nodes, forces)
        ref.set_external_forces(nodes, forces)
        for _ in range(20):
            w.run(1)
            assert ref.step(1) == 0
            _, vel, _ = b.get_nodes()
            _, rvel, _ = ref.nodes()
            worst = max(worst, rel(vel, rvel), rel(b.rhs(), ref.rhs()))
    assert worst <= 1e-5, worst


@pytest.mark.gpu
def test_gpu_external_forces_reject_bad_nodes(gpulib):
    from ffea_gb300._lib import FfeaGpuError
    from ffea_gb300.world import World
    s = spec(radius_nm=3.0)
    with World([s]) as w:
        with pytest.raises(FfeaGpuError, match="out of range"):
            w.blob(0).set_external_forces([s.mesh.num_nodes], [[1.0, 0.0, 0.0]])
