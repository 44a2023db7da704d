"""ffea_gpu_measurements (Blob::make_measurements, src/Blob.cpp:951-967,
1363-1527) against the oracle, through the C ABI.

- On the same state: the oracle is given the GPU's node positions and
  velocities, so both evaluate the same formulas on the same numbers.  FP64
  mode: 1e-9 relative (tree against sequential sums); mixed mode: 1e-6
  relative, the element volumes (and so the masses) being stored in FP32,
  and 1e-4 for the strain energy (see _compare).
- Along a trajectory: after 10 steps without state copies, to the parity
  tolerance of the positions (1e-10 absolute in FP64 mode).
- The batch call returns, for every blob, the row of the single-blob call.
"""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import spec

pytestmark = pytest.mark.gpu


def _close(got, want, tol, what):
    assert np.abs(got - want).max() <= tol, (what, got, want, tol)


def _compare(got, want, rtol, s):
    """Relative to the scale of each quantity: positions to the blob's extent,
    the centre of mass to that times the mean of (m_e + 3) / 4, energies with
    a floor of kT per element (the strain energy is 0 at rest, where both
    sides hold round-off only).  In mixed mode the strain energy is formed
    from FP32 rest-state inverses and volumes: first order in their round-off
    against second order in the strain, hence 1e-4 there."""
    e_rtol = rtol if rtol < 1e-6 else 1e-4
    pos = np.asarray(s.mesh.pos).reshape(-1, 3)
    ext = np.abs(pos).max()
    c = pos[s.mesh.topology[:, :4]]
    vol = np.abs(np.einsum("ij,ij->i", c[:, 1] - c[:, 0], np.cross(c[:, 2] - c[:, 0], c[:, 3] - c[:, 0]))) / 6
    com_scale = ext * np.mean(vol * s.material[:, 0] + 3) / 4
    e_floor = s.params.kT * len(s.mesh.topology)
    _close(got[0], want[0], rtol * max(abs(want[0]), e_floor), "kinetic")
    _close(got[1], want[1], e_rtol * max(abs(want[1]), e_floor), "strain")
    _close(got[2:5], want[2:5], rtol * ext, "centroid")
    _close(got[5], want[5], rtol * want[5], "rmsd")
    _close(got[6:9], want[6:9], rtol * com_scale, "centre of mass")
    _close(got[9:12], want[9:12], rtol * np.abs(want[9:12]).max(), "angular momentum")


@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS, P.SOLVER_LUMPED])
@pytest.mark.parametrize("precision", [P.PRECISION_FP64, P.PRECISION_MIXED])
def test_measurements_match_oracle_on_the_same_state(gpulib, oracle, solver, precision):
    from ffea_gb300.world import World
    s = spec(radius_nm=4.0, solver=solver, precision=precision, epsilon=1e-6 if precision else 1e-12)
    ref = oracle.blob_from_spec(s)
    rtol = 1e-9 if precision == P.PRECISION_FP64 else 1e-6
    with World([s]) as w:
        b = w.blob(0)
        m0 = w.measurements()[0]
        assert m0[5] == 0.0  # nothing has moved: RMSD 0 exactly
        _compare(m0, ref.measurements(), rtol, s)
        w.run(10)
        pos, vel, _ = b.get_nodes()
        ref.set_nodes(pos, vel)
        got, want = w.measurements()[0], ref.measurements()
        assert got[5] > 0
        if solver == P.SOLVER_NOMASS:
            assert got[0] == 0.0 and not got[9:12].any()
        else:
            assert np.abs(got[9:12]).max() > 0
        _compare(got, want, rtol, s)
        d = b.measurements()
        assert d["rmsd"] == got[5] and np.array_equal(d["angmom"], got[9:12])


@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS])
def test_measurements_along_a_trajectory_fp64(gpulib, oracle, solver):
    from ffea_gb300.world import World
    s = spec(radius_nm=3.0, solver=solver)
    ref = oracle.blob_from_spec(s)
    with World([s]) as w:
        w.run(10)
        assert ref.step(10) == 0
        got, want = w.measurements()[0], ref.measurements()
    # positions agree to 1e-10 absolute (meso) in FP64 mode
    _close(got[2:5], want[2:5], 1e-10, "centroid")
    _close(got[6:9], want[6:9], 1e-10 * np.abs(want[6:9]).max() / np.abs(want[2:5]).max() + 1e-10, "centre of mass")
    _close(got[5], want[5], 1e-10, "rmsd")
    _close(got[0:2], want[0:2], 1e-6 * np.abs(want[0:2]).max(), "energies")


def test_batch_rows_equal_single_blob_rows(gpulib, oracle):
    from ffea_gb300.world import World
    specs = [spec(radius_nm=r, seed=i, rng_seed=70 + i, solver=sv, precision=P.PRECISION_MIXED, epsilon=1e-6)
             for i, (r, sv) in enumerate([(2.5, P.SOLVER_NOMASS), (4.0, P.SOLVER_MASS), (3.0, P.SOLVER_LUMPED)])]
    with World(specs) as w:
        w.run(5)
        rows = w.measurements()
        for i, s in enumerate(specs):
            single = w.blob(i).measurements()
            assert single["kinetic"] == rows[i, 0] and single["strain"] == rows[i, 1]
            assert np.array_equal(single["centroid"], rows[i, 2:5]) and np.array_equal(single["com"], rows[i, 6:9])
            ref = oracle.blob_from_spec(s)
            pos, vel, _ = w.blob(i).get_nodes()
            ref.set_nodes(pos, vel)
            _compare(rows[i], ref.measurements(), 1e-6, s)
