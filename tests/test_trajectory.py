"""FFEA trajectory and checkpoint files, and restarts from them.

The reference's own restart test (tests/physics/sphere_63_120_nomass_restart/
checkRuns.py:33-83) runs 10 steps straight and 5 + 5 with a restart, and
requires the two final checkpoints to be identical and the measurements to
agree to 5e-4 relative (the trajectory holds positions to %e precision).
The same check here, on the oracle (CPU) and on the GPU handle."""
import os

import numpy as np
import pytest

from ffea_gb300 import params as P
from ffea_gb300 import trajectory as T
from tests.helpers import spec


class _OracleWorld:
    """The oracle blob behind the World/Blob calls the Recorder makes."""

    def __init__(self, oracle, s):
        self.ob = oracle.blob_from_spec(s)
        self.num_blobs = 1
        self.rng_mode = 0
        self.params = [s.params]

    def measurements(self):
        return self.ob.measurements()[None, :]

    def run(self, n):
        assert self.ob.step(n) == 0

    def blob(self, i):
        ob = self.ob

        class _B:
            n = ob.n

            def get_nodes(self):
                return ob.nodes()

            def set_nodes(self, pos, vel):
                ob.set_nodes(pos, vel)

            def rng_state(self):
                return ob.rng_state()

            def set_rng_state(self, st):
                ob.set_rng_state(st)
        return _B()


def test_header_and_frame_text(tmp_path):
    """The exact text of World::init's header and a frame
    (src/World.cpp:532-548, 4164-4177; src/Blob.cpp:1154-1168)."""
    path = tmp_path / "t.ftj"
    pos = np.array([[1.0, 2.0, 3.0], [-4.5, 0.0, 1e-3]])
    vel = np.array([[0.1, 0.2, 0.3], [0.0, -1.0, 2.0]])
    frc = np.array([[5.0, 6.0, 7.0], [8.0, 9.0, 10.0]])
    with open(path, "w") as fh:
        T.write_header(fh, [2])
        T.write_frame(fh, 7, [(pos, vel, frc)], [P.SOLVER_MASS])
        T.write_frame(fh, 8, [(pos, vel, frc)], [P.SOLVER_NOMASS])
    lines = path.read_text().split("\n")
    assert lines[:8] == ["FFEA_trajectory_file", "", "Initialisation:", "Number of Blobs 1",
                         "Number of Conformations 1", "Blob 0:\tConformation 0 Nodes 2\t", "", "*"]
    assert lines[8:10] == ["Blob 0, Conformation 0, step 7", "DYNAMIC"]
    L, V, F = P.MESO_LENGTH, P.MESO_VELOCITY, T.MESO_FORCE
    want = "%e %e %e %e %e %e %e %e %e %e" % (1.0 * L, 2.0 * L, 3.0 * L, 0.1 * V, 0.2 * V, 0.3 * V, 0.0,
                                              5.0 * F, 6.0 * F, 7.0 * F)
    assert lines[10] == want
    assert lines[12:16] == ["*", "Conformation Changes:", "Blob 0: Conformation 0 -> Conformation 0", "*"]
    # CG_nomass: positions, then zeros
    assert lines[18] == "%e %e %e %e %e %e %e %e %e %e" % (L, 2 * L, 3 * L, 0, 0, 0, 0, 0, 0, 0)
    assert "e+" in lines[10] or "e-" in lines[10]


def test_last_complete_frame_is_read(tmp_path):
    path = tmp_path / "t.ftj"
    rng = np.random.default_rng(0)
    frames = [(rng.normal(size=(3, 3)), rng.normal(size=(3, 3)), rng.normal(size=(3, 3))) for _ in range(2)]
    with open(path, "w") as fh:
        T.write_header(fh, [3, 3])
        T.write_frame(fh, 0, [frames[0], frames[1]], [1, 1])
        T.write_frame(fh, 5, [frames[1], frames[0]], [1, 1])
        fh.write("Blob 0, Conformation 0, step 10\nDYNAMIC\n1e0 2e0\n")  # cut off mid-frame
    step, got = T.read_last_frame(str(path), [3, 3])
    assert step == 5
    for (p, v), (fp, fv, _) in zip(got, [frames[1], frames[0]]):
        assert np.allclose(p, fp, rtol=1e-6) and np.allclose(v, fv, rtol=1e-6)


def test_checkpoint_round_trip(tmp_path):
    path = str(tmp_path / "c.fcp")
    st = [np.array([1, 2, 3, 4294967086, 5, 6], np.uint64), np.array([7, 8, 9, 10, 11, 12], np.uint64)]
    T.write_checkpoint(path, st)
    assert open(path).read() == ("RNGStreams dedicated to the thermal stress: 2\n"
                                 "1 2 3 4294967086 5 6\n7 8 9 10 11 12\n")
    got = T.read_checkpoint(path)
    assert all(np.array_equal(a, b) for a, b in zip(got, st))


def _restart_identity(make_world, tmp_path, solvers, check=5):
    a_t, a_c, a_m = str(tmp_path / "a.ftj"), str(tmp_path / "a.fcp"), str(tmp_path / "a_measurement.out")
    b_t, b_c, b_m = str(tmp_path / "b.ftj"), str(tmp_path / "b.fcp"), str(tmp_path / "b_measurement.out")
    wa = make_world()
    T.Recorder(wa, a_t, a_c, solvers, check=check, measurement=a_m).run(2 * check)
    wb = make_world()
    T.Recorder(wb, b_t, b_c, solvers, check=check, measurement=b_m).run(check)
    wc = make_world()  # a fresh process's handle, continued from b's files
    T.Recorder(wc, b_t, b_c, solvers, check=check, restart=True, measurement=b_m).run(check)
    # checkRuns.py:33-46: the final checkpoints are identical
    assert open(a_c).read() == open(b_c).read()
    # checkRuns.py:48-84: the measurements agree to 5e-4 relative (every row
    # here; the restart read positions and velocities at %e precision)
    ma, mb = T.read_measurements(a_m), T.read_measurements(b_m)
    assert list(ma) == list(mb) and len(ma["Time"]) == len(mb["Time"]) == 3
    for k in ma:
        a, b = ma[k], mb[k]
        d = np.abs(b - a) / np.where(a == 0, 1.0, np.abs(a))
        assert d.max() <= 5e-4, (k, a, b)
    # the same frames were written, and the final states agree to the
    # precision the trajectory stores positions with (checkRuns.py: 5e-4)
    sa, fa = T.read_last_frame(a_t, [wa.blob(0).n])
    sb, fb = T.read_last_frame(b_t, [wc.blob(0).n])
    assert sa == sb == 2 * check
    pa, pb = fa[0][0], fb[0][0]
    assert np.abs(pa - pb).max() <= 5e-4 * np.abs(pa).max()
    assert open(a_t).read().count("step %d\n" % check) == open(b_t).read().count("step %d\n" % check) == 1
    return wa, wc


def test_restart_identity_oracle(oracle, tmp_path):
    s = spec(radius_nm=3.0, epsilon=1e-6)
    _restart_identity(lambda: _OracleWorld(oracle, s), tmp_path, [s.params.solver])


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS])
def test_restart_identity_gpu(gpulib, tmp_path, solver):
    from ffea_gb300.world import World
    s = spec(radius_nm=4.0, solver=solver, precision=P.PRECISION_MIXED, epsilon=1e-6)
    made = []

    def make():
        w = World([s])
        made.append(w)
        return w
    try:
        _restart_identity(make, tmp_path, [solver])
    finally:
        for w in made:
            w.close()
    assert os.path.exists(tmp_path / "b.fcp")
