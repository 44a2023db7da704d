"""Blob::make_measurements and the measurement file (CPU).

- The oracle's C restatement of the centroid, RMSD, centre of mass and
  angular momentum (src/Blob.cpp:951-967, 1363-1527) against a numpy
  evaluation of the same formulas on the oracle's own node state.
- The measurement file: header, columns and World::make_measurements'
  node-weighted totals (src/World.cpp:4282-4366), read back the way
  ffeatools' FFEA_measurement.load_global reads it, and the truncation a
  restart does.
"""
import numpy as np
import pytest

from ffea_gb300 import params as P
from ffea_gb300 import trajectory as T
from tests.helpers import spec

MID = [(4, 0, 1), (5, 0, 2), (6, 0, 3), (7, 1, 2), (8, 1, 3), (9, 2, 3)]
MM = np.full((4, 4), 0.05) + 0.05 * np.eye(4)


def _numpy_measurements(s, pos, vel):
    """Centroid, RMSD, centre of mass, angular momentum from the formulas."""
    topo = s.mesh.topology
    pos0 = np.array(s.mesh.pos, dtype=float).reshape(-1, 3)
    for e in range(len(topo)):  # Blob::init's linearisation before set_pos_0
        for m, a, b in MID:
            pos0[topo[e, m]] = .5 * (pos0[topo[e, a]] + pos0[topo[e, b]])
    c = pos0[topo[:, :4]]
    vol0 = np.einsum("ij,ij->i", c[:, 1] - c[:, 0], np.cross(c[:, 2] - c[:, 0], c[:, 3] - c[:, 0])) / 6.0
    mass = np.abs(vol0) * s.material[:, 0]
    p = pos[topo[:, :4]]
    com = ((mass[:, None] * p[:, 0] + p[:, 1] + p[:, 2] + p[:, 3]) / 4).sum(axis=0) / len(topo)
    r = p - com
    v = vel[topo[:, :4]]
    # sum_ij MM_ij r_j x v_i per element
    lm = np.einsum("ij,ejk->eik", MM, r)  # (MM r)_i
    ang = (mass[:, None] * np.cross(lm, v).sum(axis=1)).sum(axis=0)
    if s.params.solver == P.SOLVER_NOMASS:
        ang = np.zeros(3)
    cog = pos.mean(axis=0)
    rmsd = np.sqrt(((pos - pos0) ** 2).sum() / len(pos))
    return cog, rmsd, com, ang


@pytest.mark.parametrize("solver", [P.SOLVER_NOMASS, P.SOLVER_MASS, P.SOLVER_LUMPED])
def test_oracle_measurements_match_formulas(oracle, solver):
    s = spec(radius_nm=3.0, solver=solver, epsilon=1e-6)
    b = oracle.blob_from_spec(s)
    m0 = b.measurements()
    assert m0[5] == 0.0  # RMSD from the creation positions
    assert b.step(4) == 0
    pos, vel, _ = b.nodes()
    m = b.measurements()
    cog, rmsd, com, ang = _numpy_measurements(s, pos, vel)
    strain, kinetic = b.energies()
    assert m[0] == kinetic and m[1] == strain
    np.testing.assert_allclose(m[2:5], cog, rtol=1e-12)
    assert rmsd > 0 and abs(m[5] - rmsd) <= 1e-12 * rmsd
    np.testing.assert_allclose(m[6:9], com, rtol=1e-12)
    if solver == P.SOLVER_NOMASS:
        assert not m[9:12].any() and kinetic == 0.0
    else:
        assert np.abs(ang).max() > 0
        np.testing.assert_allclose(m[9:12], ang, rtol=1e-9, atol=1e-12 * np.abs(ang).max())


def test_centre_of_mass_keeps_the_reference_parenthesisation(oracle):
    """Blob::get_CoM multiplies only the first corner by the element mass
    (src/Blob.cpp:958-960) and divides by the element count: a rigid shift d
    of every node moves it by d (m_e + 3) / 4 averaged over elements, not by d."""
    s = spec(radius_nm=3.0, solver=P.SOLVER_MASS, epsilon=1e-6)
    b = oracle.blob_from_spec(s)
    pos, vel, _ = b.nodes()
    before = b.measurements()
    d = np.array([0.5, -1.0, 2.0])
    b.set_nodes(pos + d, vel)
    after = b.measurements()
    _, _, com0, _ = _numpy_measurements(s, pos, vel)
    _, _, com1, _ = _numpy_measurements(s, pos + d, vel)
    np.testing.assert_allclose(after[6:9] - before[6:9], com1 - com0, rtol=1e-9)
    assert not np.allclose(after[6:9] - before[6:9], d)
    np.testing.assert_allclose(after[2:5] - before[2:5], d, rtol=1e-12)  # the centroid moves by d
    assert abs(after[5] - np.linalg.norm(d)) <= 1e-12 * np.linalg.norm(d)  # RMSD of a rigid shift


def test_measurement_file_totals_and_reader(tmp_path):
    path = str(tmp_path / "x_measurement.out")
    prm = spec(radius_nm=2.5).params
    nodes = [100, 300]
    meas = np.zeros((2, 12))
    meas[:, 0] = [2.0, 3.0]      # kinetic
    meas[:, 1] = [10.0, 20.0]    # strain
    meas[0, 2:5] = [1.0, 2.0, 3.0]
    meas[1, 2:5] = [5.0, 6.0, 7.0]
    meas[:, 5] = [0.1, 0.2]      # RMSD
    with open(path, "w") as fh:
        T.write_measurement_header(fh, prm, 2, True, num_steps=20, check=10)
        fh.write(T.measurement_row(0, prm.dt, meas, nodes, True))
        fh.write(T.measurement_row(10, prm.dt, meas, nodes, True))
    text = open(path).read()
    assert text.startswith("FFEA Global Measurement File\n\nSimulation Details:\n")
    assert "\nParameters:\n" in text and "\tnum_blobs = 2\n" in text
    head = text.split("Measurements:\n")[1].split("\n")[0]
    assert head == "%-14s" * 7 % ("Time", "KineticEnergy", "StrainEnergy", "Centroid.x", "Centroid.y",
                                  "Centroid.z", "RMSD")
    got = T.read_measurements(path)
    assert list(got) == ["Time", "KineticEnergy", "StrainEnergy", "Centroid.x", "Centroid.y", "Centroid.z", "RMSD"]
    np.testing.assert_allclose(got["Time"], [0.0, 10 * prm.dt * P.MESO_TIME], rtol=1e-6)
    np.testing.assert_allclose(got["KineticEnergy"], 5.0 * P.MESO_ENERGY, rtol=1e-6)
    np.testing.assert_allclose(got["StrainEnergy"], 30.0 * P.MESO_ENERGY, rtol=1e-6)
    np.testing.assert_allclose(got["Centroid.x"], (100 * 1.0 + 300 * 5.0) / 400 * P.MESO_LENGTH, rtol=1e-6)
    rmsd = np.sqrt((100 * 0.01 + 300 * 0.04) / 400) * P.MESO_LENGTH
    np.testing.assert_allclose(got["RMSD"], rmsd, rtol=1e-6)
    # no kinetic column without mass; a restart keeps the rows before it
    with open(path, "w") as fh:
        T.write_measurement_header(fh, prm, 2, False)
        for step in range(0, 50, 10):
            fh.write(T.measurement_row(step, prm.dt, meas, nodes, False))
    assert "KineticEnergy" not in T.read_measurements(path)
    T._truncate_measurements(path, 3)
    got = T.read_measurements(path)
    assert len(got["Time"]) == 3 and got["Time"][-1] == pytest.approx(20 * prm.dt * P.MESO_TIME, rel=1e-6)
