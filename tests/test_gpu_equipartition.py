"""Equipartition of an ensemble (GPU): with thermal noise on, the mean strain
energy of a NoMass blob settles at kT (3 N - 6) / 2 -- half kT per internal
degree of freedom of its N corner nodes -- which is the reference's own
statistical check (tests/physics/sphere_63_120_nomass/averages.py:51-55,
3 % on the mean strain energy, epsilon 0.01).

Here: 32 replicas of one mesh with distinct RNG seeds in one batch (one
launch sequence per step), 2,000 steps of burn-in, then 24 samples 400
steps apart (about 1.5 relaxation times eta/G = 270 steps), mixed
precision.  The per-sample spread of the strain energy is sqrt(2/(3N-6)),
about 5.5 % here, so the mean of 768 samples is good to ~0.2 %; the test
uses the reference's 3 %."""
import numpy as np
import pytest

from ffea_gb300 import params as P
from ffea_gb300.mesh import make_blob, sphere_mesh

pytestmark = pytest.mark.gpu


def test_strain_energy_equipartition(gpulib):
    from ffea_gb300.world import World
    mesh = sphere_mesh(7.5, cell_nm=2.5, seed=3)
    kT = P.kT_at(300.0) * P.MESO_ENERGY
    specs = []
    for r in range(32):
        prm = P.SimulationParams.from_si(dt=1e-14, kT=kT, epsilon=0.01, rng_seed=1000 + r, solver=P.SOLVER_NOMASS,
                                         precision=P.PRECISION_MIXED)
        specs.append(make_blob(mesh, prm))
    n = mesh.num_linear
    expected = specs[0].params.kT * (3 * n - 6) / 2
    samples = []
    with World(specs) as w:
        w.run(2000)
        for _ in range(24):
            w.run(400)
            samples.append([w.blob(i).energies()[0] for i in range(len(specs))])
            for i in range(len(specs)):
                assert w.blob(i).status()["fail_bits"] == 0
    se = np.asarray(samples)
    ratio = se.mean() / expected
    assert abs(ratio - 1.0) < 0.03, (ratio, se.mean(), expected)


def test_strain_energy_equipartition_two_level_many_replicas(gpulib):
    """The larger-ensemble check: 96 replicas (more than 64, so the solve
    reduces at the last-arriving CTA, in the memory-resident kernel with the
    two-level preconditioner) to 2 % of kT (3N - 6) / 2, with every solve at
    relative residual 1e-6 confirmed by the FP64 true residual."""
    from ffea_gb300.world import World
    mesh = sphere_mesh(7.5, cell_nm=2.5, seed=3)
    kT = P.kT_at(300.0) * P.MESO_ENERGY
    specs = [make_blob(mesh, P.SimulationParams.from_si(dt=1e-14, kT=kT, epsilon=1e-6, rng_seed=5000 + r,
                                                        solver=P.SOLVER_NOMASS, precision=P.PRECISION_MIXED))
             for r in range(96)]
    n = mesh.num_linear
    expected = specs[0].params.kT * (3 * n - 6) / 2
    samples = []
    with World(specs, true_residual=True, preconditioner=1) as w:
        assert w.preconditioner() == 1
        w.run(2000)
        for _ in range(16):
            w.run(400)
            samples.append([w.blob(i).energies()[0] for i in range(len(specs))])
            for i in range(len(specs)):
                st = w.blob(i).status()
                assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, (i, st)
    ratio = np.asarray(samples).mean() / expected
    assert abs(ratio - 1.0) < 0.02, ratio
