"""Diffusion of free blobs (GPU): the reference's statistical checks
tests/physics/sphere_diffusion/diffusion_nomass.py:63-79 and
diffusion_mass.py:60-79.

- CG_nomass: the centroid displacement (ffea_gpu_measurements) over tau
  steps has
  <dr^2> = 6 (kT / zeta) tau dt, zeta = sum of the node drags 6 pi eta r
  (the rigid translation feels the summed drag; the internal forces sum to
  zero).  The reference's tolerance, 5 %.
- CG (mass): the blob's centre moves as a free Brownian particle of mass m =
  sum rho V_e and friction zeta, <dr^2> = 6 (kT / zeta) (t - (m / zeta)
  (1 - exp(-zeta t / m))), t = tau dt (Ornstein-Uhlenbeck in equilibrium).
  The reference uses its short-time limit 3 (kT / m) t^2, valid for
  t << m / zeta; here m / zeta is about 930 steps and tau 100, where the
  limit is 3.5 % high, so the full expression is the expectation.  The
  reference's tolerance, 10 %.  The centre is the true centre of mass,
  sum m_e (corner mean) / m from the node positions: the node centroid of
  a mass blob also carries its internal vibrations (nodes of unequal mass),
  which add 2 var(centroid - centre of mass), about 20 % of <dr^2> at 100
  steps here, and vanish against it at 1,000 steps (measured: centroid 1.19
  and 0.97 of the expectation, centre of mass 0.98 and 1.00).

Replicas of one mesh with distinct RNG seeds run in one batch; the seeds are
fixed, so the test is deterministic.  NoMass: 96 replicas x 30 windows of 400
steps after 400 steps of burn-in, 2,880 samples (the mean of |dr|^2 over
3-d Gaussian samples has relative spread sqrt(2/3)/sqrt(n) = 1.5 %).  Mass:
the velocity stays correlated over m / zeta, so 128 replicas x 6 windows of
100 steps spaced 2,000 apart after 5,000 steps of burn-in (5 m / zeta), 768
samples (2.9 %)."""
import numpy as np
import pytest

from ffea_gb300 import params as P
from ffea_gb300.mesh import make_blob, sphere_mesh

pytestmark = pytest.mark.gpu


def _specs(solver, n, seed0):
    mesh = sphere_mesh(7.5, cell_nm=2.5, seed=3)
    kT = P.kT_at(300.0) * P.MESO_ENERGY
    return [make_blob(mesh, P.SimulationParams.from_si(dt=1e-14, kT=kT, epsilon=1e-6, rng_seed=seed0 + r,
                                                       solver=solver, precision=P.PRECISION_MIXED))
            for r in range(n)]


def _mass_and_drag(s):
    c = s.mesh.pos[s.mesh.topology[:, :4]]
    vol = np.abs(np.einsum("ij,ij->i", c[:, 1] - c[:, 0], np.cross(c[:, 2] - c[:, 0], c[:, 3] - c[:, 0]))) / 6
    return float((vol * s.material[:, 0]).sum()), float(s.drag.sum())


def _centroids(w):
    return w.measurements()[:, 2:5].copy()


def _centres_of_mass(w, s):
    topo = s.mesh.topology[:, :4]
    c = s.mesh.pos[topo]
    me = np.abs(np.einsum("ij,ij->i", c[:, 1] - c[:, 0], np.cross(c[:, 2] - c[:, 0], c[:, 3] - c[:, 0]))) / 6
    me = me * s.material[:, 0]
    out = []
    for i in range(w.num_blobs):
        pos = w.blob(i).get_nodes()[0]
        out.append((me[:, None] * pos[topo].mean(axis=1)).sum(axis=0) / me.sum())
    return np.array(out)


def test_nomass_centroid_diffusion(gpulib):
    from ffea_gb300.world import World
    specs = _specs(P.SOLVER_NOMASS, 96, 7000)
    p = specs[0].params
    _, zeta = _mass_and_drag(specs[0])
    tau = 400
    expected = 6 * (p.kT / zeta) * tau * p.dt
    r2 = []
    with World(specs) as w:
        w.run(400)
        c0 = _centroids(w)
        for _ in range(30):
            w.run(tau)
            c1 = _centroids(w)
            r2.append(((c1 - c0) ** 2).sum(axis=1))
            c0 = c1
        for i in range(len(specs)):
            assert w.blob(i).status()["fail_bits"] == 0
    r2 = np.concatenate(r2)
    ratio = r2.mean() / expected
    assert abs(ratio - 1.0) <= 0.05, (ratio, r2.mean(), expected)


def test_mass_centroid_diffusion(gpulib):
    from ffea_gb300.world import World
    specs = _specs(P.SOLVER_MASS, 128, 9000)
    p = specs[0].params
    m, zeta = _mass_and_drag(specs[0])
    tau = 100
    t = tau * p.dt
    gamma = zeta / m
    expected = 6 * (p.kT / zeta) * (t - (1 - np.exp(-gamma * t)) / gamma)
    ballistic = 3 * (p.kT / m) * t * t
    assert 1.0 < ballistic / expected < 1.1  # the reference's limit is close, not exact, here
    r2 = []
    with World(specs) as w:
        w.run(5000)
        for _ in range(6):
            c0 = _centres_of_mass(w, specs[0])
            w.run(tau)
            r2.append(((_centres_of_mass(w, specs[0]) - c0) ** 2).sum(axis=1))
            w.run(2000 - tau)
        for i in range(len(specs)):
            assert w.blob(i).status()["fail_bits"] == 0
    r2 = np.concatenate(r2)
    ratio = r2.mean() / expected
    assert abs(ratio - 1.0) <= 0.10, (ratio, r2.mean(), expected, ballistic)
