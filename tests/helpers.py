"""Shared builders for the parity tests."""
from __future__ import annotations

import numpy as np

from ffea_gb300 import params as P
from ffea_gb300.mesh import make_blob, sphere_mesh, cube_mesh


def spec(radius_nm=3.0, seed=1, rng_seed=44, solver=P.SOLVER_NOMASS, precision=P.PRECISION_FP64, epsilon=1e-12,
         pinned=None, cube=None, calc_noise=1, calc_stokes=1, max_iter=1000, shear_mod=3.7e8, bulk_mod=1.1e9,
         kT=None, dt=1e-14):
    mesh = cube_mesh(cube, seed=seed) if cube else sphere_mesh(radius_nm, seed=seed)
    prm = P.SimulationParams.from_si(dt=dt, kT=(P.kT_at(300.0) * P.MESO_ENERGY) if kT is None else kT,
                                     epsilon=epsilon, rng_seed=rng_seed, solver=solver, precision=precision,
                                     calc_noise=calc_noise, calc_stokes=calc_stokes, max_iterations_cg=max_iter)
    return make_blob(mesh, prm, pinned=pinned, shear_mod=shear_mod, bulk_mod=bulk_mod)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)
