"""Simulation parameters and FFEA's unit system.

Mirrors the subset of ``SimulationParams`` that the blob update reads
(src/SimulationParams.cpp:222-405) and the meso unit system of
include/dimensions.h:30-41.  Values are kept in FFEA meso units, exactly as
``SimulationParams::assign`` leaves them after parsing a ``.ffea`` script.
"""
from __future__ import annotations

import dataclasses

import numpy as np

# include/dimensions.h:30-41
MESO_LENGTH = 1.7e-10
MESO_ENERGY = 4.141945559999999e-21
MESO_MASS = 1.994307387553024e-26
MESO_VOLUME = 4.913e-30
MESO_TIME = 3.7302915560886126e-13
MESO_PRESSURE = 8.4305832688784826e8
MESO_VELOCITY = 4.5572845297447225e2

# include/mat_vec_types.h:54
PI = 3.141592653589793238462643383279502884197169399375105820974944592307816406286208998628034825342117067982148

SOLVER_NOMASS = 0   # <solver = CG_nomass>  (src/World.cpp:2545-2562)
SOLVER_MASS = 1     # <solver = CG>
SOLVER_LUMPED = 2   # <solver = masslumped>: MassLumpedSolver

PRECISION_FP64 = 0   # every kernel in FP64 (parity mode)
PRECISION_MIXED = 1  # FP32 element forces + SpMV, FP64 positions / dots / residuals

BOLTZMANN = 1.380649e-23


@dataclasses.dataclass
class SimulationParams:
    """The blob-update parameters, in meso units.

    Defaults follow SimulationParams::SimulationParams (src/SimulationParams.cpp:26-77)
    for the fields the path uses.
    """

    dt: float = 1e-14 / MESO_TIME
    kT: float = 4.11e-21 / MESO_ENERGY
    epsilon2: float = 0.01
    max_iterations_cg: int = 1000
    calc_noise: int = 1
    calc_stokes: int = 1
    stokes_visc: float = 1e-3 / (MESO_PRESSURE * MESO_TIME)
    rng_seed: int = 0
    solver: int = SOLVER_NOMASS
    precision: int = PRECISION_MIXED

    @classmethod
    def from_si(cls, dt: float = 1e-14, kT: float = 4.11e-21, epsilon: float = 1e-6,
                max_iterations_cg: int = 1000, calc_noise: int = 1, calc_stokes: int = 1,
                stokes_visc: float = 1e-3, rng_seed: int = 0, solver: int = SOLVER_NOMASS,
                precision: int = PRECISION_MIXED) -> "SimulationParams":
        """Convert script values (SI) the way SimulationParams::assign does:
        dt /= time (src/SimulationParams.cpp:222-227), epsilon2 = epsilon^2
        (:228-231), kT /= Energy (:336-340), stokes_visc /= pressure*time (:402-405)."""
        return cls(dt=dt / MESO_TIME, kT=kT / MESO_ENERGY, epsilon2=epsilon * epsilon,
                   max_iterations_cg=int(max_iterations_cg), calc_noise=int(calc_noise),
                   calc_stokes=int(calc_stokes), stokes_visc=stokes_visc / (MESO_PRESSURE * MESO_TIME),
                   rng_seed=int(rng_seed), solver=int(solver), precision=int(precision))


def material_si_to_meso(density, shear_visc, bulk_visc, shear_mod, bulk_mod) -> np.ndarray:
    """Per-element (rho, A, B, G, E) in meso units, as Blob::load_material_params
    computes them (src/Blob.cpp:2862-2867).

    The second viscosity coefficient subtracts the SI shear viscosity from a
    meso-unit bulk viscosity (src/Blob.cpp:2865); that expression is kept as
    is so results match the reference.
    """
    density = np.asarray(density, dtype=np.float64)
    shear_visc = np.asarray(shear_visc, dtype=np.float64)
    bulk_visc = np.asarray(bulk_visc, dtype=np.float64)
    shear_mod = np.asarray(shear_mod, dtype=np.float64)
    bulk_mod = np.asarray(bulk_mod, dtype=np.float64)
    rho = density * MESO_VOLUME / MESO_MASS
    A = shear_visc / (MESO_PRESSURE * MESO_TIME)
    B = bulk_visc / (MESO_PRESSURE * MESO_TIME) - (2.0 / 3.0) * shear_visc
    G = shear_mod / MESO_PRESSURE
    E = bulk_mod / MESO_PRESSURE
    return np.ascontiguousarray(np.stack(np.broadcast_arrays(rho, A, B, G, E), axis=-1), dtype=np.float64)


def stokes_drag(stokes_radius_meso: np.ndarray, stokes_visc_meso: float, calc_stokes: int = 1) -> np.ndarray:
    """6*pi*eta*r per node (src/Blob.cpp:408-412), evaluated left to right."""
    r = np.asarray(stokes_radius_meso, dtype=np.float64)
    if not calc_stokes:
        return np.zeros_like(r)
    return 6.0 * PI * stokes_visc_meso * r


def kT_at(temperature_k: float = 300.0) -> float:
    """kT in meso units at a temperature (k_B T / Energy unit)."""
    return BOLTZMANN * temperature_k / MESO_ENERGY


def nm(x_nm: float) -> float:
    """Nanometres to meso length units."""
    return x_nm * 1e-9 / MESO_LENGTH


__all__ = [
    "SimulationParams", "material_si_to_meso", "stokes_drag", "kT_at", "nm",
    "MESO_LENGTH", "MESO_ENERGY", "MESO_MASS", "MESO_VOLUME", "MESO_TIME", "MESO_PRESSURE",
    "SOLVER_NOMASS", "SOLVER_MASS", "SOLVER_LUMPED", "PRECISION_FP64", "PRECISION_MIXED", "PI",
]
