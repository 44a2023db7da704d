"""Generate the golden vectors in tests/golden/*.npz from FFEA's own objects.

Runs the reference harness (oracle/_ref/libffea_ref.so: FFEA's
tetra_element_linear, NoMassCGSolver, ConjugateGradientSolver,
MassLumpedSolver, RngStream ...
compiled from the FFEA sources by oracle/Makefile) on small synthetic blobs and
stores inputs and per-step outputs.  Needs the FFEA source tree (only present
where the reference is mounted); the fixtures it writes travel with the repo.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ffea_gb300 import params as P  # noqa: E402
from ffea_gb300.mesh import make_blob, sphere_mesh, cube_mesh  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    # name: (mesh builder, solver, pinned, rng_seed, steps)
    "nomass_sphere4": (lambda: sphere_mesh(4.0, seed=3), P.SOLVER_NOMASS, None, 7, 6),
    "mass_sphere4": (lambda: sphere_mesh(4.0, seed=3), P.SOLVER_MASS, None, 11, 6),
    "nomass_cube3_pinned": (lambda: cube_mesh(3, seed=5), P.SOLVER_NOMASS, [0, 1, 2, 5], 44, 6),
    "mass_cube3_pinned": (lambda: cube_mesh(3, seed=5), P.SOLVER_MASS, [0, 7], 44, 6),
    "lumped_cube3_pinned": (lambda: cube_mesh(3, seed=5), P.SOLVER_LUMPED, [0, 7], 9, 6),
}
RECORD_STEPS = (1, 2, 6)


def make(name):
    build, solver, pinned, seed, steps = CASES[name]
    mesh = build()
    prm = P.SimulationParams.from_si(kT=P.kT_at(300.0) * P.MESO_ENERGY, epsilon=1e-12, rng_seed=seed, solver=solver,
                                     precision=P.PRECISION_FP64)
    spec = make_blob(mesh, prm, pinned=pinned)
    ref = O.blob_from_spec(spec, impl="ref")
    out = dict(pos0=mesh.pos, topology=mesh.topology, material=spec.material, drag=spec.drag,
               pinned=spec.pinned, num_linear=mesh.num_linear,
               fparams=np.array([prm.dt, prm.kT, prm.epsilon2]),
               iparams=np.array([prm.max_iterations_cg, prm.calc_noise, prm.calc_stokes, solver, seed]),
               rng0=ref.rng_state())
    done = 0
    for s in RECORD_STEPS:
        assert ref.step(s - done) == 0
        done = s
        pos, vel, force = ref.nodes()
        out[f"pos_{s}"] = pos
        out[f"vel_{s}"] = vel
        out[f"force_{s}"] = force
        out[f"rhs_{s}"] = ref.rhs()
        out[f"efrc_{s}"] = ref.element_forces()
        out[f"rng_{s}"] = ref.rng_state()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def main():
    O.build(ref=True)
    if not O.ref_available():
        raise SystemExit("the reference objects could not be built (FFEA sources missing)")
    names = sys.argv[1:] or list(CASES)  # e.g. make_golden.py lumped_cube3_pinned
    for name in names:
        make(name)
        print("wrote", name)


if __name__ == "__main__":
    main()
