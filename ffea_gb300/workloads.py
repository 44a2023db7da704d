"""The synthetic blob workloads the measurements and the large parity tests use.

Every workload is a set of NoMass blobs with one set of physics: density
1.5e3 kg/m^3, shear/bulk modulus 3.7e8/1.1e9 Pa (scaled per blob in the
ensemble), shear/bulk viscosity 1e-3 Pa s, kT at 300 K, dt 1e-14 s, thermal
noise and Stokes drag on.  Meshes are Freudenthal-split cube grids at a
1.25 nm cell cut to spheres (ffea_gb300.mesh.sphere_mesh), positions jittered
from a seed.  Seeded synthetic inputs stand in for protein meshes.

  sphere10     16^3-cell grid, 10 nm sphere (2,771 corner nodes)
  sphere20     32^3-cell grid, 20 nm sphere (19,663)
  sphere40     64^3-cell grid, 40 nm sphere (146,737): the single-blob NoMass run
  sphere61     98^3-cell grid, 61.25 nm sphere (514,965): the ~500k-node blob
  replicas256  256 replicas of sphere20, one RNG stream each
  ensemble64   64 blobs, radii log-uniform 5-40 nm, moduli x U[0.5, 2]
  heldout      the learned preconditioner's held-out family: 10, 20, 30, 40, 50 nm
"""
from __future__ import annotations

import numpy as np

WORKLOADS = {
    "sphere40": dict(radius_nm=40.0, cell_nm=1.25, desc="64^3-cell Freudenthal grid cut to a 40 nm sphere"),
    "sphere20": dict(radius_nm=20.0, cell_nm=1.25, desc="32^3-cell Freudenthal grid cut to a 20 nm sphere"),
    "sphere10": dict(radius_nm=10.0, cell_nm=1.25, desc="16^3-cell Freudenthal grid cut to a 10 nm sphere"),
    "sphere61": dict(radius_nm=61.25, cell_nm=1.25,
                     desc="98^3-cell Freudenthal grid cut to a 61.25 nm sphere (the ~500k-node single blob)"),
    "replicas256": dict(radius_nm=20.0, cell_nm=1.25, replicas=256,
                        desc="256 replicas of the 20 nm sphere in one batch, one RNG stream each"),
    "heldout": dict(radius_nm=None, cell_nm=1.25, radii=(10.0, 20.0, 30.0, 40.0, 50.0),
                    desc="the learned preconditioner's held-out family in one batch: spheres of radius "
                         "10, 20, 30, 40 and 50 nm (the network was trained on radii 5-25 nm)"),
    "ensemble64": dict(radius_nm=None, cell_nm=1.25, blobs=64,
                       desc="64 independent blobs in one batch: radii log-uniform 5-40 nm at a 1.25 nm cell, "
                            "moduli x U[0.5, 2], one RNG stream each"),
}


def replica_seed(rank: int) -> int:
    """RNG seed of a single-blob workload's replica on one rank."""
    return 44 + rank


def ensemble_members(count: int = 64, seed: int = 2):
    """(radius_nm, modulus scale) of each ensemble blob, in blob order."""
    rng = np.random.default_rng(seed)
    radii = np.exp(rng.uniform(np.log(5.0), np.log(40.0), size=count))
    scale = rng.uniform(0.5, 2.0, size=count)
    return [(float(r), float(g)) for r, g in zip(radii, scale)]


def params(rng_seed: int, precision: str = "mixed", epsilon: float = 1e-6):
    from . import params as P
    prec = P.PRECISION_MIXED if precision == "mixed" else P.PRECISION_FP64
    return P.SimulationParams.from_si(dt=1e-14, kT=P.kT_at(300.0) * P.MESO_ENERGY, epsilon=epsilon,
                                      max_iterations_cg=10000, rng_seed=rng_seed, solver=P.SOLVER_NOMASS,
                                      precision=prec)


def ensemble_blob(i: int, rank: int = 0, precision: str = "mixed", epsilon: float = 1e-6):
    """Blob i of ensemble64.  Its mesh seed, moduli and RNG seed depend only on
    i (and on the replica rank), so any partition of the ensemble steps the
    same blobs with the same streams."""
    from .mesh import make_blob, sphere_mesh
    r, g = ensemble_members()[i]
    return make_blob(sphere_mesh(r, cell_nm=WORKLOADS["ensemble64"]["cell_nm"], seed=i),
                     params(1000 * (rank + 1) + i, precision, epsilon), shear_mod=3.7e8 * g, bulk_mod=1.1e9 * g)


def build_specs(workload: str, rank: int = 0, precision: str = "mixed", epsilon: float = 1e-6, blobs=None):
    """The blobs of one replica of the workload (rank selects the replica's
    RNG seeds).  `blobs` optionally selects a subset of a multi-blob workload
    by index (the blobs keep their own meshes and seeds)."""
    from .mesh import make_blob, sphere_mesh
    w = WORKLOADS[workload]
    if w.get("replicas"):
        mesh = sphere_mesh(w["radius_nm"], cell_nm=w["cell_nm"], seed=0)
        idx = range(w["replicas"]) if blobs is None else blobs
        return [make_blob(mesh, params(100000 * (rank + 1) + i, precision, epsilon)) for i in idx]
    if w.get("radii"):
        idx = range(len(w["radii"])) if blobs is None else blobs
        return [make_blob(sphere_mesh(w["radii"][i], cell_nm=w["cell_nm"], seed=10 + i),
                          params(2000 * (rank + 1) + i, precision, epsilon)) for i in idx]
    if w.get("blobs"):
        idx = range(w["blobs"]) if blobs is None else blobs
        return [ensemble_blob(i, rank, precision, epsilon) for i in idx]
    return [make_blob(sphere_mesh(w["radius_nm"], cell_nm=w["cell_nm"], seed=0),
                      params(replica_seed(rank), precision, epsilon))]


def blob_count(workload: str) -> int:
    w = WORKLOADS[workload]
    return int(w.get("replicas") or (len(w["radii"]) if w.get("radii") else 0) or w.get("blobs") or 1)


def blob_radii(workload: str):
    """Radius (nm) of every blob of one replica of the workload, in blob order."""
    w = WORKLOADS[workload]
    if w.get("replicas"):
        return [w["radius_nm"]] * w["replicas"]
    if w.get("radii"):
        return list(w["radii"])
    if w.get("blobs"):
        return [r for r, _ in ensemble_members(w["blobs"])]
    return [w["radius_nm"]]


def build_items(workload: str, items, precision: str = "mixed", epsilon: float = 1e-6):
    """The blobs (replica, index) of `items`: blob `index` of the workload's
    replica `replica`, with that replica's RNG seed, so that the blobs a rank
    steps do not depend on which rank steps them.  Meshes shared by several
    items are built once."""
    from .mesh import make_blob, sphere_mesh
    w = WORKLOADS[workload]
    cache = {}

    def mesh(radius, seed):
        key = (radius, seed)
        if key not in cache:
            cache[key] = sphere_mesh(radius, cell_nm=w["cell_nm"], seed=seed)
        return cache[key]

    out = []
    for rep, i in items:
        if w.get("replicas"):
            out.append(make_blob(mesh(w["radius_nm"], 0), params(100000 * (rep + 1) + i, precision, epsilon)))
        elif w.get("radii"):
            out.append(make_blob(mesh(w["radii"][i], 10 + i), params(2000 * (rep + 1) + i, precision, epsilon)))
        elif w.get("blobs"):
            r, g = ensemble_members(w["blobs"])[i]
            out.append(make_blob(mesh(r, i), params(1000 * (rep + 1) + i, precision, epsilon),
                                 shear_mod=3.7e8 * g, bulk_mod=1.1e9 * g))
        else:
            out.append(make_blob(mesh(w["radius_nm"], 0), params(replica_seed(rep), precision, epsilon)))
    return out
