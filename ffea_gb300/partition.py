"""Ensembles of independent blobs sharded over processes, one GPU each.

FFEA steps the blobs of a system one after another inside each time step
(World::run, src/World.cpp:2020-2043; with FFEA_PARALLEL_PER_BLOB an OpenMP
loop over blobs, `ffea_mb`).  Blobs that do not interact are independent:
each has its own RNG stream, so the blobs can be divided among processes
without any exchange while they step.

  blob_cost()  HBM bytes one step of a blob moves in the minimum-traffic
               model: element forces 12 N + 168 E, draws 4 (7 E + 3 N_t),
               assembly 104 E + 36 B, gather 64 E + 16 N, update 48 N, and
               `iterations` CG iterations of 40 B + 148 N each
               (B = N + 2 edges 3x3 blocks)
  pack()       greedy size-balanced bin packing: blobs in decreasing cost,
               each to the rank with the least cost so far (lowest rank on
               ties); deterministic
  estimate_sizes()  corner nodes, elements and edges of a synthetic sphere
               of radius R at cell h, without building the mesh
  ensemble_plan()   the blobs (replica, index) of an ensemble workload that
               each of `world` ranks steps

Nothing is exchanged during stepping; results are gathered on the host at
the end (energies, statistics), as files or a host-side gather.
"""
from __future__ import annotations

import math


def blob_cost(num_linear: int, num_elements: int, num_edges: int, num_total: int | None = None,
              iterations: float = 90.0) -> float:
    """Estimated HBM bytes of one NoMass step of one blob (see module doc)."""
    N, E = float(num_linear), float(num_elements)
    B = N + 2.0 * float(num_edges)
    Nt = float(num_total) if num_total is not None else N + float(num_edges)
    step = (12 * N + 168 * E) + 4 * (7 * E + 3 * Nt) + (104 * E + 36 * B) + (64 * E + 16 * N) + 48 * N
    return step + float(iterations) * (40 * B + 148 * N)


def estimate_sizes(radius_nm: float, cell_nm: float = 1.25):
    """(corner nodes, elements, edges) of a Freudenthal-split grid sphere,
    estimated from its volume: 6 tetrahedra per cell inside the sphere,
    lattice vertices within about 0.6 cell of it, and 6.5 edges per vertex
    (7 per interior vertex of the split lattice, fewer on the surface).
    Within about 10 per cent of the built meshes from 5 to 30 nm."""
    a = radius_nm / cell_nm
    cells = (4.0 / 3.0) * math.pi * a ** 3
    nodes = (4.0 / 3.0) * math.pi * (a + 0.6) ** 3
    return int(round(nodes)), int(round(6 * cells)), int(round(6.5 * nodes))


def pack(costs, ranks: int):
    """Indices of `costs` per rank, greedy largest-first onto the least-loaded
    rank.  Returns (bins, loads)."""
    if ranks < 1:
        raise ValueError("ranks must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    bins = [[] for _ in range(ranks)]
    loads = [0.0] * ranks
    for i in order:
        r = min(range(ranks), key=lambda k: (loads[k], k))
        bins[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(b) for b in bins], loads


def ensemble_plan(radii, world: int, replicas: int | None = None, cell_nm: float = 1.25, iterations: float = 90.0):
    """Shard `replicas` copies (default: one per rank) of an ensemble with the
    given blob radii over `world` ranks.  Returns, per rank, a list of
    (replica, index) pairs in ascending order, and the per-rank cost."""
    replicas = world if replicas is None else replicas
    items, costs = [], []
    for rep in range(replicas):
        for i, r in enumerate(radii):
            n, e, ed = estimate_sizes(r, cell_nm)
            items.append((rep, i))
            costs.append(blob_cost(n, e, ed, iterations=iterations))
    bins, loads = pack(costs, world)
    return [[items[k] for k in b] for b in bins], loads
