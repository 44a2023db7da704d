"""Readers and writers for the FFEA blob input files the update consumes.

Formats follow the reference loaders: ``.node`` (src/Blob.cpp:2415-2513),
``.top`` (:2517-2640), ``.mat`` (:2821-2876), ``.stokes`` (:2880-2947) and
``.pin`` (:3691-3755).  Positions and Stokes radii are multiplied by the
blob's ``scale`` exactly as the loaders do (scale already divided by the meso
length, src/World.cpp:2564-2567).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from .params import material_si_to_meso


class FormatError(ValueError):
    """A blob input file does not have the layout the reference loader expects."""


@dataclasses.dataclass
class BlobFiles:
    """Raw contents of one blob's input files, in file units (SI)."""

    pos: np.ndarray            # (N_t, 3) float64, file units
    num_surface_nodes: int
    topology: np.ndarray       # (E, 10) int32
    num_surface_elements: int
    material_si: np.ndarray    # (E, 6) float64: density, shear_visc, bulk_visc, shear_mod, bulk_mod, dielectric
    stokes_radius: np.ndarray  # (N_t,) float64, file units
    pinned: np.ndarray         # (P,) int32


def _lines(path):
    with open(path, "r") as fh:
        return [ln.rstrip("\n") for ln in fh]


def _header(lines, i, key):
    parts = lines[i].split()
    if len(parts) != 2 or parts[0] != key:
        raise FormatError(f"expected '{key} <n>' at line {i + 1}, found {lines[i]!r}")
    return int(parts[1])


def _magic(lines, kinds):
    if not lines or lines[0].strip() not in kinds:
        raise FormatError(f"not one of {kinds}: {lines[0] if lines else ''!r}")


def read_nodes(path):
    """Blob::load_nodes: header, 'surface nodes:', 'interior nodes:' sections."""
    L = _lines(path)
    _magic(L, ("ffea node file", "walrus node file"))
    n = _header(L, 1, "num_nodes")
    ns = _header(L, 2, "num_surface_nodes")
    ni = _header(L, 3, "num_interior_nodes")
    if L[4].strip() != "surface nodes:":
        raise FormatError("missing 'surface nodes:' line")
    rows, i = [], 5
    for k in range(n):
        if k == ns:
            if L[i].strip() != "interior nodes:":
                raise FormatError("missing 'interior nodes:' line")
            i += 1
        rows.append([float(v) for v in L[i].split()[:3]])
        i += 1
    if ns + ni != n:
        raise FormatError("num_surface_nodes + num_interior_nodes != num_nodes")
    return np.asarray(rows, dtype=np.float64).reshape(n, 3), ns


def read_topology(path, num_nodes=None):
    """Blob::load_topology: 10 node indices per element, bounds-checked."""
    L = _lines(path)
    _magic(L, ("ffea topology file", "walrus topology file"))
    ne = _header(L, 1, "num_elements")
    ns = _header(L, 2, "num_surface_elements")
    _header(L, 3, "num_interior_elements")
    if L[4].strip() != "surface elements:":
        raise FormatError("missing 'surface elements:' line")
    rows, i = [], 5
    for k in range(ne):
        if k == ns:
            if L[i].strip() != "interior elements:":
                raise FormatError("missing 'interior elements:' line")
            i += 1
        vals = [int(v) for v in L[i].split()]
        if len(vals) != 10:
            raise FormatError(f"element {k}: expected 10 node indices")
        rows.append(vals)
        i += 1
    topo = np.asarray(rows, dtype=np.int32).reshape(ne, 10)
    if num_nodes is not None and topo.size and (topo.min() < 0 or topo.max() >= num_nodes):
        raise FormatError("an element references an out of bounds node index")
    return topo, ns


def read_material(path):
    L = _lines(path)
    _magic(L, ("ffea material params file", "walrus material params file"))
    ne = _header(L, 1, "num_elements")
    rows = [[float(v) for v in L[2 + k].split()[:6]] for k in range(ne)]
    return np.asarray(rows, dtype=np.float64).reshape(ne, 6)


def read_stokes(path):
    L = _lines(path)
    _magic(L, ("ffea stokes radii file", "walrus stokes radii file"))
    n = _header(L, 1, "num_nodes")
    return np.asarray([float(L[2 + k].split()[0]) for k in range(n)], dtype=np.float64)


def read_pin(path):
    L = _lines(path)
    _magic(L, ("ffea pinned nodes file", "walrus pinned nodes file"))
    n = _header(L, 1, "num_pinned_nodes")
    if L[2].strip() != "pinned nodes:":
        raise FormatError("missing 'pinned nodes:' line")
    return np.asarray([int(L[3 + k].split()[0]) for k in range(n)], dtype=np.int32)


def read_blob(node, top, mat, stokes=None, pin=None) -> BlobFiles:
    pos, ns = read_nodes(node)
    topo, nse = read_topology(top, len(pos))
    material = read_material(mat)
    if len(material) != len(topo):
        raise FormatError("material file element count does not match topology")
    radius = read_stokes(stokes) if stokes else np.zeros(len(pos))
    if len(radius) != len(pos):
        raise FormatError("stokes file node count does not match node file")
    pinned = read_pin(pin) if pin else np.zeros(0, dtype=np.int32)
    return BlobFiles(pos, ns, topo, nse, material, radius, pinned)


def write_blob(prefix, files: BlobFiles):
    """Write .node/.top/.mat/.stokes/.pin in the reference layout."""
    n, e = len(files.pos), len(files.topology)
    with open(prefix + ".node", "w") as fh:
        fh.write("ffea node file\n")
        fh.write(f"num_nodes {n}\nnum_surface_nodes {files.num_surface_nodes}\n")
        fh.write(f"num_interior_nodes {n - files.num_surface_nodes}\nsurface nodes:\n")
        for k, p in enumerate(files.pos):
            if k == files.num_surface_nodes:
                fh.write("interior nodes:\n")
            fh.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
    with open(prefix + ".top", "w") as fh:
        fh.write("ffea topology file\n")
        fh.write(f"num_elements {e}\nnum_surface_elements {files.num_surface_elements}\n")
        fh.write(f"num_interior_elements {e - files.num_surface_elements}\nsurface elements:\n")
        for k, t in enumerate(files.topology):
            if k == files.num_surface_elements:
                fh.write("interior elements:\n")
            fh.write(" ".join(str(int(v)) for v in t) + " \n")
    with open(prefix + ".mat", "w") as fh:
        fh.write(f"ffea material params file\nnum_elements {e}\n")
        for m in files.material_si:
            fh.write(" ".join(repr(float(v)) for v in m) + "\n")
    with open(prefix + ".stokes", "w") as fh:
        fh.write(f"ffea stokes radii file\nnum_nodes {n}\n")
        for r in files.stokes_radius:
            fh.write(f"{float(r)!r}\n")
    with open(prefix + ".pin", "w") as fh:
        fh.write(f"ffea pinned nodes file\nnum_pinned_nodes {len(files.pinned)}\npinned nodes:\n")
        for p in files.pinned:
            fh.write(f"{int(p)}\n")


def blob_arrays_from_files(files: BlobFiles, scale_si: float, stokes_visc_meso: float, calc_stokes: int = 1):
    """Arrays in meso units as Blob::init leaves them: positions and radii
    times scale (src/Blob.cpp:2495-2497, :2925), material converted, drag
    = 6 pi eta r (src/Blob.cpp:408-412)."""
    from .params import MESO_LENGTH, stokes_drag
    scale = scale_si / MESO_LENGTH
    pos = scale * files.pos
    radius = files.stokes_radius * scale
    mat = material_si_to_meso(*files.material_si[:, :5].T)
    drag = stokes_drag(radius, stokes_visc_meso, calc_stokes)
    return pos, files.topology.astype(np.int32), mat, drag, files.pinned.astype(np.int32)


def exists(prefix):
    return all(os.path.exists(prefix + ext) for ext in (".node", ".top", ".mat"))
