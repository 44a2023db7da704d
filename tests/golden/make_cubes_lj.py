"""Generate tests/golden/cubes_lj.npz: the reference's LJ known-answer case.

FFEA's tests/physics/cubes_lj runs two 1 nm cubes (tests/physics/
fine_cube_structure/veryFine.*) with only their top faces of interaction type
0 (veryFine_topface0.vdw), the second cube rotated by 180 degrees about z and
centred 2 nm away along y (cube_veryFine.ffea), so that the two top faces are
parallel unit squares 1 nm apart.  checkE.py asserts the surface-surface
energy -1.7870e-19 J within 1 % (the CUBA value -0.704384545 of the double
integral, times Emin = 2.537e17 J/m^4 and Rmin^4 = 1e-36 m^4).

The box is FFEA's: ssint_cutoff 3 nm (its default, src/SimulationParams.cpp:42)
times es_N = 10 cells a side, the system centroid moved to the box centre
(src/World.cpp:455-480).  The script stores the inputs in meso units, the
oracle's forces, energy matrix and pair count, and the known answer.

Run from the repository root (it reads the reference's structure files):
    python tests/golden/make_cubes_lj.py [reference-root]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from ffea_gb300.formats import read_nodes  # noqa: E402
from ffea_gb300.params import MESO_ENERGY, MESO_LENGTH  # noqa: E402
from oracle import oracle  # noqa: E402

KNOWN_ENERGY_J = -1.7870e-19
KNOWN_TOL = 1e-2


def _read_surf(path):
    L = [ln.split() for ln in open(path).read().splitlines()]
    n = int(L[1][1])
    assert L[2] == ["faces:"]
    rows = np.array([[int(v) for v in r] for r in L[3:3 + n]], np.int32)
    return rows[:, 1:4], rows[:, 0]


def _read_vdw(path):
    L = open(path).read().split()
    n = int(L[L.index("num_faces") + 1])
    i = L.index("params:") + 1
    return np.array([int(v) for v in L[i:i + n]], np.int32)


def _read_lj(path):
    txt = open(path).read().splitlines()
    t = int(txt[1].split()[1])
    vals = []
    for ln in txt[2:2 + t]:
        for pair in ln.replace("(", " ").replace(")", " ").split():
            vals.append(float(pair.strip(",")))
    a = np.array(vals).reshape(t, t, 2)
    return a[:, :, 0], a[:, :, 1]


def main(ref_root):
    d = os.path.join(ref_root, "tests", "physics", "fine_cube_structure")
    nodes, _ = read_nodes(os.path.join(d, "veryFine.node"))
    faces, _ = _read_surf(os.path.join(d, "veryFine.surf"))
    ftype = _read_vdw(os.path.join(d, "veryFine_topface0.vdw"))
    emin_si, rmin_si = _read_lj(os.path.join(d, "veryFine.lj"))
    scale = 1e-9 / MESO_LENGTH                     # <scale = 1.00e-9>
    x = nodes * scale
    b1 = x - x.mean(0)                              # centroid (0, 0, 0)
    b2 = (x - x.mean(0)) * np.array([-1.0, -1.0, 1.0]) + np.array([0.0, 2.0, 0.0]) * scale  # 180 deg about z
    pos = np.concatenate([b1, b2])
    h = 3e-9 / MESO_LENGTH
    grid = (10, 10, 10)
    pos = pos - pos.mean(0) + 0.5 * h * np.array(grid)
    nn = len(nodes)
    all_faces = np.concatenate([faces, faces + nn]).astype(np.int32)
    face_blob = np.repeat(np.arange(2, dtype=np.int32), len(faces))
    face_type = np.concatenate([ftype, ftype])
    area = MESO_LENGTH ** 2
    emin = emin_si * area * area / MESO_ENERGY      # SSINT_matrix::init, src/LJ_matrix.cpp:141-142
    rmin = rmin_si / MESO_LENGTH
    force, energy, pairs = oracle.ssint_lj(pos, all_faces, face_blob, face_type, emin, rmin, 2, h, grid)
    e_j = energy.sum() * MESO_ENERGY
    rel = abs(e_j - KNOWN_ENERGY_J) / abs(KNOWN_ENERGY_J)
    print(f"energy {e_j:.6e} J, known {KNOWN_ENERGY_J:.4e} J, relative error {rel:.3e}, {pairs} face pairs")
    assert rel < KNOWN_TOL
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cubes_lj.npz")
    np.savez_compressed(out, pos=pos, faces=all_faces, face_blob=face_blob, face_type=face_type, emin=emin,
                        rmin=rmin, h=h, grid=np.array(grid), force=force, energy=energy, pairs=pairs,
                        known_energy_j=KNOWN_ENERGY_J, known_tol=KNOWN_TOL)
    print("wrote", out)


if __name__ == "__main__":
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
    from oracle import oracle as O
    src = sys.argv[1] if len(sys.argv) > 1 else O.reference_src()
    if not src:
        raise SystemExit("usage: make_cubes_lj.py <FFEA source tree> (or set FFEA_REFERENCE_SRC)")
    main(src)
