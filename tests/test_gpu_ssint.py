"""Surface-surface LJ interaction on the GPU (ffea_gpu_ssint_*, through the C
ABI) against the oracle (oracle/ssint_oracle.c, a restatement of FFEA's
VdW_solver for "lennard-jones").

Tolerances: the kernels are compiled without FMA contraction, so cell binning
and the normal test decide as the oracle does, and the pair counts must be
equal exactly; a pair's force differs from FFEA's only in rounding (a
reciprocal for a divide, regrouped sums).  Per-face sums run in another order than FFEA's
(each pair from both sides), and the energy is summed with atomics (its last bits
may vary from run to run; the forces do not), so forces
agree to 1e-12 of the largest force and energies to 1e-12 relative."""
import os
import time

import numpy as np
import pytest

from ffea_gb300.params import MESO_ENERGY, nm
from oracle import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "cubes_lj.npz")
FORCE_TOL = 1e-12
ENERGY_TOL = 1e-12


def _solver(**kw):
    from ffea_gb300.surface import LJSurfaceSolver
    return LJSurfaceSolver(**kw)


def _compare(kw, pos):
    s = _solver(**kw)
    f_gpu, e_gpu, p_gpu = s.forces(pos)
    f_ref, e_ref, p_ref = oracle.ssint_lj(pos, kw["faces"], kw["face_blob"], kw["face_type"], kw["emin"], kw["rmin"],
                                          kw["num_blobs"], kw["cell_size"], kw["grid"], kw.get("inc_self", 0))
    assert p_gpu == p_ref
    scale = max(np.abs(f_ref).max(), 1e-300)
    np.testing.assert_allclose(f_gpu, f_ref, rtol=0, atol=FORCE_TOL * scale)
    np.testing.assert_allclose(e_gpu, e_ref, rtol=ENERGY_TOL, atol=ENERGY_TOL * np.abs(e_ref).max())
    s.close()
    return f_gpu, e_gpu, p_gpu


def _cubes_kw(g, **over):
    kw = dict(num_nodes=len(g["pos"]), faces=g["faces"], face_blob=g["face_blob"], face_type=g["face_type"],
              emin=g["emin"], rmin=g["rmin"], num_blobs=2, cell_size=float(g["h"]), grid=tuple(g["grid"]))
    kw.update(over)
    return kw


def test_cubes_lj_known_answer_and_golden():
    g = dict(np.load(GOLDEN))
    f, e, p = _compare(_cubes_kw(g), g["pos"])
    assert p == int(g["pairs"])
    np.testing.assert_allclose(f, g["force"], rtol=0, atol=FORCE_TOL * np.abs(g["force"]).max())
    e_j = e.sum() * MESO_ENERGY
    assert abs(e_j - g["known_energy_j"]) <= g["known_tol"] * abs(g["known_energy_j"])


def test_cubes_lj_every_face_active_and_self_interaction():
    g = dict(np.load(GOLDEN))
    rng = np.random.default_rng(3)
    ftype = rng.integers(0, 3, len(g["face_type"])).astype(np.int32)
    ftype[rng.random(len(ftype)) < 0.1] = -1  # some faces inactive
    pos = g["pos"] + rng.normal(0, 0.02 * nm(1.0), g["pos"].shape)
    _compare(_cubes_kw(g, face_type=ftype, inc_self=1), pos)


def test_small_grid_wrapped_neighbour_cells():
    g = dict(np.load(GOLDEN))
    h = float(g["h"]) * 5
    pos = g["pos"] - g["pos"].mean(0) + h
    _, _, p = _compare(_cubes_kw(g, cell_size=h, grid=(2, 2, 2)), pos)
    assert p > 200 * 200


def _two_spheres(radius_nm, gap_nm, seed):
    from ffea_gb300.mesh import sphere_mesh
    from ffea_gb300.surface import surface_faces
    m = sphere_mesh(radius_nm, seed=seed)
    tri = surface_faces(m.pos, m.topology)
    x = m.pos - m.pos.mean(0)
    shift = np.array([2 * nm(radius_nm) + nm(gap_nm), 0.0, 0.0])
    pos = np.concatenate([x, x + shift])
    n = len(x)
    faces = np.concatenate([tri, tri + n]).astype(np.int32)
    blob = np.repeat(np.arange(2, dtype=np.int32), len(tri))
    h = nm(3.0)
    span = pos.max(0) - pos.min(0)
    grid = tuple(int(v) for v in 2 * np.ceil(span / h))  # World::init's box (src/World.cpp:455-466)
    pos = pos - pos.mean(0) + 0.5 * h * np.array(grid)
    return pos, faces, blob, grid, h


def test_two_spheres_in_contact_with_self_interaction():
    pos, faces, blob, grid, h = _two_spheres(4.0, 0.6, seed=5)
    rng = np.random.default_rng(7)
    T = 2
    emin = rng.uniform(0.5, 2.0, (T, T))
    emin = 0.5 * (emin + emin.T)
    rmin = np.full((T, T), nm(1.0))
    ftype = rng.integers(0, T, len(faces)).astype(np.int32)
    kw = dict(num_nodes=len(pos), faces=faces, face_blob=blob, face_type=ftype, emin=emin, rmin=rmin,
              num_blobs=2, cell_size=h, grid=grid, inc_self=1)
    f, e, p = _compare(kw, pos)
    assert p > 0 and e[0, 1] != 0


def test_centroid_outside_the_grid_is_an_error_and_the_handle_recovers():
    from ffea_gb300._lib import FfeaGpuError
    g = dict(np.load(GOLDEN))
    s = _solver(**_cubes_kw(g))
    bad = g["pos"].copy()
    bad[:, 0] += 3 * float(g["h"]) * g["grid"][0]
    with pytest.raises(FfeaGpuError, match="outside the interaction grid"):
        s.forces(bad)
    f, e, p = s.forces(g["pos"])
    assert p == int(g["pairs"])
    s.close()


def test_no_active_faces_gives_zero():
    g = dict(np.load(GOLDEN))
    s = _solver(**_cubes_kw(g, face_type=np.full(len(g["face_type"]), -1, np.int32)))
    f, e, p = s.forces(g["pos"])
    assert p == 0 and not f.any() and not e.any()
    s.close()


def test_throughput_two_20nm_spheres(capsys):
    """Device-resident timing of one solve (face geometry, grid, pairs, node
    gather) for two 20 nm spheres 0.6 nm apart; printed, not asserted."""
    import torch
    pos, faces, blob, grid, h = _two_spheres(20.0, 0.6, seed=11)
    kw = dict(num_nodes=len(pos), faces=faces, face_blob=blob, face_type=np.zeros(len(faces), np.int32),
              emin=np.ones((1, 1)), rmin=np.full((1, 1), nm(1.0)), num_blobs=2, cell_size=h, grid=grid, inc_self=1)
    s = _solver(**kw)
    d_pos = torch.tensor(pos, device="cuda")
    d_f = torch.zeros_like(d_pos)
    d_e = torch.zeros(4, dtype=torch.float64, device="cuda")
    st = torch.cuda.ExternalStream(s.stream)
    for _ in range(3):
        s.forces_device(d_pos.data_ptr(), d_f.data_ptr(), d_e.data_ptr())
    pairs = s.synchronize()
    reps = 20
    with torch.cuda.stream(st):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(reps):
            s.forces_device(d_pos.data_ptr(), d_f.data_ptr(), d_e.data_ptr())
        b.record(st)
    s.synchronize()
    ms = a.elapsed_time(b) / reps
    t0 = time.perf_counter()
    oracle.ssint_lj(pos, faces, blob, kw["face_type"], kw["emin"], kw["rmin"], 2, h, grid, 1)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    with capsys.disabled():
        print(f"\nssint two 20 nm spheres: {len(faces)} faces, {pairs} pairs, GPU {ms * 1e3:.1f} us/solve "
              f"({pairs / ms * 1e-6:.3f} G pairs/s; each pair evaluated from both sides), "
              f"oracle 1 core {cpu_ms:.1f} ms")
    f_ref, _, _ = oracle.ssint_lj(pos, faces, blob, kw["face_type"], kw["emin"], kw["rmin"], 2, h, grid, 1)
    np.testing.assert_allclose(d_f.cpu().numpy(), f_ref, rtol=0, atol=FORCE_TOL * np.abs(f_ref).max())
    s.close()


def test_large_cells_sorted_by_a_cta_each():
    """A coarse grid (8 nm cells over two 4 nm spheres) puts more than 64
    faces in a cell, so the cells are sorted by the one-CTA-per-cell path:
    the results match the oracle and repeat bit for bit."""
    pos, faces, blob, _, _ = _two_spheres(4.0, 0.6, seed=5)
    h = nm(8.0)
    span = pos.max(0) - pos.min(0)
    grid = tuple(int(v) for v in 2 * np.ceil(span / h))
    pos = pos - pos.mean(0) + 0.5 * h * np.array(grid)
    cells = np.floor((pos[faces].mean(1)) / h).astype(int)
    _, per_cell = np.unique(cells[:, 0] * 10000 + cells[:, 1] * 100 + cells[:, 2], return_counts=True)
    assert per_cell.max() > 64, per_cell.max()
    kw = dict(num_nodes=len(pos), faces=faces, face_blob=blob, face_type=np.zeros(len(faces), np.int32),
              emin=np.ones((1, 1)), rmin=np.full((1, 1), nm(1.0)), num_blobs=2, cell_size=h, grid=grid, inc_self=1)
    f1, _, p1 = _compare(kw, pos)
    s = _solver(**kw)
    f2, _, p2 = s.forces(pos)
    s.close()
    assert p1 == p2 and np.array_equal(f1, f2)


def test_overfull_cell_is_an_error():
    """More than 4096 faces in one cell (one 20 nm sphere in a single-cell
    grid) fails the call at once with a message, instead of a long serial sort."""
    from ffea_gb300._lib import FfeaGpuError
    from ffea_gb300.mesh import sphere_mesh
    from ffea_gb300.surface import surface_faces
    m = sphere_mesh(20.0, seed=2)
    tri = surface_faces(m.pos, m.topology).astype(np.int32)
    assert len(tri) > 4096
    h = 1.1 * float((m.pos.max(0) - m.pos.min(0)).max())
    pos = m.pos - m.pos.mean(0) + 0.5 * h
    kw = dict(num_nodes=len(pos), faces=tri, face_blob=np.zeros(len(tri), np.int32),
              face_type=np.zeros(len(tri), np.int32), emin=np.ones((1, 1)), rmin=np.full((1, 1), nm(1.0)),
              num_blobs=1, cell_size=h, grid=(1, 1, 1), inc_self=1)
    s = _solver(**kw)
    t = time.perf_counter()
    for _ in range(2):
        with pytest.raises(FfeaGpuError, match="too coarse"):
            s.forces(pos)
    assert time.perf_counter() - t < 10.0
    s.close()


@pytest.mark.parametrize("ssint_type", [1, 2, 3])
@pytest.mark.parametrize("inc_self", [0, 1])
def test_steric_types_match_oracle(ssint_type, inc_self):
    """steric, ljsteric and gensoft on two spheres pushed 0.6 nm into each
    other (element tetrahedra overlap across the contact): the GPU against
    the oracle (oracle/steric_oracle.c, pinned to FFEA's own geometry code
    in tests/test_steric_oracle.py).  The overlap of each pair is the same
    clipping arithmetic on both sides; forces agree to 1e-9 of the largest,
    energies to 1e-9, the interacting pair counts exactly."""
    from tests.test_steric_oracle import overlapping_spheres
    pos, faces, apex, blob, h, grid = overlapping_spheres()
    rng = np.random.default_rng(11)
    T = 2
    emin = rng.uniform(0.5, 2.0, (T, T))
    emin = 0.5 * (emin + emin.T)
    rmin = np.full((T, T), nm(1.0))
    k0 = np.full((T, T), 0.3)
    ftype = rng.integers(0, T, len(faces)).astype(np.int32)
    kw = dict(num_nodes=len(pos), faces=faces, face_blob=blob, face_type=ftype, emin=emin, rmin=rmin, num_blobs=2,
              cell_size=h, grid=grid, inc_self=inc_self, ssint_type=ssint_type, face_apex=apex, steric_factor=50.0,
              steric_dr=5e-3, k0=k0)
    s = _solver(**kw)
    f_gpu, e_gpu, p_gpu = s.forces(pos)
    s.close()
    f_ref, e_ref, p_ref = oracle.ssint(pos, faces, blob, ftype, emin, rmin, 2, h, grid, inc_self, ssint_type, apex,
                                       50.0, 5e-3, k0)
    assert p_gpu == p_ref and p_ref > 0
    scale = np.abs(f_ref).max()
    np.testing.assert_allclose(f_gpu, f_ref, rtol=0, atol=1e-9 * scale)
    np.testing.assert_allclose(e_gpu, e_ref, rtol=1e-9, atol=1e-9 * np.abs(e_ref).max())
    # the steric share: the same pass with the steric part alone
    if ssint_type != 1:
        _, e_st, p_st = oracle.ssint(pos, faces, blob, ftype, emin, rmin, 2, h, grid, inc_self, 1, apex, 50.0, 5e-3)
        assert 0 < p_st < p_ref


@pytest.mark.parametrize("ssint_type", [0, 1, 2, 3])
def test_periodic_corrections_match_oracle(ssint_type):
    """force_pbc: the second sphere translated by one box length in x and
    minus one in z, the blob corrections from the blobs' centroids
    (SurfaceSolver.blob_corr, the library's World::calc_blob_corr_matrix).
    The GPU against the oracle with the same corrections (forces to 1e-9 of
    the largest, energies to 1e-9, pair counts exactly), and against the
    untranslated pass without corrections (the same geometry: 1e-9)."""
    from tests.test_steric_oracle import overlapping_spheres
    pos, faces, apex, blob, h, grid = overlapping_spheres()
    rng = np.random.default_rng(13)
    T = 2
    emin = rng.uniform(0.5, 2.0, (T, T))
    emin = 0.5 * (emin + emin.T)
    rmin = np.full((T, T), nm(1.0))
    k0 = np.full((T, T), 0.3)
    ftype = rng.integers(0, T, len(faces)).astype(np.int32)
    kw = dict(num_nodes=len(pos), faces=faces, face_blob=blob, face_type=ftype, emin=emin, rmin=rmin, num_blobs=2,
              cell_size=h, grid=grid, inc_self=1, ssint_type=ssint_type, face_apex=apex, steric_factor=50.0,
              steric_dr=5e-3, k0=k0)
    s = _solver(**kw)
    f0, e0, p0 = s.forces(pos)
    n = len(pos) // 2
    moved = pos.copy()
    moved[n:] += np.array([1.0, 0.0, -1.0]) * s.box
    bc = s.blob_corr(np.array([moved[:n].mean(0), moved[n:].mean(0)]))
    assert np.array_equal(bc[0, 1], np.array([1.0, 0.0, -1.0]) * s.box)
    s.set_pbc(bc)
    f1, e1, p1 = s.forces(moved)
    s.set_pbc(None)
    f2, e2, p2 = s.forces(pos)
    s.close()
    f_ref, e_ref, p_ref = oracle.ssint(moved, faces, blob, ftype, emin, rmin, 2, h, grid, 1, ssint_type, apex, 50.0,
                                       5e-3, k0, blob_corr=bc)
    scale = np.abs(f_ref).max()
    assert p1 == p_ref == p0 == p2 and p0 > 0
    np.testing.assert_allclose(f1, f_ref, rtol=0, atol=1e-9 * scale)
    np.testing.assert_allclose(e1, e_ref, rtol=1e-9, atol=1e-9 * np.abs(e_ref).max())
    np.testing.assert_allclose(f1, f0, rtol=0, atol=1e-9 * scale)
    assert np.array_equal(f2, f0)  # turned off again


@pytest.mark.parametrize("ssint_type", [0, 2])
def test_sticky_wall_matches_oracle(ssint_type):
    """sticky_wall_xz: a sphere resting 0.4 nm above y = 0 in a 6^3 grid, plus
    the pair pass; the GPU against the oracle (forces to 1e-10 of the
    largest); the walls need two rows of cells."""
    from ffea_gb300._lib import FfeaGpuError
    from ffea_gb300.mesh import sphere_mesh
    from ffea_gb300.surface import surface_faces
    m = sphere_mesh(2.5, seed=8)
    tri, apex = surface_faces(m.pos, m.topology, with_apex=True)
    tri = tri.astype(np.int32)
    h = nm(1.5)
    grid = (6, 6, 6)
    pos = m.pos - m.pos.mean(0) + np.array([3.0, 0.0, 3.0]) * h
    pos[:, 1] += -pos[:, 1].min() + nm(0.4)
    rng = np.random.default_rng(2)
    ftype = rng.integers(0, 2, len(tri)).astype(np.int32)
    emin = np.array([[1.0, 0.7], [0.7, 1.3]])
    rmin = np.full((2, 2), nm(0.6))
    blob = np.zeros(len(tri), np.int32)
    kw = dict(num_nodes=len(pos), faces=tri, face_blob=blob, face_type=ftype, emin=emin, rmin=rmin, num_blobs=1,
              cell_size=h, grid=grid, inc_self=1, ssint_type=ssint_type, face_apex=apex, steric_factor=50.0,
              steric_dr=5e-3, sticky_wall=True)
    s = _solver(**kw)
    f_gpu, e_gpu, p_gpu = s.forces(pos)
    s.close()
    f_ref, e_ref, p_ref = oracle.ssint(pos, tri, blob, ftype, emin, rmin, 1, h, grid, 1, ssint_type, apex, 50.0, 5e-3,
                                       sticky_wall=True)
    f_nowall, _, _ = oracle.ssint(pos, tri, blob, ftype, emin, rmin, 1, h, grid, 1, ssint_type, apex, 50.0, 5e-3)
    assert p_gpu == p_ref and np.abs(f_ref - f_nowall).max() > 0
    np.testing.assert_allclose(f_gpu, f_ref, rtol=0, atol=1e-10 * np.abs(f_ref).max())
    kw["grid"] = (6, 1, 6)
    with pytest.raises(FfeaGpuError, match="two rows"):
        _solver(**kw)
