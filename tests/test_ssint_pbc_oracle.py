"""Periodic blob corrections and the sticky wall in the surface oracle
(oracle/ssint_oracle.c), on the CPU.

  - blob_corr follows World::calc_blob_corr_matrix (src/World.cpp:4460-4483):
    box * floor((c_j - c_i + box / 2) / box), antisymmetric;
  - translating one blob of an interacting pair by whole box lengths, with
    the corrections computed from the blobs' centroids, leaves every force,
    energy and pair count of the pass as it was without periodicity (the
    faces sit in the same cells after the grid's one wrap, and FFEA's shifts
    -- f1's points by -blob_corr[b2][b1], f2's tetrahedron by
    -blob_corr[b1][b2], the in-front separation c2 - c1 - blob_corr[b1][b2]
    -- undo the translation): all four interaction types, shifts along each
    axis and both signs;
  - the sticky wall against a plain restatement of do_sticky_xz_interaction
    (src/VdW_solver.cpp:396-456) on the faces of the bottom and top rows.
"""
import numpy as np
import pytest

from oracle import oracle as O


def test_blob_corr_matrix():
    box = np.array([10.0, 20.0, 30.0])
    c = np.array([[1.0, 1.0, 1.0], [9.5, 2.0, -14.0], [4.0, 21.0, 16.5]])
    bc = O.blob_corr(c, box)
    assert np.array_equal(bc, -bc.transpose(1, 0, 2))
    assert not bc[np.arange(3), np.arange(3)].any()
    for i in range(3):
        for j in range(i + 1, 3):
            want = box * np.floor((c[j] - c[i] + 0.5 * box) / box)
            assert np.array_equal(bc[i, j], want)
    assert np.array_equal(bc[0, 1], [10.0, 0.0, 0.0]) and np.array_equal(bc[0, 2], [0.0, 20.0, 30.0])


def _pair_setup(ssint_type):
    from ffea_gb300.params import nm
    from tests.test_steric_oracle import overlapping_spheres
    pos, faces, apex, blob, h, grid = overlapping_spheres()
    rng = np.random.default_rng(4)
    T = 2
    emin = rng.uniform(0.5, 2.0, (T, T))
    emin = 0.5 * (emin + emin.T)
    rmin = np.full((T, T), nm(1.0))
    k0 = np.full((T, T), 0.3)
    ftype = rng.integers(0, T, len(faces)).astype(np.int32)
    return pos, faces, apex, blob, h, grid, ftype, emin, rmin, k0


@pytest.mark.parametrize("ssint_type", [0, 1, 2, 3])
@pytest.mark.parametrize("shift", [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, 0, -1), (1, -1, 1)])
def test_translated_blob_with_corrections_is_unchanged(ssint_type, shift):
    pos, faces, apex, blob, h, grid, ftype, emin, rmin, k0 = _pair_setup(ssint_type)
    box = h * np.asarray(grid, np.float64)
    args = (faces, blob, ftype, emin, rmin, 2, h, grid, 1, ssint_type, apex, 50.0, 5e-3, k0)
    f0, e0, p0 = O.ssint(pos, *args)
    assert p0 > 0
    n = len(pos) // 2
    moved = pos.copy()
    moved[n:] += np.asarray(shift, np.float64) * box
    cen = np.array([moved[:n].mean(0), moved[n:].mean(0)])
    bc = O.blob_corr(cen, box)
    assert np.array_equal(bc[0, 1], np.asarray(shift, np.float64) * box)
    f1, e1, p1 = O.ssint(moved, *args, blob_corr=bc)
    assert p1 == p0
    scale = np.abs(f0).max()
    np.testing.assert_allclose(f1, f0, rtol=0, atol=1e-9 * scale)
    np.testing.assert_allclose(e1, e0, rtol=1e-9, atol=1e-9 * np.abs(e0).max())
    # without the corrections the translated blob interacts differently
    f2, e2, p2 = O.ssint(moved, *args)
    assert p2 != p0 or not np.allclose(f2, f0, rtol=0, atol=1e-6 * scale)


def _sticky_ref(pos, faces, ftype, emin, rmin, h, grid):
    """do_sticky_xz_interaction restated in numpy for the faces whose cell is in
    the bottom (y = 0) or top (y = Ny - 1) row: y force on their corners."""
    W = 0.333333333333333
    eta = np.array([[0.666666666666667, 0.166666666666667, 0.166666666666667],
                    [0.166666666666667, 0.666666666666667, 0.166666666666667],
                    [0.166666666666667, 0.166666666666667, 0.666666666666667]])
    ny = grid[1]
    out = np.zeros_like(pos)
    for f, tri in enumerate(faces):
        v = pos[tri]
        c = v.mean(0)
        cy = int(np.floor(c[1] / h)) % ny
        if cy not in (0, ny - 1):
            continue
        bottom = cy == 0
        nrm = np.cross(v[1] - v[0], v[2] - v[0])
        area = 0.5 * np.linalg.norm(nrm)
        nrm = nrm / np.linalg.norm(nrm)
        if (bottom and nrm[1] > 0) or (not bottom and nrm[1] < 0):
            continue
        y_wall = 0.0 if bottom else h * ny
        py = eta @ v[:, 1]
        t = ftype[f]
        r6 = rmin[t, t] ** 6
        fpm = np.zeros((3, 3))
        for k in range(3):
            for l in range(k, 3):
                r = py[k] - y_wall
                fpm[k, l] = fpm[l, k] = -12 * r6 * emin[t, t] * (r ** -7 - r6 * r ** -13)
        for j in range(3):
            out[tri[j], 1] += W * W * (eta[:, j][None, :] * fpm).sum() * area * area
    return out


def test_sticky_wall_matches_its_restatement():
    from ffea_gb300.mesh import sphere_mesh
    from ffea_gb300.params import nm
    from ffea_gb300.surface import surface_faces
    m = sphere_mesh(2.5, seed=8)
    tri = surface_faces(m.pos, m.topology).astype(np.int32)
    h = nm(1.5)
    grid = (6, 6, 6)
    pos = m.pos - m.pos.mean(0) + np.array([3.0, 0.0, 3.0]) * h
    pos[:, 1] += -pos[:, 1].min() + nm(0.4)  # the sphere sits just above y = 0
    rng = np.random.default_rng(2)
    ftype = rng.integers(0, 2, len(tri)).astype(np.int32)
    emin = np.array([[1.0, 0.7], [0.7, 1.3]])
    rmin = np.full((2, 2), nm(0.6))
    blob = np.zeros(len(tri), np.int32)
    f0, _, _ = O.ssint(pos, tri, blob, ftype, emin, rmin, 1, h, grid)
    f1, _, _ = O.ssint(pos, tri, blob, ftype, emin, rmin, 1, h, grid, sticky_wall=True)
    wall = f1 - f0
    ref = _sticky_ref(pos, tri, ftype, emin, rmin, h, grid)
    assert np.abs(ref).max() > 0 and not wall[:, [0, 2]].any()
    np.testing.assert_allclose(wall, ref, rtol=0, atol=1e-10 * np.abs(ref).max())
    with pytest.raises(ValueError, match="two rows"):
        O.ssint(pos, tri, blob, ftype, emin, rmin, 1, h, (6, 1, 6), sticky_wall=True)


def test_library_blob_corr_matches_oracle(gpulib_cpu):
    """ffea_gpu_ssint_blob_corr (host code of the library) equals the oracle's
    World::calc_blob_corr_matrix, bit for bit."""
    import ctypes
    rng = np.random.default_rng(5)
    c = rng.uniform(-40.0, 80.0, (7, 3))
    box = np.array([25.0, 31.0, 40.0])
    out = np.zeros((7, 7, 3))
    dp = ctypes.POINTER(ctypes.c_double)
    rc = gpulib_cpu.ffea_gpu_ssint_blob_corr(7, c.ctypes.data_as(dp), box.ctypes.data_as(dp), out.ctypes.data_as(dp))
    assert rc == 0
    assert np.array_equal(out, O.blob_corr(c, box))
