"""The synthetic meshes that stand in for FFEA's protein meshes
(ffea_gb300.mesh), on the CPU: FFEA's 10-node tetrahedron layout (corners
0-3, the midpoints of edges 01, 02, 03, 12, 13, 23 in 4-9), positive rest
volumes after the jitter, midpoint nodes shared by every element on the
edge and placed at the edge's middle, and no unused node."""
import numpy as np
import pytest

from ffea_gb300.mesh import cube_mesh, sphere_mesh

EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


@pytest.mark.parametrize("make", [lambda: sphere_mesh(5.0, seed=3), lambda: sphere_mesh(10.0, seed=0),
                                  lambda: cube_mesh(4, seed=1)])
def test_mesh_layout(make):
    m = make()
    N, t, p = m.num_linear, m.topology.astype(np.int64), m.pos
    corners, mids = t[:, :4], t[:, 4:]
    assert corners.min() >= 0 and corners.max() < N
    assert mids.min() >= N and mids.max() < m.num_nodes
    # every node is used, every element has four distinct corners
    assert np.array_equal(np.unique(t), np.arange(m.num_nodes))
    assert all(len(set(row)) == 4 for row in corners[:200])
    # positive rest volume (FFEA's orientation) after the jitter
    a, b, c, d = (p[corners[:, i]] for i in range(4))
    vol = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) / 6.0
    assert vol.min() > 0.5 * m.cell ** 3 / 6.0
    # the midpoint of each edge: one node per edge, at its middle
    seen = {}
    for k, (i, j) in enumerate(EDGES):
        lo = np.minimum(corners[:, i], corners[:, j])
        hi = np.maximum(corners[:, i], corners[:, j])
        np.testing.assert_allclose(p[mids[:, k]], 0.5 * (p[corners[:, i]] + p[corners[:, j]]), rtol=0, atol=1e-12)
        for e_lo, e_hi, mid in zip(lo[:500], hi[:500], mids[:500, k]):
            assert seen.setdefault((int(e_lo), int(e_hi)), int(mid)) == int(mid)
    # stokes radius only on the corner nodes
    assert (m.stokes_radius[:N] > 0).all() and (m.stokes_radius[N:] == 0).all()


def test_meshes_are_seeded():
    a, b, c = sphere_mesh(4.0, seed=7), sphere_mesh(4.0, seed=7), sphere_mesh(4.0, seed=8)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.topology, b.topology)
    assert np.array_equal(a.topology, c.topology) and not np.array_equal(a.pos, c.pos)
