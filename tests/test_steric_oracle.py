"""The steric restatement (oracle/steric_oracle.c) on the CPU.

  - exact cases: identical tetrahedra (the whole volume, the vertex mean),
    disjoint ones (nothing), one inside the other (the inner volume);
  - against FFEA's own compiled geometry (oracle/_ref: volumeIntersectionII,
    Face::getTetraIntersectionVolumeTotalGradientAndShapeFunctions), where
    the FFEA sources are present, on 3,000 random tetrahedron pairs:
      * the overlap volume and centre agree to 1e-9 on at least 97 % of
        the overlapping pairs; on the others FFEA's volume is wrong: a Monte
        Carlo estimate (200,000 points) sides with the restatement;
      * where all seven of FFEA's volumes of a pair are right, the forces
        agree to 1e-7 of their scale (the larger of their largest component
        and the overlap's V^(2/3), the order of dV/dr);
  - the steric pass over two overlapping spheres conserves momentum: every
    pair adds phi1 k dV/dr to one face and -phi2 k dV/dr to the other, and
    each set of barycentric weights sums to one.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O


def test_exact_cases():
    T = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.]])
    v, cm = O.steric_overlap(T, T)
    assert v == pytest.approx(1 / 6, rel=1e-14) and np.allclose(cm, 0.25, atol=1e-14)
    v, _ = O.steric_overlap(T, T + 5.0)
    assert v == 0.0
    v, _ = O.steric_overlap(T, 0.5 * T + 0.05)
    assert v == pytest.approx(1 / 48, rel=1e-12)
    assert O.steric_pair(T, T + 5.0, 5e-3) is None


def _inside(T, X):
    M = np.array([T[1] - T[0], T[2] - T[0], T[3] - T[0]]).T
    L = np.linalg.solve(M, (X - T[0]).T).T
    return (L >= 0).all(1) & (L.sum(1) <= 1)


def test_against_ffea_geometry(oracle):
    oracle.build(ref=True)
    if not oracle.ref_available():
        pytest.skip("FFEA sources not present")
    ref = oracle.ref_lib()
    dp = ctypes.POINTER(ctypes.c_double)
    ref.ref_overlap_volume.restype = ctypes.c_double
    ref.ref_overlap_volume.argtypes = [dp, dp, ctypes.c_int, dp]
    ref.ref_steric_pair.argtypes = [dp, dp, ctypes.c_double, dp]
    P = lambda a: a.ctypes.data_as(dp)

    def ffea_volume(A, B, cm=None):
        c = np.zeros(3)
        v = ref.ref_overlap_volume(P(np.ascontiguousarray(A)), P(np.ascontiguousarray(B)), cm is not None, P(c))
        if cm is not None:
            cm[:] = c
        return v

    rng = np.random.default_rng(1)
    dr = 5e-3
    n_ov = n_agree = n_force = 0
    worst_force = 0.0
    for _ in range(3000):
        A = rng.normal(size=(4, 3))
        B = rng.normal(size=(4, 3)) * rng.uniform(0.3, 1.5) + rng.normal(size=3) * 0.7
        cm_f = np.zeros(3)
        vf = ffea_volume(A, B, cm_f)
        vo, cm_o = O.steric_overlap(A, B)
        if vf <= 1e-6:
            continue
        n_ov += 1
        if abs(vo - vf) <= 1e-9 * vf and np.abs(cm_o - cm_f).max() <= 1e-9 * np.abs(A).max():
            n_agree += 1
        else:
            # FFEA's volume is off: a Monte Carlo estimate decides
            lo = np.minimum(A.min(0), B.min(0))
            hi = np.maximum(A.max(0), B.max(0))
            X = lo + (hi - lo) * rng.random((200_000, 3))
            mc = (_inside(A, X) & _inside(B, X)).mean() * np.prod(hi - lo)
            se = np.prod(hi - lo) * np.sqrt(max(mc / np.prod(hi - lo), 1e-6) / 200_000)
            assert abs(mc - vo) < 5 * se + 1e-3 * vo < abs(mc - vf) + 5 * se, (vo, vf, mc)
        # forces where every volume FFEA takes for the gradient is right
        shifted = [(A, B)] + [(A, B + dr * np.eye(3)[d]) for d in range(3)] + [(B, A + dr * np.eye(3)[d]) for d in range(3)]
        if all(abs(O.steric_overlap(X, Y)[0] - ffea_volume(X, Y)) <= 1e-9 * max(ffea_volume(X, Y), 1e-300)
               for X, Y in shifted):
            out = np.zeros(14)
            ref.ref_steric_pair(P(np.ascontiguousarray(A)), P(np.ascontiguousarray(B)), dr, P(out))
            r1 = np.outer(out[6:10], out[3:6])
            r2 = -np.outer(out[10:14], out[3:6])
            _, f1, f2 = O.steric_pair(A, B, dr)
            # dV/dr is of the order of the overlap's surface area (where the
            # overlap hardly changes under a shift, it is at round-off level)
            scale = max(np.abs(r1).max(), np.abs(r2).max(), vf ** (2.0 / 3.0))
            worst_force = max(worst_force, np.abs(f1 - r1).max() / scale, np.abs(f2 - r2).max() / scale)
            n_force += 1
    assert n_ov > 900
    assert n_agree >= 0.97 * n_ov, (n_agree, n_ov)
    assert n_force >= 0.95 * n_ov
    assert worst_force <= 1e-7, worst_force


def overlapping_spheres(radius_nm=2.5, overlap_nm=0.6, seed=3):
    """Two spheres pushed 0.6 nm into each other: faces, fourth nodes, blobs, grid."""
    from ffea_gb300.mesh import sphere_mesh
    from ffea_gb300.params import nm
    from ffea_gb300.surface import surface_faces
    m = sphere_mesh(radius_nm, seed=seed)
    tri, apex = surface_faces(m.pos, m.topology, with_apex=True)
    x = m.pos - m.pos.mean(0)
    shift = np.array([2 * nm(radius_nm) - nm(overlap_nm), 0.0, 0.0])
    pos = np.concatenate([x, x + shift])
    n = len(x)
    faces = np.concatenate([tri, tri + n]).astype(np.int32)
    apexes = np.concatenate([apex, apex + n]).astype(np.int32)
    blob = np.repeat(np.arange(2, dtype=np.int32), len(tri))
    h = nm(1.5)
    span = pos.max(0) - pos.min(0)
    grid = tuple(int(v) for v in 2 * np.ceil(span / h))
    pos = pos - pos.mean(0) + 0.5 * h * np.array(grid)
    return pos, faces, apexes, blob, h, grid


@pytest.mark.parametrize("inc_self", [0, 1])
def test_steric_pass_conserves_momentum(inc_self):
    from ffea_gb300.params import nm
    pos, faces, apex, blob, h, grid = overlapping_spheres()
    f, e, pairs = O.ssint(pos, faces, blob, np.zeros(len(faces), np.int32), np.ones((1, 1)),
                          np.full((1, 1), nm(1.0)), 2, h, grid, inc_self, 1, apex, 50.0, 5e-3)
    assert pairs > 0 and e[0, 1] > 0
    assert np.abs(f.sum(0)).max() <= 1e-9 * np.abs(f).max()
