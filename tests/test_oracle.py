"""The oracle pinned against FFEA's own known answers and compiled objects (CPU).

- RngStream's package known-answer test (tests/consistency/rngstream/
  testRngStream.cpp: the sum printed at precision 14 must read 39.697547445251).
- World::init's seeding for rng_seed 44 and a 2e7-draw stream fingerprint.
- The glibc rand() restatement against the C library itself.
- Golden vectors made by FFEA's own objects (tests/golden/make_golden.py):
  bit-exact positions, velocities, rhs, element forces and RNG state.
- Where the FFEA sources are present: the oracle against the reference
  objects step by step, bit for bit.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_rngstream_package_kat(oracle):
    assert f"{oracle.rng_package_kat():.14g}" == "39.697547445251"


def test_ffea_seed_44(oracle):
    assert [int(v) for v in oracle.ffea_seed(44)] == [3015861669, 1834431885, 558792412, 113187832, 1288513475,
                                                      2073327934]


def test_glibc_rand_restatement_matches_libc(oracle):
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("not a glibc system")
    for seed in (0, 1, 44, 12345, 2**31 - 1, 987654321):
        libc.srand(ctypes.c_uint(seed))
        two_max = [4294967087, 4294944443]
        want = []
        for i in range(6):
            a, b = libc.rand(), libc.rand()
            s = (a + b + 2**31) % 2**32 - 2**31  # the int sum wraps
            want.append((s % 2**64) % two_max[i // 3])
        assert [int(v) for v in oracle.ffea_seed(seed)] == want, seed


def test_stream_fingerprint_2e7_draws(oracle):
    # rng[0] of a one-thread run with rng_seed 44: the sequential sum of 2e7
    # draws, and a word-wise FNV-style hash h = (h ^ bits(u)) * 0x100000001b3
    # (start 0xcbf29ce484222325) of the raw doubles; both values were produced
    # by FFEA's own RngStream objects, compiled from its sources (oracle/_ref).
    total, h = oracle.rng_fingerprint(oracle.ffea_seed(44), 20_000_000)
    assert f"{total:.9f}" == "9999475.672332041"
    assert f"{h:016x}" == "59ab4718a3015f4e"


def test_jump_equals_sequential(oracle):
    st = oracle.ffea_seed(7)
    seq, _ = oracle.rng_draws(st, 5000)
    for off in (0, 1, 17, 256, 4095, 4999):
        jumped = oracle.rng_jump(st, off)
        d, _ = oracle.rng_draws(jumped, 1)
        assert d[0] == seq[off]


def _golden_cases():
    # blob-update step goldens; cubes_lj.npz (surface interactions) has its own tests
    return sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz")) if not p.endswith("cubes_lj.npz"))


@pytest.mark.parametrize("path", _golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_golden(oracle, path):
    g = np.load(path)
    fp, ip = g["fparams"], g["iparams"]
    b = oracle.OracleBlob(g["pos0"], g["topology"], g["material"], g["drag"], g["pinned"], fp[0], fp[1], fp[2],
                          int(ip[0]), int(ip[1]), int(ip[2]), int(ip[3]), 1, "port")
    b.seed(int(ip[4]))
    assert np.array_equal(b.rng_state(), g["rng0"])
    done = 0
    for s in (1, 2, 6):
        assert b.step(s - done) == 0
        done = s
        pos, vel, force = b.nodes()
        assert np.array_equal(pos, g[f"pos_{s}"]), s
        assert np.array_equal(vel, g[f"vel_{s}"]), s
        assert np.array_equal(force, g[f"force_{s}"]), s
        assert np.array_equal(b.rhs(), g[f"rhs_{s}"]), s
        assert np.array_equal(b.element_forces(), g[f"efrc_{s}"]), s
        assert np.array_equal(b.rng_state(), g[f"rng_{s}"]), s


def _ref_mesh():
    from oracle import oracle as O
    src = O.reference_src()
    return os.path.join(src, "tests/physics/sphere_63_120_structure/sphere_63_120") if src else ""


REF_MESH = _ref_mesh()


@pytest.mark.skipif(not os.path.exists(REF_MESH + ".node"), reason="FFEA sources not present")
@pytest.mark.parametrize("solver", [0, 1, 2])
def test_oracle_matches_reference_objects_sphere_63_120(oracle, solver):
    oracle.build(ref=True)
    if not oracle.ref_available():
        pytest.skip("reference objects not built")
    from ffea_gb300 import formats, params as P
    f = formats.read_blob(REF_MESH + ".node", REF_MESH + ".top", REF_MESH + ".mat", REF_MESH + ".stokes",
                          REF_MESH + ".pin")
    prm = P.SimulationParams.from_si(dt=1e-14, kT=4.11e-21, epsilon=1e-12, rng_seed=44, solver=solver)
    pos, topo, mat, drag, pins = formats.blob_arrays_from_files(f, 5e-9, prm.stokes_visc)
    blobs = [oracle.OracleBlob(pos, topo, mat, drag, pins, prm.dt, prm.kT, prm.epsilon2, 1000, 1, 1, solver, 1, impl)
             for impl in ("port", "ref")]
    for b in blobs:
        b.seed(44)
    for _ in range(10):
        assert [b.step(1) for b in blobs] == [0, 0]
        for x, y in zip(blobs[0].nodes(), blobs[1].nodes()):
            assert np.array_equal(x, y)
        assert np.array_equal(blobs[0].rng_state(), blobs[1].rng_state())


def test_all_pinned_blob_draws_node_noise_only(oracle):
    """A blob with every node pinned skips its element loop
    (src/Blob.cpp:643-645), so a step draws only the 3 N_t node values of
    aggregate_forces_and_solve.  With the mass solver nothing moves; FFEA's
    NoMassCGSolver divides 0 by 0 on the all-zero rhs (alpha before its
    stopping test, src/NoMassCGSolver.cpp:165-197), so its positions become
    NaN -- the oracle restates that too.  The reference objects agree where
    they are built."""
    from tests.helpers import spec
    s0 = spec(radius_nm=3.0)
    for solver in (0, 1):
        s = spec(radius_nm=3.0, solver=solver, pinned=list(range(s0.mesh.num_nodes)))
        b = oracle.blob_from_spec(s)
        st0 = b.rng_state()
        assert b.step(3) == 0
        assert np.array_equal(b.rng_state(), oracle.rng_jump(st0, 3 * 3 * s.mesh.num_nodes))
        pos, vel, _ = b.nodes()
        if solver == 1:
            corner = np.zeros(len(pos), bool)
            corner[s.mesh.topology[:, :4]] = True
            assert np.array_equal(pos[corner], s.mesh.pos[corner]) and not vel.any()
        else:
            assert np.isnan(pos).all()
        if oracle.ref_available():
            r = oracle.blob_from_spec(s, impl="ref")
            assert r.step(3) == 0
            assert np.array_equal(r.rng_state(), b.rng_state())
            for x, y in zip(r.nodes(), b.nodes()):
                assert np.array_equal(x, y, equal_nan=True)
