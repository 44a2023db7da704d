"""The .ffea script front end (ffea_gpu_script_load, C++), on the CPU.

  - the <param> values against FFEA's own SimulationParams reading of the same
    script (oracle/_ref: FFEA_input_reader + SimulationParams::extract_params,
    where the FFEA sources are present), exactly;
  - the blob arrays against the Python loaders of ffea_gb300.formats with
    Blob::init's scaling, material conversion and Stokes drag, and FFEA's
    centroid placement (Blob::position: node sum, times 1/N, shift) and
    velocity_all, exactly;
  - comments (one spanning lines), file names relative to the script, a
    blob written without a <conformation> block, FFEA's default output names;
  - the errors: an unknown parameter, a missing scale, a switch of work
    outside the blob update, a missing file, an out-of-bounds topology.
The scripts and mesh files are written by the test from synthetic meshes."""
import ctypes
import os

import numpy as np
import pytest

from ffea_gb300 import formats as F
from ffea_gb300 import params as P
from ffea_gb300.mesh import cube_mesh, sphere_mesh

PARAM = """<param>
    <!-- a comment on one line -->
    <restart = 0>
    <dt = 2e-14>
    <kT = 4.11e-21>
    <check = 5>
    <num_steps = 1e3>
    <rng_seed = 31>
    <trajectory_out_fname = out/run_trajectory.ftj>
    <measurement_out_fname = out/run_measurement.out>
    <epsilon = 1e-6>
    <max_iterations_cg = 700>
    <kappa = 1e9>
    <!-- a comment
         over two lines -->
    <dielec_ext = 1>
    <epsilon_0 = 1>
    <do_stokes = 1>
    <stokes_visc = 2e-03>
    <calc_vdw = 0>
    <calc_noise = 1>
    <calc_kinetics = 0>
    <calc_es = 0>
    <es_N_x = 0>
    <wall_x_1 = PBC>
    <es_h = 3>
    <num_blobs = 2>
    <num_conformations = (1,1)>
    <num_states = (1,1)>
</param>
"""

SYSTEM = """<system>
    <blob>
        <conformation>
            <motion_state = DYNAMIC>
            <nodes = mesh/a.node>
            <topology = mesh/a.top>
            <surface = mesh/a.surf>
            <material = mesh/a.mat>
            <stokes = mesh/a.stokes>
            <vdw = mesh/a.vdw>
            <pin = mesh/a.pin>
        </conformation>
        <solver = CG_nomass>
        <scale = 1e-9>
        <centroid = (1.5, -2.0, 0.25)>
    </blob>
    <blob>
        <motion_state = DYNAMIC>
        <nodes = mesh/b.node>
        <topology = mesh/b.top>
        <material = mesh/b.mat>
        <stokes = mesh/b.stokes>
        <solver = CG>
        <scale = 2e-9>
        <velocity = (10.0, 0.0, -5.0)>
    </blob>
</system>
"""


def _files(mesh, seed, pinned=()):
    rng = np.random.default_rng(seed)
    n, e = mesh.num_nodes, mesh.num_elements
    mat = np.column_stack([np.full(e, 1.5e3), np.full(e, 1e-3), np.full(e, 1e-3), rng.uniform(1e8, 5e8, e),
                           np.full(e, 1.1e9), np.ones(e)])
    pos_file = mesh.pos * P.MESO_LENGTH / 1e-9  # file units of a scale-1e-9 script
    return F.BlobFiles(pos=pos_file, num_surface_nodes=n // 3, topology=mesh.topology, num_surface_elements=e // 4,
                       material_si=mat, stokes_radius=np.where(np.arange(n) < mesh.num_linear, 0.3, 0.0),
                       pinned=np.asarray(pinned, np.int32))


@pytest.fixture()
def script(tmp_path):
    os.makedirs(tmp_path / "mesh")
    a = _files(sphere_mesh(3.0, seed=3), 1, pinned=(0, 5))
    b = _files(cube_mesh(2, seed=4), 2)
    F.write_blob(str(tmp_path / "mesh" / "a"), a)
    F.write_blob(str(tmp_path / "mesh" / "b"), b)
    path = tmp_path / "run.ffea"
    path.write_text(PARAM + "\n" + SYSTEM)
    return str(path), a, b


def _load(path):
    from ffea_gb300.script import Script
    return Script(path)


def _expected_blob(files, scale_si, stokes_visc, centroid=None, velocity=None):
    pos, topo, mat, drag, pinned = F.blob_arrays_from_files(files, scale_si, stokes_visc)
    if centroid is not None:
        scale = scale_si / P.MESO_LENGTH
        c = [0.0, 0.0, 0.0]
        for k in range(len(pos)):
            for d in range(3):
                c[d] += pos[k, d]
        for d in range(3):
            c[d] *= 1.0 / len(pos)
            pos[:, d] += centroid[d] * scale - c[d]
    vel = np.zeros_like(pos)
    if velocity is not None:
        vel[:] = np.asarray(velocity) / P.MESO_VELOCITY
    return pos, vel, topo, mat, drag, pinned


def test_params_and_blobs(gpulib_cpu, script):
    path, a, b = script
    with _load(path) as sc:
        p = sc.params
        assert p["num_blobs"] == 2 and sc.num_blobs == 2
        assert p["dt"] == 2e-14 / P.MESO_TIME
        assert p["kT"] == 4.11e-21 / P.MESO_ENERGY
        assert p["epsilon2"] == 1e-6 * 1e-6
        assert p["stokes_visc"] == 2e-3 / (P.MESO_PRESSURE * P.MESO_TIME)
        assert (p["num_steps"], p["check"], p["rng_seed"], p["max_iterations_cg"]) == (1000, 5, 31, 700)
        assert (p["calc_noise"], p["calc_stokes"], p["restart"]) == (1, 1, 0)
        d = os.path.dirname(path)
        assert p["trajectory_out_fname"] == os.path.join(d, "out/run_trajectory.ftj")
        assert p["measurement_out_fname"] == os.path.join(d, "out/run_measurement.out")
        assert p["checkpoint_out"] == os.path.join(d, "run.fcp") and p["checkpoint_in"] == ""
        for i, (files, scale, kw, solver) in enumerate(
                ((a, 1e-9, {"centroid": (1.5, -2.0, 0.25)}, P.SOLVER_NOMASS),
                 (b, 2e-9, {"velocity": (10.0, 0.0, -5.0)}, P.SOLVER_MASS))):
            got = sc.blob(i)
            pos, vel, topo, mat, drag, pinned = _expected_blob(files, scale, p["stokes_visc"], **kw)
            assert np.array_equal(got["pos"], pos), i
            assert np.array_equal(got["vel"], vel), i
            assert np.array_equal(got["topology"], topo), i
            assert np.array_equal(got["material"], mat), i
            assert np.array_equal(got["drag"], drag), i
            assert np.array_equal(got["pinned"], pinned), i
            assert got["params"]["solver"] == solver
            assert got["params"]["rng_seed"] == 31 and got["params"]["epsilon2"] == p["epsilon2"]
        # the centroid lands where the script puts it
        c = sc.blob(0)["pos"].mean(axis=0) * P.MESO_LENGTH / 1e-9
        assert np.allclose(c, (1.5, -2.0, 0.25), atol=1e-12)


def test_params_match_ffea_simulation_params(gpulib_cpu, script, oracle):
    """The reference's own SimulationParams reading of the same script."""
    oracle.build(ref=True)
    if not oracle.ref_available():
        pytest.skip("FFEA sources not present")
    path, _, _ = script
    lib = oracle.ref_lib()
    fn = lib.ref_script_params
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    out = np.zeros(12)
    assert fn(path.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    with _load(path) as sc:
        p = sc.params
        got = [p["dt"], p["kT"], p["epsilon2"], p["stokes_visc"], p["num_steps"], p["check"], p["rng_seed"],
               p["max_iterations_cg"], p["calc_noise"], p["calc_stokes"], p["restart"], p["num_blobs"]]
    assert np.array_equal(np.asarray(got, dtype=np.float64), out), (got, out)


@pytest.mark.parametrize("edit,message", [
    (lambda t: t.replace("<es_h = 3>", "<es_h = 3>\n    <not_a_parameter = 1>"), "not a recognised parameter"),
    (lambda t: t.replace("<scale = 2e-9>", ""), "scale not set"),
    (lambda t: t.replace("<calc_es = 0>", "<calc_es = 1>"), "outside the GPU blob update"),
    (lambda t: t.replace("mesh/b.top", "mesh/missing.top"), "does not exist"),
    (lambda t: t.replace("<motion_state = DYNAMIC>\n        <nodes = mesh/b.node>",
                         "<motion_state = FROZEN>\n        <nodes = mesh/b.node>"), "DYNAMIC only"),
    (lambda t: t.replace("<solver = CG>", "<solver = direct>"), "direct solver"),
    (lambda t: t.replace("<rng_seed = 31>", ""), "rng_seed"),
])
def test_errors(gpulib_cpu, script, edit, message):
    from ffea_gb300._lib import FfeaGpuError
    path, _, _ = script
    with open(path) as fh:
        text = fh.read()
    with open(path, "w") as fh:
        fh.write(edit(text))
    with pytest.raises(FfeaGpuError, match=message):
        _load(path)


def test_out_of_bounds_topology(gpulib_cpu, script):
    from ffea_gb300._lib import FfeaGpuError
    path, _, b = script
    d = os.path.join(os.path.dirname(path), "mesh")
    bad = F.BlobFiles(**{**b.__dict__, "topology": np.where(b.topology == 0, 10 ** 6, b.topology)})
    F.write_blob(os.path.join(d, "b"), bad)
    with pytest.raises(FfeaGpuError, match="out of bounds"):
        _load(path)
