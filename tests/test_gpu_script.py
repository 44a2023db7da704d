"""FFEA scripts run on the GPU (World.from_script, ffea_gb300.script.run).

  - a two-blob script (NoMass with pins and a centroid, mass solver with a
    velocity) built by the C++ front end steps bit for bit like the same
    blobs handed to ffea_gpu_create_batch from Python (one shared stream);
  - a one-blob script in FP64 against the oracle stepping the script's
    arrays: velocities to 1e-9 relative, positions to 1e-10, RNG state exact;
  - script.run writes FFEA's trajectory, measurement and checkpoint files,
    and a restart from checkpoint_in (restart = 1) ends where a straight run
    ends: the same final checkpoint and positions to 5e-4 of the largest
    coordinate (the trajectory holds FFEA's %e precision), as the
    reference's restart test checks (tests/physics/sphere_63_120_nomass_restart/checkRuns.py:33-83).
"""
import os

import numpy as np
import pytest

from tests.helpers import rel
from tests.test_script import PARAM, SYSTEM, _files

pytestmark = pytest.mark.gpu


def _write(tmp_path, param=PARAM, system=SYSTEM, name="run.ffea"):
    from ffea_gb300 import formats as F
    from ffea_gb300.mesh import cube_mesh, sphere_mesh
    os.makedirs(tmp_path / "mesh", exist_ok=True)
    os.makedirs(tmp_path / "out", exist_ok=True)
    F.write_blob(str(tmp_path / "mesh" / "a"), _files(sphere_mesh(3.0, seed=3), 1, pinned=(0, 5)))
    F.write_blob(str(tmp_path / "mesh" / "b"), _files(cube_mesh(2, seed=4), 2))
    path = tmp_path / name
    path.write_text(param + "\n" + system)
    return str(path)


def test_script_world_equals_python_batch(gpulib, tmp_path):
    from ffea_gb300.params import PRECISION_MIXED
    from ffea_gb300.script import Script
    from ffea_gb300.world import RNG_SHARED, World
    path = _write(tmp_path)
    with Script(path) as sc:
        blobs = []
        for i in range(sc.num_blobs):
            b = sc.blob(i)
            blobs.append({"mesh": {"pos": b["pos"], "topology": b["topology"]}, "material": b["material"],
                          "drag": b["drag"], "pinned": b["pinned"], "params": sc.simulation_params(i, PRECISION_MIXED)})
        vels = [sc.blob(i)["vel"] for i in range(sc.num_blobs)]
    with World.from_script(path) as w1, World(blobs, rng_mode=RNG_SHARED, true_residual=True, velocities=vels) as w2:
        w1.run(5)
        w2.run(5)
        for i in range(2):
            for x, y in zip(w1.blob(i).get_nodes(), w2.blob(i).get_nodes()):
                assert np.array_equal(x, y), i
            assert np.array_equal(w1.blob(i).rng_state(), w2.blob(i).rng_state())


def test_one_blob_script_fp64_matches_oracle(gpulib, oracle, tmp_path):
    from ffea_gb300.params import PRECISION_FP64
    from ffea_gb300.script import Script
    from ffea_gb300.world import World
    param = PARAM.replace("<num_blobs = 2>", "<num_blobs = 1>").replace("(1,1)", "(1)").replace(
        "<epsilon = 1e-6>", "<epsilon = 1e-12>")
    system = SYSTEM[:SYSTEM.index("    <blob>\n        <motion_state")] + "</system>\n"
    path = _write(tmp_path, param, system)
    with Script(path) as sc:
        b = sc.blob(0)
        p = sc.params
        ref = oracle.OracleBlob(b["pos"], b["topology"], b["material"], b["drag"], b["pinned"], p["dt"], p["kT"],
                                p["epsilon2"], p["max_iterations_cg"], p["calc_noise"], p["calc_stokes"], 0)
        ref.seed(p["rng_seed"])
    with World.from_script(path, precision=PRECISION_FP64, true_residual=False) as w:
        for step in range(5):
            w.run(1)
            assert ref.step(1) == 0
            pos, vel, _ = w.blob(0).get_nodes()
            rpos, rvel, _ = ref.nodes()
            assert np.array_equal(w.blob(0).rng_state(), ref.rng_state()), step
            assert rel(vel, rvel) < 1e-9, step
            assert np.abs(pos - rpos).max() < 1e-10, step


def _last_checkpoint(path):
    with open(path) as fh:
        return fh.read()


def test_run_and_restart(gpulib, tmp_path):
    from ffea_gb300 import script as S
    from ffea_gb300.trajectory import read_last_frame
    straight = _write(tmp_path / "a", PARAM.replace("<num_steps = 1e3>", "<num_steps = 10>"))
    S.run(straight)
    d = os.path.dirname(straight)
    traj = os.path.join(d, "out/run_trajectory.ftj")
    meas = os.path.join(d, "out/run_measurement.out")
    assert os.path.exists(traj) and os.path.exists(meas) and os.path.exists(os.path.join(d, "run.fcp"))
    with open(traj) as fh:
        text = fh.read()
    assert all(f"Blob 0, Conformation 0, step {s}\n" in text for s in (0, 5, 10))
    # 5 steps, then restart = 1 from the checkpoint for 10 steps in all
    first = _write(tmp_path / "b", PARAM.replace("<num_steps = 1e3>", "<num_steps = 5>"))
    S.run(first)
    d2 = os.path.dirname(first)
    os.replace(os.path.join(d2, "run.fcp"), os.path.join(d2, "run_in.fcp"))
    second = PARAM.replace("<num_steps = 1e3>", "<num_steps = 10>").replace(
        "<restart = 0>", "<restart = 1>\n    <checkpoint_in = run_in.fcp>")
    path2 = os.path.join(d2, "run.ffea")
    with open(path2, "w") as fh:
        fh.write(second + "\n" + SYSTEM)
    S.run(path2)
    assert _last_checkpoint(os.path.join(d2, "run.fcp")) == _last_checkpoint(os.path.join(d, "run.fcp"))
    nodes = None
    from ffea_gb300.script import Script
    with Script(straight) as sc:
        nodes = [len(sc.blob(i)["pos"]) for i in range(sc.num_blobs)]
    s1, f1 = read_last_frame(traj, nodes)
    s2, f2 = read_last_frame(os.path.join(d2, "out/run_trajectory.ftj"), nodes)
    assert s1 == s2 == 10
    for (p1, v1), (p2, v2) in zip(f1, f2):
        assert np.abs(p1 - p2).max() <= 5e-4 * np.abs(p1).max()
