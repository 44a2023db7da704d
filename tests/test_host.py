"""Host-side logic and the C ABI surface, without a GPU.

- The shared library loads and exports every function include/ffea_gpu.h declares.
- Invalid meshes are rejected on the host, with FFEA-style messages, before
  any device work.
- File formats round-trip; synthetic mesh sizes; unit conversions.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from ffea_gb300 import formats, params as P
from ffea_gb300.mesh import cube_mesh, make_blob, sphere_mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from ffea_gb300 import build as B
    B.build()
    from ffea_gb300 import _lib as L
    return L.lib()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "ffea_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ffea_gpu_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    from ffea_gb300 import _lib as L
    assert set(names) == set(L.SIGNATURES), set(names) ^ set(L.SIGNATURES)


def test_host_rejects_out_of_range_topology(lib):
    from ffea_gb300 import _lib as L
    from ffea_gb300.world import World
    s = make_blob(sphere_mesh(2.5, seed=0), P.SimulationParams())
    topo = s.mesh.topology.copy()
    topo[3, 7] = s.mesh.num_nodes + 5
    bad = {"mesh": {"pos": s.mesh.pos, "topology": topo}, "material": s.material, "drag": s.drag,
           "pinned": None, "params": s.params}
    with pytest.raises(L.FfeaGpuError, match="out of bounds node index"):
        World([bad])


def test_host_rejects_corner_midpoint_mixup(lib):
    from ffea_gb300 import _lib as L
    from ffea_gb300.world import World
    s = make_blob(sphere_mesh(2.5, seed=0), P.SimulationParams())
    topo = s.mesh.topology.copy()
    topo[0, 5] = topo[1, 0]
    bad = {"mesh": {"pos": s.mesh.pos, "topology": topo}, "material": s.material, "drag": s.drag,
           "pinned": None, "params": s.params}
    with pytest.raises(L.FfeaGpuError, match="corner of one element and a midpoint"):
        World([bad])


def _with(s, **over):
    d = {"mesh": {"pos": s.mesh.pos, "topology": s.mesh.topology}, "material": s.material, "drag": s.drag,
         "pinned": None, "params": s.params}
    for k, v in over.items():
        if k in ("pos", "topology"):
            d["mesh"][k] = v
        else:
            d[k] = v
    return d


@pytest.mark.parametrize("case,match", [
    ("pinned_high", "pinned node index out of range"),
    ("pinned_negative", "pinned node index out of range"),
    ("repeated_corner", "repeats a corner node"),
    ("negative_index", "out of bounds node index"),
    ("empty", "empty mesh"),
])
def test_host_rejects_invalid_blobs(lib, case, match):
    """Each invalid blob is refused by ffea_gpu_create_batch on the host, with
    FFEA_ERROR and a message naming the fault, before any device work."""
    from ffea_gb300 import _lib as L
    from ffea_gb300.world import World
    s = make_blob(sphere_mesh(2.5, seed=0), P.SimulationParams())
    t = s.mesh.topology.copy()
    if case == "pinned_high":
        bad = _with(s, pinned=np.array([s.mesh.num_nodes + 3], np.int32))
    elif case == "pinned_negative":
        bad = _with(s, pinned=np.array([-1], np.int32))
    elif case == "repeated_corner":
        t[0, 1] = t[0, 0]
        bad = _with(s, topology=t)
    elif case == "negative_index":
        t[2, 2] = -1
        bad = _with(s, topology=t)
    else:
        bad = _with(s, topology=np.zeros((0, 10), np.int32), material=np.zeros((0, 5)))
    with pytest.raises(L.FfeaGpuError, match=match):
        World([bad])


def test_ffea_seed_through_the_abi(lib, oracle):
    from ffea_gb300.world import ffea_seed
    for s in (0, 44, 123456789):
        assert np.array_equal(ffea_seed(s), oracle.ffea_seed(s))


def test_mesh_sizes_match_the_stated_configs():
    m = sphere_mesh(10.0)
    assert (m.num_linear, m.num_elements, m.num_nodes) == (2771, 12996, 19683)
    m = cube_mesh(16)
    assert (m.num_linear, m.num_elements, m.num_nodes) == (4913, 24576, 35937)
    # every element positively oriented, midpoints exact
    a, b, c, d = (m.pos[m.topology[:, i]] for i in range(4))
    det = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    assert (det > 0).all()
    assert np.allclose(m.pos[m.topology[:, 4]], 0.5 * (a + b))


def test_formats_round_trip(tmp_path):
    m = sphere_mesh(3.0, seed=2)
    E = m.num_elements
    mat = np.tile([1.5e3, 1e-3, 1e-3, 3.7e8, 1.1e9, 1.0], (E, 1))
    files = formats.BlobFiles(m.pos, len(m.pos), m.topology, E, mat, m.stokes_radius, np.array([0, 4], np.int32))
    prefix = str(tmp_path / "blob")
    formats.write_blob(prefix, files)
    back = formats.read_blob(prefix + ".node", prefix + ".top", prefix + ".mat", prefix + ".stokes", prefix + ".pin")
    assert np.array_equal(back.pos, m.pos)
    assert np.array_equal(back.topology, m.topology)
    assert np.array_equal(back.material_si, mat)
    assert np.array_equal(back.stokes_radius, m.stokes_radius)
    assert list(back.pinned) == [0, 4]


def test_unit_conversions():
    p = P.SimulationParams.from_si(dt=1e-14, kT=4.11e-21, epsilon=1e-6, stokes_visc=1e-3)
    assert abs(p.dt - 1e-14 / 3.7302915560886126e-13) < 1e-15
    assert abs(p.epsilon2 - 1e-12) < 1e-24
    m = P.material_si_to_meso([1.5e3], [1e-3], [1e-3], [3.7e8], [1.1e9])[0]
    A = 1e-3 / (8.4305832688784826e8 * 3.7302915560886126e-13)
    assert abs(m[1] - A) < 1e-12
    # the second viscosity subtracts an SI shear viscosity (src/Blob.cpp:2865)
    assert abs(m[2] - (A - (2.0 / 3.0) * 1e-3)) < 1e-12
    assert abs(P.kT_at(300.0) - 1.380649e-23 * 300 / 4.141945559999999e-21) < 1e-12


def test_torch_custom_op_is_registered():
    """The training-loop operator registers with torch.library without a GPU
    and checks the parameter count before it reaches the library."""
    import pytest
    import torch

    from ffea_gb300 import learned, torch_ops
    assert hasattr(torch.ops.ffea.mpnn_loss_grad, "default")

    class _W:
        handle = 0
    with pytest.raises(ValueError, match=str(learned.NUM_PARAMS)):
        torch_ops.mpnn_loss(_W(), torch.zeros(3))
