"""The learned preconditioner's host side (ffea_gb300.learned), on the CPU:
the flat parameter layout (the library's MPNN_NUM_PARAMS = 4,737), the
initialisation that makes the untrained network the plain two-level
preconditioner, Adam against its published update, the weight file, and
the seeded training family."""
import numpy as np
import pytest

from ffea_gb300 import learned as Lr


def test_layout_is_contiguous_and_complete():
    lay, total = Lr.layout()
    assert total == Lr.NUM_PARAMS == 2 * 32 * 8 + 32 + 2 * (2 * 32 * 32 + 32) + 32 + 1 == 4737
    spans = sorted((o, o + int(np.prod(s))) for o, s in lay.values())
    assert spans[0][0] == 0 and spans[-1][1] == total
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    parts = Lr.unpack(np.arange(total, dtype=np.float32))
    assert parts["ws0"].shape == (32, 8) and parts["wn2"].shape == (32, 32) and parts["bo"].shape == (1,)
    assert parts["ws0"][0, 0] == lay["ws0"][0] and parts["bo"][0] == total - 1


def test_untrained_network_is_the_plain_two_level_preconditioner():
    th = Lr.init_params(5)
    p = Lr.unpack(th)
    # omega = 2 sigmoid(wo . h + bo) = 1 for every node when wo = bo = 0
    assert not p["wo"].any() and not p["bo"].any()
    assert not any(p[f"b{l}"].any() for l in range(3))
    assert np.array_equal(th, Lr.init_params(5)) and not np.array_equal(th, Lr.init_params(6))
    assert p["ws1"].std() == pytest.approx(np.sqrt(1.0 / 32), rel=0.1)


def test_adam_matches_its_published_update():
    opt = Lr.Adam(lr=0.1)
    theta = np.ones(Lr.NUM_PARAMS, np.float32)
    g = np.full(Lr.NUM_PARAMS, 2.0, np.float32)
    t1 = opt.step(theta, g)
    # first step: m^ = g, v^ = g^2, so theta - lr * g / (|g| + eps)
    np.testing.assert_allclose(t1, 1.0 - 0.1 * 2.0 / (2.0 + 1e-8), rtol=1e-6)
    t2 = opt.step(t1, -g)
    m = 0.9 * 0.1 * 2.0 + 0.1 * -2.0
    v = 0.999 * 0.001 * 4.0 + 0.001 * 4.0
    mh, vh = m / (1 - 0.9 ** 2), v / (1 - 0.999 ** 2)
    np.testing.assert_allclose(t2, t1 - 0.1 * mh / (np.sqrt(vh) + 1e-8), rtol=1e-6)


def test_weight_file_round_trip_and_committed_weights(tmp_path):
    th = Lr.init_params(1)
    path = str(tmp_path / "w.npz")
    Lr.save(th, path, pairs=10)
    assert np.array_equal(Lr.load(path), th)
    Lr.save(th[:-1], path)
    with pytest.raises(ValueError, match="parameters, expected 4737"):
        Lr.load(path)
    committed = Lr.load()
    assert committed.dtype == np.float32 and np.isfinite(committed).all()
    assert np.abs(Lr.unpack(committed)["wo"]).sum() > 0  # trained, not the initial state


def test_training_family_is_seeded():
    a, b = Lr.training_meshes(3), Lr.training_meshes(3)
    assert [s.mesh.num_linear for s in a] == [s.mesh.num_linear for s in b]
    radii_nodes = [s.mesh.num_linear for s in Lr.training_meshes(8)]
    assert min(radii_nodes) > 200 and max(radii_nodes) < 40000
    assert len({s.params.rng_seed for s in a}) == 3
