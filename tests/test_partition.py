"""The ensemble partitioner (ffea_gb300.partition) on the CPU.

  - estimate_sizes() against the synthetic sphere meshes it stands in for:
    corner nodes and elements within 10 %, edges within 15 %, 5-30 nm;
  - blob_cost() is the per-step byte model of its docstring;
  - pack() puts every blob in exactly one bin, is deterministic, never does
    worse than the largest single blob above the mean load, and beats a
    round-robin deal on an uneven ensemble.
"""
import numpy as np
import pytest

from ffea_gb300 import partition as Pt


@pytest.mark.parametrize("radius", [5.0, 10.0, 20.0, 30.0])
def test_estimated_sizes_match_built_spheres(radius):
    from ffea_gb300.mesh import sphere_mesh
    m = sphere_mesh(radius, cell_nm=1.25, seed=0)
    nodes, elems, edges = Pt.estimate_sizes(radius, 1.25)
    topo = np.asarray(m.topology).reshape(-1, 10)[:, :4]
    pairs = set()
    for t in topo:
        for a in range(4):
            for b in range(a + 1, 4):
                pairs.add((min(t[a], t[b]), max(t[a], t[b])))
    assert abs(nodes - m.num_linear) <= 0.10 * m.num_linear
    assert abs(elems - m.num_elements) <= 0.10 * m.num_elements
    assert abs(edges - len(pairs)) <= 0.15 * len(pairs)


def test_blob_cost_is_the_byte_model():
    N, E, ed, it = 1000, 5000, 6500, 90.0
    B = N + 2 * ed
    Nt = N + ed
    want = (12 * N + 168 * E) + 4 * (7 * E + 3 * Nt) + (104 * E + 36 * B) + (64 * E + 16 * N) + 48 * N
    want += it * (40 * B + 148 * N)
    assert Pt.blob_cost(N, E, ed, iterations=it) == pytest.approx(want)


def test_pack_balances_and_is_deterministic():
    rng = np.random.default_rng(0)
    costs = np.exp(rng.uniform(np.log(1.0), np.log(500.0), size=64))
    for ranks in (1, 2, 3, 8):
        bins, loads = Pt.pack(costs, ranks)
        assert sorted(i for b in bins for i in b) == list(range(64))
        assert np.allclose(loads, [costs[b].sum() for b in bins])
        assert max(loads) <= np.mean(loads) + costs.max() + 1e-9
        assert Pt.pack(costs, ranks) == (bins, loads)
        rr = [costs[r::ranks].sum() for r in range(ranks)]
        assert max(loads) <= max(rr) + 1e-9
    with pytest.raises(ValueError):
        Pt.pack(costs, 0)
