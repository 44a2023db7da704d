"""The CPU restatement of the smoother-weight network checks itself: its
backward pass against central differences (FP64, no BF16 emulation), and its
BF16 emulation against PyTorch's rounding."""
import numpy as np

from ffea_gb300.mesh import sphere_mesh
from oracle import mpnn


def _setup(seed=0):
    m = sphere_mesh(3.0, seed=seed)
    ptr, idx = mpnn.edge_neighbours(m.topology, m.num_nodes)
    n = m.num_linear
    rng = np.random.default_rng(seed)
    feats = np.zeros((m.num_nodes, mpnn.FEATURES))
    feats[:n] = rng.normal(size=(n, mpnn.FEATURES))
    feats[:n, 7] = 1.0
    from ffea_gb300.learned import NUM_PARAMS
    theta = rng.normal(0.0, 0.3, size=NUM_PARAMS)
    domega = np.zeros(m.num_nodes)
    domega[:n] = rng.normal(size=n)
    return theta, feats, ptr, idx, domega


def test_backward_matches_central_differences():
    theta, feats, ptr, idx, domega = _setup()
    om, cache = mpnn.forward(theta, feats, ptr, idx, emulate_bf16=False)
    g = mpnn.backward(theta, cache, om, domega, ptr, idx)
    rng = np.random.default_rng(1)
    for k in rng.choice(len(theta), size=40, replace=False):
        e = np.zeros_like(theta)
        e[k] = 1e-6
        fp = domega @ mpnn.forward(theta + e, feats, ptr, idx, emulate_bf16=False)[0]
        fm = domega @ mpnn.forward(theta - e, feats, ptr, idx, emulate_bf16=False)[0]
        fd = (fp - fm) / 2e-6
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding_matches_torch():
    import torch
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.normal(size=10000) * 10.0 ** rng.integers(-8, 8, size=10000), [0.0, -0.0, 1.0]])
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy().astype(np.float64)
    assert np.array_equal(mpnn.bf16(x), ref)
