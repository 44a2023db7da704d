"""The learned smoother weights on the GPU: the network's forward and backward
passes against the CPU restatement (oracle/mpnn.py), the training loss
gradient against central differences, and what training buys over the
untrained (omega = 1) two-level preconditioner on a held-out mesh.

Tolerances: omega to 5e-3 absolute and the parameter gradient to 2e-2
relative (2-norm) against the oracle -- both sides store BF16 activations,
and a value that sits on a BF16 rounding boundary can round either way
under the different FP32 summation orders; the loss gradient with respect
to the output bias to 2 % against central differences."""
import numpy as np
import pytest

from ffea_gb300 import params as P
from tests.helpers import spec

pytestmark = pytest.mark.gpu

LEARNED, TWO_LEVEL = 2, 1


def _world(specs, **kw):
    from ffea_gb300.world import World
    return World(specs, **kw)


def _theta(seed):
    from ffea_gb300 import learned
    th = learned.init_params(seed)
    lay, _ = learned.layout()
    rng = np.random.default_rng(seed + 100)
    o, s = lay["wo"]
    th[o:o + s[0]] = rng.normal(0.0, 0.3, size=s[0])
    o, _ = lay["bo"]
    th[o] = 0.1
    return th


def test_network_matches_cpu_oracle(gpulib):
    from ffea_gb300 import learned
    from oracle import mpnn
    s = spec(radius_nm=6.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    theta = _theta(3)
    with _world([s], preconditioner=LEARNED) as w:
        w.run(1)
        n = s.mesh.num_nodes
        rng = np.random.default_rng(4)
        domega = np.zeros(n, np.float32)
        domega[:s.mesh.num_linear] = rng.normal(size=s.mesh.num_linear)
        feats, om, grad = learned.probe(w, 0, theta, domega)
    ptr, idx = mpnn.edge_neighbours(s.mesh.topology, n)
    nl = s.mesh.num_linear
    assert np.all(np.isfinite(feats)) and np.all(feats[:nl, 7] == 1.0)
    om_ref, cache = mpnn.forward(theta, feats.astype(np.float64), ptr, idx)
    assert np.max(np.abs(om[:nl] - om_ref[:nl])) < 5e-3
    g_ref = mpnn.backward(theta, cache, om_ref, domega.astype(np.float64), ptr, idx)
    err = np.linalg.norm(grad - g_ref) / np.linalg.norm(g_ref)
    assert err < 2e-2, err


def test_loss_gradient_matches_central_differences(gpulib):
    """With every weight zero the activations are exactly zero and omega =
    2 sigmoid(bo) is uniform, so the loss is a smooth function of bo alone
    (no BF16 rounding anywhere): dloss/dbo from the backward pass must match
    central differences.  The network part of the gradient is checked
    against the CPU restatement above."""
    from ffea_gb300 import learned
    s = spec(radius_nm=6.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    lay, _ = learned.layout()
    bo = lay["bo"][0]
    with _world([s], true_residual=True, preconditioner=LEARNED) as w:
        w.run(2)
        for b0 in (-0.5, 0.0, 0.7):
            theta = np.zeros(learned.NUM_PARAMS, np.float32)
            theta[bo] = b0
            loss, g = learned.loss_grad(w, theta)
            assert np.isfinite(loss) and 0.0 <= loss <= 1.0  # 1 - cos^2 of the A-angle of M f and x
            h = 1e-2
            tp, tm = theta.copy(), theta.copy()
            tp[bo] += h
            tm[bo] -= h
            fd = (learned.loss_grad(w, tp, with_grad=False)[0] - learned.loss_grad(w, tm, with_grad=False)[0]) / (2 * h)
            assert abs(fd - g[bo]) <= 2e-2 * abs(fd) + 1e-6, (b0, fd, g[bo])


def test_training_gains_over_the_untrained_preconditioner(gpulib):
    """Trains on small meshes, evaluates on a held-out larger one: the loss of
    the trained network is lower and the solves need no more iterations than
    the two-level preconditioner with omega = 1 (the untrained network)."""
    from ffea_gb300 import learned
    train_specs = [spec(radius_nm=r, seed=i, rng_seed=70 + i, precision=P.PRECISION_MIXED, epsilon=1e-6)
                   for i, r in enumerate((6.0, 7.5, 9.0))]
    theta0 = learned.init_params(0)
    theta, losses = learned.train(train_specs, pairs=240, theta=theta0, lr=3e-3)
    assert np.all(np.isfinite(losses))
    held = spec(radius_nm=12.0, seed=9, rng_seed=99, precision=P.PRECISION_MIXED, epsilon=1e-6)
    res = {}
    for name, th in (("untrained", theta0), ("trained", theta)):
        with _world([held], true_residual=True, preconditioner=LEARNED) as w:
            learned.apply(w, th)
            iters, loss = 0, 0.0
            for _ in range(6):
                w.run(1)
                st = w.blob(0).status()
                assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6, st
                iters += st["cg_iters"]
                loss += learned.loss_grad(w, th, with_grad=False)[0]
            res[name] = (iters, loss)
    assert res["trained"][1] < res["untrained"][1], res
    assert res["trained"][0] <= res["untrained"][0] + 2, res


def test_torch_custom_op_trains_the_network(gpulib):
    """ffea::mpnn_loss_grad (torch.library) gives the loss and gradient of
    the library's own kernels, and torch's Adam on it lowers the loss of the
    same (rhs, solution) pair."""
    import torch

    from ffea_gb300 import learned, torch_ops
    from ffea_gb300.world import World
    s = spec(radius_nm=8.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    with World([s], true_residual=True, preconditioner=2) as w:
        theta0 = learned.init_params(seed=3)
        learned.apply(w, theta0)
        w.run(1)
        ref_loss, ref_grad = learned.loss_grad(w, theta0)
        theta = torch.nn.Parameter(torch.from_numpy(theta0.copy()))
        loss = torch_ops.mpnn_loss(w, theta)
        assert abs(loss.item() - ref_loss) <= 1e-12 * max(1.0, abs(ref_loss))
        loss.backward()
        assert np.array_equal(theta.grad.numpy(), ref_grad)
        opt = torch.optim.Adam([theta], lr=3e-3)
        first = loss.item()
        for _ in range(20):
            opt.zero_grad()
            loss = torch_ops.mpnn_loss(w, theta)
            loss.backward()
            opt.step()
        assert torch_ops.mpnn_loss(w, theta).item() < first


@pytest.mark.parametrize("memory_state", ["0", "1"])
def test_committed_weights_take_effect_in_a_batch(gpulib, monkeypatch, memory_state):
    """The network's smoother weights reach the solve of every blob of a
    batch, in the register-resident and the memory-resident solve: after
    two steps each blob's velocities differ from those of the same batch
    with every weight 1 (the two-level preconditioner), and two learned
    worlds agree bit for bit.  (The weights' upload once raced with the
    zero fill of their buffer, which left every weight at 1 in some
    processes.)"""
    from ffea_gb300 import learned
    specs = [spec(radius_nm=r, seed=i, rng_seed=40 + i, precision=P.PRECISION_MIXED, epsilon=1e-6)
             for i, r in enumerate((6.0, 8.0, 5.0))]
    theta = learned.load()
    vels = {}
    for name, pc in (("two-level", TWO_LEVEL), ("learned", LEARNED), ("learned-again", LEARNED)):
        monkeypatch.setenv("FFEA_GPU_CG_MEMORY_STATE", memory_state)
        w = _world(specs, true_residual=True, preconditioner=pc)
        monkeypatch.delenv("FFEA_GPU_CG_MEMORY_STATE", raising=False)
        with w:
            assert w.preconditioner() == pc
            if pc == LEARNED:
                learned.apply(w, theta)
            w.run(2)
            vels[name] = [w.blob(i).get_nodes()[1].copy() for i in range(len(specs))]
            for i in range(len(specs)):
                assert w.blob(i).status()["fail_bits"] == 0
    for i in range(len(specs)):
        assert np.array_equal(vels["learned"][i], vels["learned-again"][i]), i
        assert not np.array_equal(vels["learned"][i], vels["two-level"][i]), i
