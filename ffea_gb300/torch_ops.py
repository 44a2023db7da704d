"""The learned preconditioner's training signal as a PyTorch custom operator.

`mpnn_loss(world, theta)` is the network loss of the handle's last solve
(the A-norm error of the best multiple of one preconditioner application,
`ffea_gpu_mpnn_loss_grad`) as a differentiable function of the parameter
vector `theta` (float32, `learned.NUM_PARAMS`): the forward and backward
passes are the library's own GPU kernels, reached through the C ABI, so a
torch optimizer can train the network:

    theta = torch.nn.Parameter(torch.from_numpy(learned.init_params()))
    opt = torch.optim.Adam([theta], lr=3e-3)
    w.run(1)                                  # a solve gives an (rhs, solution) pair
    loss = torch_ops.mpnn_loss(w, theta)
    opt.zero_grad(); loss.backward(); opt.step()

Registered as `ffea::mpnn_loss_grad` (torch.library), for the training loop
only: the blob update itself is called through the C ABI (`world.World`).
"""
from __future__ import annotations

import numpy as np
import torch

from . import learned


@torch.library.custom_op("ffea::mpnn_loss_grad", mutates_args=())
def mpnn_loss_grad(handle: int, theta: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """(loss, dloss/dtheta) of the handle's last solve; theta on the CPU."""

    class _W:  # the handle is all learned.loss_grad reads
        pass
    w = _W()
    w.handle = handle
    loss, grad = learned.loss_grad(w, theta.detach().cpu().numpy().astype(np.float32))
    return torch.tensor(loss, dtype=torch.float64), torch.from_numpy(grad)


@mpnn_loss_grad.register_fake
def _(handle, theta):
    return theta.new_empty((), dtype=torch.float64), torch.empty_like(theta)


def _setup_context(ctx, inputs, output):
    ctx.save_for_backward(output[1])


def _backward(ctx, g_loss, g_grad):
    (grad,) = ctx.saved_tensors
    return None, (g_loss.to(grad.dtype) * grad)


torch.library.register_autograd("ffea::mpnn_loss_grad", _backward, setup_context=_setup_context)


def mpnn_loss(world, theta: torch.Tensor) -> torch.Tensor:
    """The network loss of `world`'s last solve, differentiable in `theta`."""
    if theta.numel() != learned.NUM_PARAMS:
        raise ValueError(f"theta must hold {learned.NUM_PARAMS} parameters")
    loss, _ = mpnn_loss_grad(int(world.handle.value if hasattr(world.handle, "value") else world.handle), theta)
    return loss
