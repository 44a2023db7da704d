"""Training and use of the learned smoother weights of the two-level preconditioner.

The network and its gradient run on the GPU inside the library
(ffea_gpu_mpnn_*): a 3-layer mesh message-passing network of width 32 that
maps 8 per-node features of the current matrix to a weight omega_p in (0, 2)
of the Jacobi term of M = diag(omega) D^-1 + P A_c^-1 P^T.  Training pairs
(rhs f, solution x) come from the NoMass solves of ordinary time steps, one
pair per step, and the loss of a pair is the energy-norm error of the best
multiple of one application of M, relative to |x|_A:
1 - (f.z)^2 / ((z.Az)(x.f)) with z = M f -- invariant to the scale of M, as
CG is.  The solve itself does not change: it stops on the same residual
test with any omega.  data/mpnn_weights.npz holds the weights trained by
running this module (20,000 pairs over training_meshes()).

This module holds the parameter layout (the same as the library's), the
initialisation, Adam, the training loop and the weight file.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Sequence

import numpy as np

from . import _lib as L

HIDDEN = 32
FEATURES = 8
WEIGHTS_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "mpnn_weights.npz")


def layout():
    """Offsets of (Ws_l, Wn_l, b_l) for l = 0..2, wo, bo in the flat parameter vector."""
    off, out = 0, {}
    for l in range(3):
        din = FEATURES if l == 0 else HIDDEN
        out[f"ws{l}"] = (off, (HIDDEN, din))
        off += HIDDEN * din
        out[f"wn{l}"] = (off, (HIDDEN, din))
        off += HIDDEN * din
        out[f"b{l}"] = (off, (HIDDEN,))
        off += HIDDEN
    out["wo"] = (off, (HIDDEN,))
    off += HIDDEN
    out["bo"] = (off, (1,))
    off += 1
    return out, off


NUM_PARAMS = layout()[1]


def unpack(theta: np.ndarray) -> dict:
    lay, _ = layout()
    return {k: theta[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation; wo = 0 and bo = 0 give omega = 1 everywhere,
    i.e. the untrained network is the plain two-level preconditioner."""
    rng = np.random.default_rng(seed)
    theta = np.zeros(NUM_PARAMS, np.float32)
    lay, _ = layout()
    for l in range(3):
        din = FEATURES if l == 0 else HIDDEN
        for k in (f"ws{l}", f"wn{l}"):
            o, s = lay[k]
            theta[o:o + s[0] * s[1]] = rng.normal(0.0, np.sqrt(1.0 / din), size=s[0] * s[1])
    return theta


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def apply(world, theta: np.ndarray) -> None:
    """Use the network's omega in the solves of a World (LEARNED preconditioner)."""
    t = np.ascontiguousarray(theta, np.float32)
    L.check(L.lib().ffea_gpu_mpnn_apply(world.handle, _fp(t)), "ffea_gpu_mpnn_apply")


def loss_grad(world, theta: np.ndarray, with_grad: bool = True):
    """Loss of the last solve's (rhs, solution) pair and its gradient."""
    t = np.ascontiguousarray(theta, np.float32)
    g = np.zeros(NUM_PARAMS, np.float32) if with_grad else None
    loss = ctypes.c_double()
    L.check(L.lib().ffea_gpu_mpnn_loss_grad(world.handle, _fp(t), ctypes.byref(loss), _fp(g) if with_grad else None),
            "ffea_gpu_mpnn_loss_grad")
    return loss.value, g


def probe(world, blob: int, theta: np.ndarray, domega: np.ndarray | None = None):
    """Features, omega (blob node order) and, given domega, d(sum domega*omega)/dtheta."""
    n = world.num_nodes[blob]
    t = np.ascontiguousarray(theta, np.float32)
    feats = np.zeros((n, FEATURES), np.float32)
    om = np.zeros(n, np.float32)
    grad = np.zeros(NUM_PARAMS, np.float32)
    dw = None if domega is None else np.ascontiguousarray(domega, np.float32)
    L.check(L.lib().ffea_gpu_mpnn_probe(world.handle, int(blob), _fp(t), None if dw is None else _fp(dw), _fp(feats),
                                        _fp(om), _fp(grad) if dw is not None else None), "ffea_gpu_mpnn_probe")
    return feats, om, (grad if dw is not None else None)


@dataclasses.dataclass
class Adam:
    lr: float = 3e-3
    b1: float = 0.9
    b2: float = 0.999
    eps: float = 1e-8

    def __post_init__(self):
        self.m = np.zeros(NUM_PARAMS)
        self.v = np.zeros(NUM_PARAMS)
        self.t = 0

    def step(self, theta: np.ndarray, grad: np.ndarray) -> np.ndarray:
        self.t += 1
        g = grad.astype(np.float64)
        self.m = self.b1 * self.m + (1 - self.b1) * g
        self.v = self.b2 * self.v + (1 - self.b2) * g * g
        mh = self.m / (1 - self.b1 ** self.t)
        vh = self.v / (1 - self.b2 ** self.t)
        return (theta - self.lr * mh / (np.sqrt(vh) + self.eps)).astype(np.float32)


def train(specs: Sequence, pairs: int, theta: np.ndarray | None = None, lr: float = 3e-3, apply_every: int = 50,
          log=None, seed: int = 0):
    """Train on `pairs` (rhs, solution) pairs, one per time step, round-robin
    over one World per spec (LEARNED preconditioner, true-residual check on).
    Returns (theta, losses)."""
    from .world import PRECOND_LEARNED, World
    theta = init_params(seed) if theta is None else np.asarray(theta, np.float32).copy()
    opt = Adam(lr=lr)
    worlds = [World([s], true_residual=True, preconditioner=PRECOND_LEARNED) for s in specs]
    losses = []
    try:
        for w in worlds:
            apply(w, theta)
        for k in range(pairs):
            w = worlds[k % len(worlds)]
            w.run(1)
            loss, g = loss_grad(w, theta)
            if not np.isfinite(loss) or not np.all(np.isfinite(g)):
                raise RuntimeError(f"non-finite loss or gradient at pair {k}")
            theta = opt.step(theta, g)
            losses.append(loss)
            if (k + 1) % apply_every == 0:
                for ww in worlds:
                    apply(ww, theta)
            if log and (k + 1) % max(1, pairs // 20) == 0:
                log(f"pair {k + 1}/{pairs}: loss {np.mean(losses[-max(1, pairs // 20):]):.5f}")
    finally:
        for w in worlds:
            w.close()
    return theta, np.asarray(losses)


def save(theta: np.ndarray, path: str = WEIGHTS_FILE, **meta) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, theta=np.asarray(theta, np.float32), **{k: np.asarray(v) for k, v in meta.items()})


def load(path: str = WEIGHTS_FILE) -> np.ndarray:
    with np.load(path) as z:
        theta = z["theta"].astype(np.float32)
    if theta.size != NUM_PARAMS:
        raise ValueError(f"{path}: {theta.size} parameters, expected {NUM_PARAMS}")
    return theta


def training_meshes(count: int = 8, seed: int = 0):
    """The training family: spheres of radius log-uniform in [5, 25] nm at the
    1.25 nm cell, moduli scaled uniformly by [0.5, 2] around 3.7e8 / 1.1e9
    Pa, NoMass CG to epsilon 1e-6 in mixed precision, one RNG seed each."""
    from . import params as P
    from .mesh import make_blob, sphere_mesh
    rng = np.random.default_rng(seed)
    radii = np.exp(rng.uniform(np.log(5.0), np.log(25.0), size=count))
    out = []
    for i, r in enumerate(radii):
        g = float(rng.uniform(0.5, 2.0))
        prm = P.SimulationParams.from_si(dt=1e-14, kT=P.kT_at(300.0) * P.MESO_ENERGY, epsilon=1e-6,
                                         max_iterations_cg=10000, rng_seed=200 + i, solver=P.SOLVER_NOMASS,
                                         precision=P.PRECISION_MIXED)
        out.append(make_blob(sphere_mesh(float(r), seed=i), prm, shear_mod=3.7e8 * g, bulk_mod=1.1e9 * g))
    return out


if __name__ == "__main__":
    # Regenerates data/mpnn_weights.npz: 20,000 (rhs, solution) pairs, one per
    # time step, round-robin over the training family (needs a GPU).
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=WEIGHTS_FILE)
    a = ap.parse_args()
    theta, losses = train(training_meshes(), pairs=a.pairs, lr=a.lr, log=print)
    save(theta, a.out, pairs=a.pairs, losses=losses)
    print(f"saved {a.out}: loss {losses[:100].mean():.5f} -> {losses[-100:].mean():.5f}")
