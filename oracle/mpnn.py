"""CPU restatement of the learned smoother-weight network (numpy, FP64 math).

TEST INFRASTRUCTURE ONLY: the GPU tests check the library's network forward
and backward passes (ffea_gpu_mpnn_probe) against this module.  The network
has no counterpart in the reference: it weights the Jacobi term of the
two-level preconditioner, which FFEA does not have.  The definition it
restates:

  h0 = features (8 per node)
  h(l+1)_p = bf16(ReLU(Ws_l h(l)_p + Wn_l mean_{q ~ p} h(l)_q + b_l)),  l = 0..2
  omega_p = 2 sigmoid(wo . h3_p + bo)

with q ~ p the corner nodes sharing an element edge with p, and bf16() the
round-to-nearest-even storage of the activations (emulated here, so that
the comparison isolates the arithmetic order).
"""
from __future__ import annotations

import numpy as np

HIDDEN = 32
FEATURES = 8


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), back to float."""
    x = np.ascontiguousarray(a, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(theta):
    off, out = 0, {}
    theta = np.asarray(theta, dtype=np.float64)
    for l in range(3):
        din = FEATURES if l == 0 else HIDDEN
        for k in ("ws", "wn"):
            out[f"{k}{l}"] = theta[off:off + HIDDEN * din].reshape(HIDDEN, din)
            off += HIDDEN * din
        out[f"b{l}"] = theta[off:off + HIDDEN]
        off += HIDDEN
    out["wo"] = theta[off:off + HIDDEN]
    off += HIDDEN
    out["bo"] = theta[off]
    return out


def edge_neighbours(topology: np.ndarray, num_nodes: int):
    """Adjacency (CSR over node ids) of corner nodes sharing an element edge."""
    t = np.asarray(topology)[:, :4].astype(np.int64)
    pairs = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(4) if a != b])
    key = np.unique(pairs[:, 0] * num_nodes + pairs[:, 1])
    src, dst = key // num_nodes, key % num_nodes
    ptr = np.zeros(num_nodes + 1, np.int64)
    np.add.at(ptr, src + 1, 1)
    return np.cumsum(ptr), dst


def _mean(h, ptr, idx):
    n = len(ptr) - 1
    deg = np.diff(ptr)
    s = np.zeros((n, h.shape[1]))
    np.add.at(s, np.repeat(np.arange(n), deg), h[idx])
    return s / np.maximum(deg, 1)[:, None], deg


def forward(theta, feats, ptr, idx, emulate_bf16=True):
    P = unpack(theta)
    hs, ms, pre = [np.asarray(feats, np.float64)], [], []
    for l in range(3):
        m, _ = _mean(hs[-1], ptr, idx)
        a = hs[-1] @ P[f"ws{l}"].T + m @ P[f"wn{l}"].T + P[f"b{l}"]
        h = np.maximum(a, 0.0)
        hs.append(bf16(h) if emulate_bf16 else h)
        ms.append(m)
        pre.append(a)
    s = hs[-1] @ P["wo"] + P["bo"]
    omega = 2.0 / (1.0 + np.exp(-s))
    return omega, {"h": hs, "m": ms, "a": pre}


def backward(theta, cache, omega, domega, ptr, idx):
    """Gradient of sum(domega * omega) with respect to theta (flat, FP64)."""
    P = unpack(theta)
    hs, ms = cache["h"], cache["m"]
    grads = {}
    ds = domega * omega * (1.0 - 0.5 * omega)
    grads["wo"] = ds @ hs[3]
    grads["bo"] = np.array([ds.sum()])
    dh = np.outer(ds, P["wo"])
    deg = np.maximum(np.diff(ptr), 1)
    n = len(ptr) - 1
    rows = np.repeat(np.arange(n), np.diff(ptr))
    for l in (2, 1, 0):
        da = dh * (hs[l + 1] > 0)
        grads[f"ws{l}"] = da.T @ hs[l]
        grads[f"wn{l}"] = da.T @ ms[l]
        grads[f"b{l}"] = da.sum(axis=0)
        t = (da @ P[f"wn{l}"]) / deg[:, None]
        dprev = da @ P[f"ws{l}"]
        np.add.at(dprev, rows, t[idx])  # q ~ p is symmetric: dh[q] += sum_{p ~ q} t[p]
        dh = dprev
    out = []
    for l in range(3):
        out += [grads[f"ws{l}"].ravel(), grads[f"wn{l}"].ravel(), grads[f"b{l}"]]
    out += [grads["wo"], grads["bo"]]
    return np.concatenate(out)
