"""Autotuner of the CG solve's launch shape for a given batch on the current GPU.

The library reads these knobs when a handle is created:

  FFEA_GPU_CG_SMEM_SLOTS   matrix slots per row whose values the register-
                           resident solve keeps in shared memory (the rest
                           stream from L2); column indices are kept for all
  FFEA_GPU_CG_MAX_CTAS     cap on the persistent grid, hence on the number of
                           CG segments (one per CTA): fewer, longer segments
                           trade SM count for fewer coarse dofs and partials
  FFEA_GPU_COARSE_REFRESH  steps between refreshes of the coarse space

`tune` times each candidate on the batch itself (a fresh handle per
candidate, warm-up steps, then timed steps with a device synchronisation on
both sides) and returns the fastest; results are cached per device and batch
signature in a JSON file, so a later run of the same batch reuses them.
`applied` sets a tuning for the handles created inside a `with` block.
"""
from __future__ import annotations

import contextlib
import hashlib
import json
import os
import time
from typing import Iterable, Sequence

KNOBS = ("FFEA_GPU_CG_SMEM_SLOTS", "FFEA_GPU_CG_MAX_CTAS", "FFEA_GPU_COARSE_REFRESH")
DEFAULT_CACHE = os.path.join(os.environ.get("XDG_CACHE_HOME", os.path.expanduser("~/.cache")), "ffea_gb300",
                             "autotune.json")


@contextlib.contextmanager
def applied(config: dict | None):
    """Set the knobs of `config` (name -> int) for handles created inside."""
    saved = {k: os.environ.get(k) for k in KNOBS}
    try:
        for k in KNOBS:
            os.environ.pop(k, None)
        for k, v in (config or {}).items():
            if k not in KNOBS:
                raise KeyError(f"unknown tuning knob {k}")
            os.environ[k] = str(int(v))
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def signature(specs: Sequence, preconditioner: int) -> str:
    """Device + batch key: GPU name and SM count, blob sizes, precision,
    solver and preconditioner."""
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    desc = {
        "gpu": p.name, "sms": p.multi_processor_count,
        "blobs": [[int(s.mesh.num_linear), int(s.mesh.num_elements), int(s.params.precision), int(s.params.solver)]
                  for s in specs],
        "precond": int(preconditioner),
    }
    return hashlib.sha1(json.dumps(desc, sort_keys=True).encode()).hexdigest()[:16]


def candidates(sms: int) -> list[dict]:
    """The search space: on-chip matrix slots x grid size x coarse refresh."""
    out = []
    for slots in (0, 1, 2, 3, 64):
        for ctas in (sms, (3 * sms) // 4):
            for refresh in (5, 10, 25):
                out.append({"FFEA_GPU_CG_SMEM_SLOTS": slots, "FFEA_GPU_CG_MAX_CTAS": ctas,
                            "FFEA_GPU_COARSE_REFRESH": refresh})
    return out


def time_config(specs: Sequence, config: dict, preconditioner: int, steps: int = 6, warmup: int = 3,
                weights=None) -> float:
    """Seconds per step of `specs` under `config` (fresh handle)."""
    from .world import World
    with applied(config):
        w = World(list(specs), true_residual=True, preconditioner=preconditioner)
    try:
        if weights is not None and w.preconditioner() == 2:
            from . import learned
            learned.apply(w, weights)
        w.run(warmup)
        w.synchronize()
        t0 = time.perf_counter()
        w.run(steps)
        w.synchronize()
        return (time.perf_counter() - t0) / steps
    finally:
        w.close()


def tune(specs: Sequence, preconditioner: int = 0, space: Iterable[dict] | None = None, cache: str = DEFAULT_CACHE,
         steps: int = 6, weights=None, log=None) -> dict:
    """The fastest configuration of `space` for this batch (cached)."""
    import torch
    key = signature(specs, preconditioner)
    table = {}
    if cache and os.path.exists(cache):
        with open(cache) as fh:
            table = json.load(fh)
        if key in table:
            return table[key]
    if space is None:
        space = candidates(torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count)
    best, results = None, []
    for cfg in space:
        t = time_config(specs, cfg, preconditioner, steps=steps, weights=weights)
        results.append((t, cfg))
        if log:
            log(f"{cfg}: {1e3 * t:.3f} ms/step")
        if best is None or t < best[0]:
            best = (t, cfg)
    entry = {"config": best[1], "ms_per_step": 1e3 * best[0], "tried": len(results)}
    if cache:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        table[key] = entry
        with open(cache, "w") as fh:
            json.dump(table, fh, indent=1, sort_keys=True)
    return entry
