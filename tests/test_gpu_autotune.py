"""The launch-shape autotuner (GPU): times candidates on the batch, returns
the fastest, caches it per device and batch, and the tuned handle still
meets the solve's true-residual test."""
import json

import pytest

from ffea_gb300 import params as P
from tests.helpers import spec

pytestmark = pytest.mark.gpu


def test_tune_picks_a_candidate_and_caches_it(gpulib, tmp_path):
    from ffea_gb300 import autotune
    from ffea_gb300.world import World
    s = spec(radius_nm=6.0, precision=P.PRECISION_MIXED, epsilon=1e-6)
    space = [{"FFEA_GPU_CG_SMEM_SLOTS": 0, "FFEA_GPU_CG_MAX_CTAS": 152, "FFEA_GPU_COARSE_REFRESH": 10},
             {"FFEA_GPU_CG_SMEM_SLOTS": 64, "FFEA_GPU_CG_MAX_CTAS": 64, "FFEA_GPU_COARSE_REFRESH": 5}]
    cache = str(tmp_path / "tune.json")
    seen = []
    best = autotune.tune([s], preconditioner=1, space=space, cache=cache, steps=3, log=seen.append)
    assert best["config"] in space and best["tried"] == 2 and len(seen) == 2
    table = json.load(open(cache))
    assert list(table.values()) == [best]
    again = autotune.tune([s], preconditioner=1, space=space, cache=cache, steps=3, log=seen.append)
    assert again == best and len(seen) == 2  # served from the cache
    with autotune.applied(best["config"]):
        w = World([s], true_residual=True, preconditioner=1)
    with w:
        w.run(3)
        st = w.blob(0).status()
        assert st["fail_bits"] == 0 and st["true_relres"] < 1e-6
