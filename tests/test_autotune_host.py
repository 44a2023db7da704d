"""The launch-shape autotuner's host logic (ffea_gb300.autotune), on the CPU:
knob scoping, the search space, and the choice and caching of the fastest
configuration (the timing itself is faked here; tests/test_gpu_autotune.py
times real handles)."""
import json
import os

import pytest

from ffea_gb300 import autotune as A


def test_applied_scopes_and_restores_the_knobs(monkeypatch):
    monkeypatch.setenv("FFEA_GPU_CG_MAX_CTAS", "77")
    monkeypatch.delenv("FFEA_GPU_CG_SMEM_SLOTS", raising=False)
    monkeypatch.setenv("FFEA_GPU_COARSE_REFRESH", "3")
    with A.applied({"FFEA_GPU_CG_SMEM_SLOTS": 2}):
        assert os.environ["FFEA_GPU_CG_SMEM_SLOTS"] == "2"
        # knobs the configuration leaves out are unset inside, not inherited
        assert "FFEA_GPU_CG_MAX_CTAS" not in os.environ
        assert "FFEA_GPU_COARSE_REFRESH" not in os.environ
    assert os.environ["FFEA_GPU_CG_MAX_CTAS"] == "77"
    assert os.environ["FFEA_GPU_COARSE_REFRESH"] == "3"
    assert "FFEA_GPU_CG_SMEM_SLOTS" not in os.environ
    with pytest.raises(KeyError, match="unknown tuning knob"):
        with A.applied({"FFEA_GPU_NOT_A_KNOB": 1}):
            pass
    assert os.environ["FFEA_GPU_CG_MAX_CTAS"] == "77"


def test_candidates_cover_the_search_space():
    c = A.candidates(152)
    assert len(c) == 30
    assert len({tuple(sorted(x.items())) for x in c}) == 30
    assert {x["FFEA_GPU_CG_MAX_CTAS"] for x in c} == {152, 114}
    assert all(set(x) == set(A.KNOBS) for x in c)


def test_tune_picks_the_fastest_and_caches_it(monkeypatch, tmp_path):
    times = {5: 3e-3, 10: 2e-3, 25: 4e-3}
    calls = []

    def fake_time(specs, cfg, preconditioner, steps=6, weights=None):
        calls.append(cfg)
        return times[cfg["FFEA_GPU_COARSE_REFRESH"]]
    monkeypatch.setattr(A, "signature", lambda specs, pc: "key0")
    monkeypatch.setattr(A, "time_config", fake_time)
    space = [{"FFEA_GPU_COARSE_REFRESH": r} for r in (5, 10, 25)]
    cache = str(tmp_path / "sub" / "autotune.json")
    entry = A.tune([], 2, space=space, cache=cache)
    assert entry == {"config": {"FFEA_GPU_COARSE_REFRESH": 10}, "ms_per_step": pytest.approx(2.0), "tried": 3}
    assert len(calls) == 3
    assert json.load(open(cache))["key0"]["config"] == {"FFEA_GPU_COARSE_REFRESH": 10}
    # a second run of the same batch reads the cache and times nothing
    assert A.tune([], 2, space=space, cache=cache)["config"] == {"FFEA_GPU_COARSE_REFRESH": 10}
    assert len(calls) == 3
