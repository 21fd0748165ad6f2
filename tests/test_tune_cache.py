"""The tile-policy autotuner's cache file: a cached policy is set without timing (CPU: the library
calls that set the policy need no device)."""

from __future__ import annotations

import json

import pytest


def test_cached_policy_is_used_without_timing(tmp_path, monkeypatch):
    from autojax_gb300 import tune

    cache = tmp_path / "tile_policy.json"
    monkeypatch.setenv("AUTOJAX_GB300_CACHE", str(cache))
    assert tune.cache_path() == cache
    cache.write_text(json.dumps({"gpu|S=1500": [64, 96]}))
    saved = tune.get_tile_policy()
    try:
        def never_called():
            raise AssertionError("a cached key must not be timed")

        out = tune.tune_tile_policy(never_called, key="gpu|S=1500")
        assert out["cached"] and out["policy"] == (64, 96)
        assert tune.get_tile_policy() == (64, 96)
    finally:
        tune.set_tile_policy(*saved)


def test_policy_rejects_non_positive_thresholds():
    from autojax_gb300 import _lib, tune

    with pytest.raises(Exception):
        tune.set_tile_policy(0, 1)
    assert _lib.load().aj_set_tile_policy(1, -3) == _lib.AJ_ERR_ARG


def test_descent_finds_the_fastest_policy_and_caches_it(tmp_path, monkeypatch):
    """Coordinate descent over the two thresholds on a synthetic cost with one minimum: the
    tuner sets it, times each candidate once, calls ``prepare`` after every policy it sets and
    writes the result under its key."""
    import math

    from autojax_gb300 import tune

    cache = tmp_path / "tile_policy.json"
    monkeypatch.setenv("AUTOJAX_GB300_CACHE", str(cache))
    target = (64, tune.NEVER)

    def cost(policy):
        return sum(abs(math.log2(p) - math.log2(t)) for p, t in zip(policy, target))

    timed = []
    monkeypatch.setattr(tune, "_time", lambda run, reps: timed.append(tune.get_tile_policy()) or
                        cost(tune.get_tile_policy()))
    prepared = []
    saved = tune.get_tile_policy()
    try:
        out = tune.tune_tile_policy(lambda: None, key="gpu|S=777", prepare=lambda: prepared.append(1))
        assert out["policy"] == target and not out["cached"]
        assert tune.get_tile_policy() == target
        assert len(set(timed)) == len(timed) == out["candidates_timed"]
        assert len(prepared) == len(timed) + 1  # each timed policy, then the chosen one
        assert json.loads(cache.read_text())["gpu|S=777"] == list(target)
    finally:
        tune.set_tile_policy(*saved)
