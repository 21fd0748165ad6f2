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
    cache.write_text(json.dumps({"gpu|S=1500": [64, 96, 32]}))
    saved = tune.get_tile_policy()
    try:
        def never_called():
            raise AssertionError("a cached key must not be timed")

        out = tune.tune_tile_policy(never_called, key="gpu|S=1500")
        assert out["cached"] and out["policy"] == (64, 96, 32)
        assert tune.get_tile_policy() == (64, 96, 32)
    finally:
        tune.set_tile_policy(*saved)


def test_policy_rejects_non_positive_thresholds():
    from autojax_gb300 import _lib, tune

    with pytest.raises(Exception):
        tune.set_tile_policy(0, 1, 1)
    assert _lib.load().aj_set_tile_policy(1, 1, -3) == _lib.AJ_ERR_ARG
