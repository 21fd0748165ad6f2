"""Autotuner for the tile shapes of the double-float factorisation.

Each step of the trailing update and of L^-1 runs in 64 x 64 or 32 x 32
output tiles; the switch points (minimum 64-tile counts,
``aj_set_tile_policy``) decide how the lanes share the GPU and depend on S,
on how many matrices run at once and on the GPU.  The results do not depend
on the choice (the two tile sizes add in the same order), so the tuner only
times: coordinate descent over the two thresholds, each candidate timed
with CUDA events on the work the caller passes (an evaluation or a batch).
"""

from __future__ import annotations

import ctypes
import json
import os
from pathlib import Path

import torch

from . import _lib

NEVER = 1 << 30  # a threshold no step reaches: always 32 x 32 tiles
CANDIDATES = (32, 64, 128, 256, NEVER)


def get_tile_policy() -> tuple[int, int]:
    out = (ctypes.c_int * 2)()
    _lib.check(_lib.load().aj_get_tile_policy(out), "aj_get_tile_policy")
    return tuple(int(v) for v in out)


def set_tile_policy(update_min_tiles: int, inverse_min_tiles: int) -> None:
    _lib.check(_lib.load().aj_set_tile_policy(int(update_min_tiles), int(inverse_min_tiles)), "aj_set_tile_policy")


def _time(run, reps: int) -> float:
    st = torch.cuda.current_stream()
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        run()
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def cache_path() -> Path:
    """The tuner's cache file: $AUTOJAX_GB300_CACHE, else $XDG_CACHE_HOME (or ~/.cache)/autojax_gb300."""
    env = os.environ.get("AUTOJAX_GB300_CACHE")
    if env:
        return Path(env)
    base = Path(os.environ.get("XDG_CACHE_HOME", Path.home() / ".cache"))
    return base / "autojax_gb300" / "tile_policy.json"


def cache_key(label: str) -> str:
    """A cache key for ``label`` (e.g. the problem sizes) on this GPU model."""
    return f"{torch.cuda.get_device_name()}|{label}"


def tune_tile_policy(run, candidates=CANDIDATES, reps: int = 4, rounds: int = 2, key: str | None = None,
                     prepare=None) -> dict:
    """Set the fastest tile policy for ``run`` (a callable that enqueues the work to tune on the
    current stream, e.g. ``evaluator.launch``) and return it with the timings seen.

    ``prepare``, when given, runs after each policy is set and before it is timed: pass the
    evaluator's ``capture`` with ``run=evaluator.step`` to tune graph replays (a captured graph
    keeps the policy it was captured with).

    With ``key`` (see ``cache_key``) a policy found before for the same key is read from the cache
    file and set without timing, and a newly found one is written there.
    """
    if key is not None:
        try:
            cached = json.loads(cache_path().read_text()).get(key)
        except (OSError, ValueError):
            cached = None
        if cached:
            set_tile_policy(*cached)
            return {"policy": tuple(cached), "ms": None, "candidates_timed": 0, "ms_default": None, "cached": True}
    def timed(policy):
        set_tile_policy(*policy)
        if prepare is not None:
            prepare()
        return _time(run, reps)

    best = list(get_tile_policy())
    best_ms = timed(best)
    tried = {tuple(best): best_ms}
    for _ in range(rounds):
        improved = False
        for axis in range(2):
            for c in candidates:
                cand = list(best)
                cand[axis] = c
                ck = tuple(cand)
                if ck not in tried:
                    tried[ck] = timed(cand)
                if tried[ck] < best_ms:
                    best, best_ms, improved = cand, tried[ck], True
        if not improved:
            break
    set_tile_policy(*best)
    if prepare is not None:
        prepare()
    if key is not None:
        path = cache_path()
        try:
            table = json.loads(path.read_text())
        except (OSError, ValueError):
            table = {}
        table[key] = list(best)
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(table, indent=1))
        except OSError:
            pass
    return {"policy": tuple(best), "ms": best_ms, "candidates_timed": len(tried),
            "ms_default": tried.get((128, 128)), "cached": False}


__all__ = ["tune_tile_policy", "get_tile_policy", "set_tile_policy", "cache_path", "cache_key", "NEVER", "CANDIDATES"]
