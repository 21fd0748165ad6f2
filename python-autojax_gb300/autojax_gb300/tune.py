"""Autotuner for the tile shapes of the double-float factorisation.

Each step of the trailing update, of L^-1 and of the streamed A^-1 runs in
64 x 64 or 32 x 32 output tiles; the switch points (minimum 64-tile counts,
``aj_set_tile_policy``) decide how the lanes share the GPU and depend on S,
on how many matrices run at once and on the GPU.  The results do not depend
on the choice (the two tile sizes add in the same order), so the tuner only
times: coordinate descent over the three thresholds, each candidate timed
with CUDA events on the work the caller passes (an evaluation or a batch).
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib

NEVER = 1 << 30  # a threshold no step reaches: always 32 x 32 tiles
CANDIDATES = (32, 64, 128, 256, NEVER)


def get_tile_policy() -> tuple[int, int, int]:
    out = (ctypes.c_int * 3)()
    _lib.check(_lib.load().aj_get_tile_policy(out), "aj_get_tile_policy")
    return tuple(int(v) for v in out)


def set_tile_policy(update_min_tiles: int, inverse_min_tiles: int, lauum_min_tiles: int) -> None:
    _lib.check(_lib.load().aj_set_tile_policy(int(update_min_tiles), int(inverse_min_tiles), int(lauum_min_tiles)),
               "aj_set_tile_policy")


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


def tune_tile_policy(run, candidates=CANDIDATES, reps: int = 4, rounds: int = 2) -> dict:
    """Set the fastest tile policy for ``run`` (a callable that enqueues the work to tune on the
    current stream, e.g. ``evaluator.launch``) and return it with the timings seen."""
    best = list(get_tile_policy())
    set_tile_policy(*best)
    best_ms = _time(run, reps)
    tried = {tuple(best): best_ms}
    for _ in range(rounds):
        improved = False
        for axis in range(3):
            for c in candidates:
                cand = list(best)
                cand[axis] = c
                key = tuple(cand)
                if key not in tried:
                    set_tile_policy(*cand)
                    tried[key] = _time(run, reps)
                if tried[key] < best_ms:
                    best, best_ms, improved = cand, tried[key], True
        if not improved:
            break
    set_tile_policy(*best)
    return {"policy": tuple(best), "ms": best_ms, "candidates_timed": len(tried),
            "ms_default": tried.get((128, 128, 96))}


__all__ = ["tune_tile_policy", "get_tile_policy", "set_tile_policy", "NEVER", "CANDIDATES"]
