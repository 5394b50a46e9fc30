"""Autotuner for the batch and launch shape of the multi-stream pass.

The shape of a pass over several streams has three parts:

* ``wave``: how many 143-snapshot batches of every stream one stage-A /
  stage-BC launch pair covers.  Larger waves amortise the per-launch table
  loads and the persistent grid's last round; smaller ones keep the stage-A
  scratch closer to L2 and start shipping payloads earlier.
* ``per_launch``: how many stream handles share one fused launch
  (``sdbe_process_multi``); fewer per launch gives shorter launches that the
  next call can overlap, more gives fuller persistent grids.
* ``stages``: for ``SDBE_PRECISION_TC16_FAST``, whether a wave's three
  transform stages run as one persistent launch on a device work queue
  (``SDBE_STAGES_FUSED``: no grid tail and launch gap between the stages)
  or as a launch per stage (``SDBE_STAGES_SPLIT``).
* ``precision``: the FFT form, when the caller admits more than one
  (``SDBE_PRECISION_FP32`` and ``SDBE_PRECISION_TC16_FAST`` both meet the
  99.9% 2-bit agreement bar; which is faster depends on the stream mix).

``tune_shape`` times candidate shapes on the caller's own workload (its
``measure`` callback, CUDA events after a warm-up pass) by coordinate descent
from the default shape, and caches the winner and the timings per device and
workload key in a JSON file (``$SDBE_AUTOTUNE_CACHE`` or
``~/.cache/sdbe_gb300/autotune.json``).  ``tune`` is the wave-only form.
"""
from __future__ import annotations

import json
import os
from typing import Callable, Iterable

DEFAULT_WAVES = (16, 32, 48, 64)


def _cache_path() -> str:
    return os.environ.get("SDBE_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "sdbe_gb300", "autotune.json"))


def _load() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def device_key() -> str:
    import torch

    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"


def tune(workload_key: str, measure: Callable[[int], float], candidates: Iterable[int] = DEFAULT_WAVES,
         use_cache: bool = True) -> tuple[int, dict]:
    """Return (best wave, {wave: ms}) for the workload; ``measure(wave)`` gives
    milliseconds per pass.  A cached result for this device and key is
    returned without measuring."""
    key = f"{device_key()}|{workload_key}"
    cache = _load() if use_cache else {}
    if key in cache:
        ent = cache[key]
        return int(ent["best"]), {int(k): v for k, v in ent["ms"].items()}
    table = {int(w): float(measure(int(w))) for w in candidates}
    best = min(table, key=table.get)
    if use_cache:
        cache[key] = {"best": best, "ms": {str(k): v for k, v in table.items()}}
        _store(cache)
    return best, table


def _shape_key(shape: dict) -> str:
    return ",".join(f"{k}={shape[k]}" for k in sorted(shape))


def tune_shape(workload_key: str, measure: Callable[[dict], float], space: dict, default: dict,
               use_cache: bool = True, rounds: int = 2) -> tuple[dict, dict]:
    """Return (best shape, {shape key: ms}) for the workload.

    ``space`` maps each dimension to its candidate values, ``default`` is the
    starting shape (one value per dimension) and ``measure(shape)`` gives
    milliseconds per pass.  Coordinate descent: each round sweeps the
    dimensions in turn, keeping the others at the best shape so far; shapes
    already timed are not timed again.  A cached result for this device,
    workload and search space is returned without measuring."""
    space = {k: list(v) for k, v in space.items()}
    key = f"{device_key()}|{workload_key}|" + ";".join(f"{k}:{'/'.join(map(str, space[k]))}" for k in sorted(space))
    cache = _load() if use_cache else {}
    if key in cache:
        ent = cache[key]
        return dict(ent["best"]), dict(ent["ms"])
    table: dict = {}

    def timed(shape):
        k = _shape_key(shape)
        if k not in table:
            table[k] = float(measure(dict(shape)))
        return table[k]

    best = dict(default)
    best_ms = timed(best)
    for _ in range(rounds):
        moved = False
        for dim, values in space.items():
            for v in values:
                cand = dict(best, **{dim: v})
                ms = timed(cand)
                if ms < best_ms:
                    best, best_ms, moved = cand, ms, True
        if not moved:
            break
    if use_cache:
        cache[key] = {"best": best, "ms": table}
        _store(cache)
    return best, table
