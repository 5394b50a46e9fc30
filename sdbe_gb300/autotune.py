"""Wave-size autotuner for the multi-stream pass.

The tunable shape of this stage is the FFT wave: how many 143-snapshot
batches of every stream one stage-A / stage-BC launch pair covers.  Larger
waves amortise the per-launch twiddle-table loads and the persistent grid's
last round; smaller ones keep the stage-A scratch closer to L2 and start
shipping payloads earlier.  ``tune`` times each candidate on the caller's own
workload (CUDA events, after a warm-up pass) and caches the winner per device
and workload key in a JSON file (``$SDBE_AUTOTUNE_CACHE`` or
``~/.cache/sdbe_gb300/autotune.json``).
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
