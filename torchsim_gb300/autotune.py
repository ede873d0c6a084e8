"""A small measuring autotuner for launch shapes.

Candidates are timed with CUDA events on the current stream (warm-up, then the
best of a few runs) and the winner is cached in memory and in a JSON file
(``$TORCHSIM_GB300_CACHE`` or ``~/.cache/torchsim_gb300/tuning.json``) under a
key that names the workload (kernel family, state count, program length,
voxel count bucket, device name).
"""

from __future__ import annotations

import json
import os
import threading
from collections.abc import Callable, Iterable
from pathlib import Path
from typing import Any

import torch

_lock = threading.Lock()
_memory: dict[str, Any] = {}


def cache_path() -> Path:
    root = os.environ.get("TORCHSIM_GB300_CACHE")
    if root:
        return Path(root)
    return Path.home() / ".cache" / "torchsim_gb300" / "tuning.json"


def _load() -> dict[str, Any]:
    path = cache_path()
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, value: Any) -> None:
    path = cache_path()
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        data = _load()
        data[key] = value
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs a re-tune


def workload_key(family: str, **fields: Any) -> str:
    device = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    parts = [family, device] + [f"{k}={fields[k]}" for k in sorted(fields)]
    return "|".join(parts)


def time_ms(fn: Callable[[], Any], warmup: int = 2, repeats: int = 3) -> float:
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(repeats):
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        fn()
        end.record()
        end.synchronize()
        best = min(best, start.elapsed_time(end))
    return best


def tune(key: str, candidates: Iterable[Any], run: Callable[[Any], Any], *,
         use_cache: bool = True, warmup: int = 2, repeats: int = 3) -> tuple[Any, dict]:
    """The fastest candidate for ``key`` and the timings measured (ms)."""
    with _lock:
        if use_cache:
            if key in _memory:
                return _memory[key], {}
            stored = _load().get(key)
            if stored is not None:
                value = tuple(stored) if isinstance(stored, list) else stored
                _memory[key] = value
                return value, {}
    timings: dict[Any, float] = {}
    for cand in candidates:
        try:
            timings[cand] = time_ms(lambda c=cand: run(c), warmup, repeats)
        except (RuntimeError, ValueError):
            continue  # a shape the kernel table does not serve
    if not timings:
        raise RuntimeError(f"no candidate ran for {key}")
    best = min(timings, key=timings.get)
    with _lock:
        _memory[key] = best
    _store(key, list(best) if isinstance(best, tuple) else best)
    return best, {str(k): v for k, v in timings.items()}


def sweep_shapes(states: int, family_shapes: list[tuple[int, int]],
                 warps: Iterable[int] = (2, 4, 8)) -> list[tuple[int, int, int]]:
    """(lanes, orders, warps) candidates whose padded orders cover ``states``."""
    return [(lanes, orders, w) for lanes, orders in family_shapes if lanes * orders >= states
            for w in warps]
