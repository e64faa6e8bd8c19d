"""Autotuner for the batched form's launch shape.

The batched kernel processes one tile (threads x particles-per-thread) of one realisation per CTA.
Small tiles waste fewer padded slots on small realisations; large tiles amortise the per-CTA work and
give the fp64 pipe more independent chains.  `choose_tile` times a bounded sample of the batch (a
deterministic subset of the realisations, a few protocol cycles) for every candidate shape and keeps
the fastest; the choice is cached in a JSON file keyed by the GPU name and a summary of the size
distribution, so later batches of the same kind reuse it without timing.
"""

from __future__ import annotations

import json
import os
import pathlib
import time

import numpy as np

CANDIDATES = [(64, 1), (128, 1), (256, 1), (128, 2), (256, 2)]
CACHE = pathlib.Path(os.environ.get("FQSB_AUTOTUNE_CACHE", pathlib.Path.home() / ".cache" / "fqsb_autotune.json"))


def _key(sizes, gpu: str) -> str:
    s = np.asarray(sizes)
    q = np.quantile(s, [0.1, 0.5, 0.9]).round().astype(int).tolist()
    return f"{gpu}|n={len(s)}|q={q}"


def _gpu_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001
        pass
    return "unknown"


def _load() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def _store(d: dict):
    try:
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        tmp = CACHE.with_suffix(".tmp")
        tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
        os.replace(tmp, CACHE)
    except OSError:
        pass


def choose_tile(sizes, make, sample: int = 256, cycles: int = 2, eps: float = 1e-5, use_cache: bool = True):
    """Return (threads, ppt) for a batch with these realisation sizes.

    make(sizes_subset, threads, ppt) must build a batch (Line1d_System_Cuspy_Laplace) over the given
    subset; each candidate runs `cycles` quasistatic cycles on the same subset and is timed."""
    key = _key(sizes, _gpu_name())
    cache = _load() if use_cache else {}
    if key in cache:
        t, p = cache[key]["tile"]
        return int(t), int(p)
    sizes = np.asarray(sizes)
    idx = np.linspace(0, len(sizes) - 1, min(sample, len(sizes))).round().astype(int)
    subset = sizes[idx]
    timings = {}
    for threads, ppt in CANDIDATES:
        b = make(subset, threads, ppt)
        t0 = time.perf_counter()
        b.quasistatic(cycles, eps)
        timings[(threads, ppt)] = time.perf_counter() - t0
        del b
    best = min(timings, key=timings.get)
    cache[key] = {"tile": list(best), "timings_s": {f"{t}x{p}": v for (t, p), v in timings.items()}}
    if use_cache:
        _store(cache)
    return best
