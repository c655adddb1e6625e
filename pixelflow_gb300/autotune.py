"""Autotuner for the batched form's launch shape.

The persistent batch kernel's tile shape is the thread-block cluster (CTAs
per case) and the CTA size.  `tune_batch` times every candidate shape on the
batch's own cases for a few steps (device time of the persistent launch) and
configures the batch with the fastest; results are cached per machine and
workload signature in a JSON file so later runs start tuned.
"""
from __future__ import annotations

import json
import os
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

CANDIDATES: Tuple[Tuple[int, int], ...] = ((1, 256), (1, 512), (2, 256), (2, 512), (4, 256), (4, 512),
                                           (8, 256), (8, 512), (2, 1024), (4, 1024), (16, 256), (16, 512))


def cache_path() -> str:
    base = os.environ.get("PF_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache",
                                                                "pixelflow_gb300")
    return os.path.join(base, "autotune.json")


def _load() -> Dict[str, dict]:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d: Dict[str, dict]) -> None:
    try:
        os.makedirs(os.path.dirname(cache_path()), exist_ok=True)
        with open(cache_path(), "w") as f:
            json.dump(d, f, indent=1)
    except OSError:
        pass


def signature(shapes: Iterable[Sequence[int]]) -> str:
    """Workload signature: dimension mix and size histogram (powers of two of cells)."""
    hist: Dict[str, int] = {}
    for sh in shapes:
        cells = 1
        for x in sh:
            cells *= int(x)
        key = f"{len(sh)}d:{cells.bit_length()}"
        hist[key] = hist.get(key, 0) + 1
    return ",".join(f"{k}x{hist[k]}" for k in sorted(hist))


def tune_batch(batch, slots: List[int], steps: int = 2, candidates=CANDIDATES, use_cache: bool = True,
               repeats: int = 1) -> Tuple[Tuple[int, int], List[dict]]:
    """Time each (cluster, threads) on `steps` steps of the given slots and keep
    the fastest.  The trial steps advance the cases (use them as warm-up)."""
    sig = signature(batch.shapes[s] for s in slots)
    cache = _load() if use_cache else {}
    if use_cache and sig in cache:
        best = tuple(cache[sig]["best"])
        batch.configure(*best)
        return best, cache[sig].get("trials", [])
    trials = []
    for (cl, th) in candidates:
        try:
            batch.configure(cl, th)
            ms = []
            for _ in range(repeats):
                batch.step_slots(slots, [steps] * len(slots))
                ms.append(batch.last_ms())
            trials.append({"cluster": cl, "threads": th, "ms": min(ms)})
        except Exception as exc:  # a shape the device cannot schedule
            trials.append({"cluster": cl, "threads": th, "error": str(exc)})
    ok = [t for t in trials if "ms" in t]
    if not ok:
        raise RuntimeError("autotune: no launch shape could run")
    b = min(ok, key=lambda t: t["ms"])
    best = (b["cluster"], b["threads"])
    batch.configure(*best)
    if use_cache:
        cache[sig] = {"best": list(best), "trials": trials}
        _save(cache)
    return best, trials
