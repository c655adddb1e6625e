"""Autotuner for launch shapes, tile shapes and sweep schedules.

* `tune_batch`: the persistent batch kernel's launch shape -- the
  thread-block cluster (CTAs per case) and the CTA size -- timed on the
  batch's own cases for a few steps (device time of the persistent launch).
* `tune_fused`: the tile of the precision form's fused FP32 sweep (3D) --
  rows per tile and the cap on (tile, plane) pairs per CTA -- and the split
  sweep, timed on the case itself.
* `tune_schedule`: the precision form's outer x inner schedule (FP64
  defect-correction passes x FP32 sweeps per pass, product = iter_max):
  every candidate runs the case for a few steps beside the plain FP64 step,
  and the fastest schedule whose pressure error against FP64 (relative L2)
  stays within `bound` wins.  The time grows with the passes; the error,
  since the FP32 sweep keeps its operator's row sum (pf_cells.cuh), hardly
  depends on the schedule, so when no candidate meets the bound the fastest
  of those within twice the smallest error is taken.
* `tune_batch_schedule`: the same for a batch, on a sample of its cases.
  The serving loop (`serve.Server.tune_schedules`) runs `tune_schedule` once
  per 3D grid size of its requests.

Results are cached per machine and workload signature in a JSON file so
later runs start tuned.
"""
from __future__ import annotations

import json
import os
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

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


FUSED_ROWS: Tuple[int, ...] = (0, 4, 6, 8, 10, 12)
FUSED_PLANES: Tuple[int, ...] = (0, 32)
SCHEDULES: Tuple[Tuple[int, int], ...] = ((1, 100), (2, 50), (4, 25), (5, 20), (10, 10), (20, 5))


def _open_case(settings, shape, vals=None, shapes=None):
    """A case from porosity values, or from analytic shapes (generated on the GPU)."""
    from .solver import Case
    if shapes is not None:
        return Case.from_shapes(settings, shape, shapes)
    return Case(settings, shape, vals)


def _case_ms(settings, shape, vals, steps: int, shapes=None) -> float:
    """Device ms per step of a precision-form case (after one untimed step)."""
    with _open_case(settings, shape, vals, shapes) as c:
        c.initial_conditions()
        c.step(1)
        c.synchronize()
        c.profile_begin()
        c.step(steps)
        return c.profile_end()["step_ms"] / steps


def tune_fused(settings, shape, vals, steps: int = 2, rows=FUSED_ROWS, planes=FUSED_PLANES,
               use_cache: bool = True) -> Tuple[dict, List[dict]]:
    """Times the split FP32 sweep and each fused tile (rows per tile, cap on
    the (tile, plane) pairs per CTA; 0 = the library's choice) on the case;
    returns the fastest as Settings fields ({"sweep_form", "fused_rows",
    "fused_planes"}) and the trials.  The forms give the same bits, so only
    time decides."""
    base = settings.replace(precision="mixed")
    sig = f"fused:{tuple(shape)}:{base.outer_max}x{base.inner_sweeps}"
    cache = _load() if use_cache else {}
    if use_cache and sig in cache:
        return cache[sig]["best"], cache[sig]["trials"]
    trials = []
    cands = [{"sweep_form": "split", "fused_rows": 0, "fused_planes": 0}]
    cands += [{"sweep_form": "fused", "fused_rows": r, "fused_planes": p} for r in rows for p in planes]
    for cand in cands:
        try:
            ms = _case_ms(base.replace(**cand), shape, vals, steps)
            trials.append(dict(cand, ms=ms))
        except Exception as exc:  # a tile that does not fit this grid
            trials.append(dict(cand, error=str(exc)[:120]))
    ok = [t for t in trials if "ms" in t]
    if not ok:
        raise RuntimeError("tune_fused: no sweep form could run")
    b = min(ok, key=lambda t: t["ms"])
    best = {k: b[k] for k in ("sweep_form", "fused_rows", "fused_planes")}
    if use_cache:
        cache[sig] = {"best": best, "trials": trials}
        _save(cache)
    return best, trials


def _rel_l2(a, b) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _pick(trials, error) -> Tuple[int, int]:
    """The fastest trial within the bound, else the fastest of those within
    twice the smallest error (schedules of one accuracy class)."""
    ok = [t for t in trials if t["within_bound"]]
    if not ok:
        floor = min(error(t) for t in trials)
        ok = [t for t in trials if error(t) <= 2.0 * floor]
    pick = min(ok, key=lambda t: t["ms"])
    return pick["outer"], pick["inner"]


def tune_schedule(settings, shape, vals, bound: float = 1e-4, steps: int = 5, schedules=SCHEDULES,
                  use_cache: bool = True, shapes=None) -> Tuple[Tuple[int, int], List[dict]]:
    """The fastest outer x inner schedule of the precision form whose
    pressure (and velocity) error against the plain FP64 step after `steps`
    steps from the initial state stays within `bound` (relative L2).  When
    no candidate meets the bound, the fastest of those within twice the
    smallest error is returned.  The case comes from porosity values `vals`
    or, with `shapes`, from analytic shapes generated on the GPU."""
    it = int(settings.iter_max)
    cands = [(o, i) for (o, i) in schedules if o * i == it]
    sig = f"schedule:{tuple(shape)}:{it}:{bound:g}:{steps}:{cands}"
    cache = _load() if use_cache else {}
    if use_cache and sig in cache:
        return tuple(cache[sig]["best"]), cache[sig]["trials"]
    with _open_case(settings.replace(precision="fp64"), shape, vals, shapes) as c:
        c.initial_conditions()
        c.step(steps)
        ref = c.get_state()
    trials = []
    for (o, i) in cands:
        s = settings.replace(precision="mixed", outer_max=o, inner_sweeps=i)
        with _open_case(s, shape, vals, shapes) as c:
            c.initial_conditions()
            c.step(steps)
            got = c.get_state()
        err = {f: _rel_l2(got[f], ref[f]) for f in ref}
        ms = _case_ms(s, shape, vals, 2, shapes)
        trials.append({"outer": o, "inner": i, "ms": ms, "rel_l2": err, "within_bound": max(err.values()) <= bound})
    best = _pick(trials, lambda t: max(t["rel_l2"].values()))
    if use_cache:
        cache[sig] = {"best": list(best), "trials": trials}
        _save(cache)
    return best, trials


def tune_batch_schedule(cases, bound: float = 1e-4, steps: int = 20, sample: int = 16, seed: int = 0,
                        schedules=SCHEDULES, cluster: int = 4, threads: int = 1024,
                        use_cache: bool = True) -> Tuple[Tuple[int, int], List[dict]]:
    """The schedule for a batch of 2D precision-form cases (`cases`: objects
    with .settings, .m, .n and .porosity()): on a sample of them, each
    candidate's error against the plain FP64 single-case step after `steps`
    steps, and its device time in the persistent kernel (a batch of the
    sample); the fastest within `bound` wins (else the fastest within twice
    the smallest error)."""
    from .batch import Batch
    from .solver import Case
    rng = np.random.default_rng(seed)
    pick_ix = sorted(rng.choice(len(cases), size=min(sample, len(cases)), replace=False).tolist())
    sub = [cases[k] for k in pick_ix]
    it = int(sub[0].settings.iter_max)
    cands = [(o, i) for (o, i) in schedules if o * i == it]
    sig = "batch_schedule:" + signature((c.m, c.n) for c in sub) + f":{it}:{bound:g}:{steps}"
    cache = _load() if use_cache else {}
    if use_cache and sig in cache:
        return tuple(cache[sig]["best"]), cache[sig]["trials"]
    refs = []
    for c in sub:
        with Case(c.settings.replace(precision="fp64"), (c.m, c.n), c.porosity()) as sc:
            sc.initial_conditions()
            sc.step(steps)
            refs.append(sc.get_state())
    trials = []
    for (o, i) in cands:
        with Batch(cluster=cluster, threads=threads, max_cases=len(sub)) as b:
            slots = [b.add(c.settings.replace(outer_max=o, inner_sweeps=i), (c.m, c.n), c.porosity()) for c in sub]
            b.step_slots(slots, [steps] * len(slots))
            ms = b.last_ms()
            errs = [max(_rel_l2(b.get_state(sl)[f], r[f]) for f in r) for sl, r in zip(slots, refs)]
        cell_steps = sum(c.m * c.n for c in sub) * steps
        worst = float(max(errs))
        trials.append({"outer": o, "inner": i, "ms": ms, "mcell_steps_per_s": cell_steps / (ms / 1e3) / 1e6,
                       "max_rel_l2": worst, "within_bound": worst <= bound})
    best = _pick(trials, lambda t: t["max_rel_l2"])
    if use_cache:
        cache[sig] = {"best": list(best), "trials": trials}
        _save(cache)
    return best, trials
