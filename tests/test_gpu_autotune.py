"""The autotuner beyond launch shapes: the fused sweep's tile and the
precision form's outer x inner schedule (held to an error bound against the
plain FP64 step), for single cases and for a batch."""
import numpy as np
import pytest

from pixelflow_gb300 import autotune as A
from pixelflow_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def test_tune_fused_times_split_and_tiles():
    s = G.settings_spheres_3d(iter_max=20, outer_max=4, inner_sweeps=5)
    shape = (48, 40, 32)
    vals = G.spheres_3d(*shape, count=4, seed=1)
    best, trials = A.tune_fused(s, shape, vals, steps=1, rows=(0, 2, 4), planes=(0, 8), use_cache=False)
    assert len(trials) == 1 + 3 * 2
    assert trials[0]["sweep_form"] == "split" and "ms" in trials[0]
    timed = [t for t in trials if "ms" in t]
    assert best == {k: min(timed, key=lambda t: t["ms"])[k] for k in ("sweep_form", "fused_rows", "fused_planes")}


def test_tune_schedule_respects_the_bound():
    s = G.settings_spheres_3d(iter_max=20)
    shape = (32, 30, 28)
    vals = G.spheres_3d(*shape, count=3, seed=2)
    scheds = ((1, 20), (4, 5), (20, 1))
    loose, trials = A.tune_schedule(s, shape, vals, bound=1.0, steps=3, schedules=scheds, use_cache=False)
    assert all(t["within_bound"] for t in trials)
    fastest = min(trials, key=lambda t: t["ms"])
    assert loose == (fastest["outer"], fastest["inner"])
    tight, trials = A.tune_schedule(s, shape, vals, bound=0.0, steps=3, schedules=scheds, use_cache=False)
    # nothing meets a zero bound: the fastest of the schedules within twice
    # the smallest error (one accuracy class) is returned
    worst = {(t["outer"], t["inner"]): max(t["rel_l2"].values()) for t in trials}
    ms = {(t["outer"], t["inner"]): t["ms"] for t in trials}
    floor = min(worst.values())
    assert tight == min((k for k in worst if worst[k] <= 2 * floor), key=ms.get)
    print("schedule errors", worst)
    # the FP32 sweep keeps its operator's row sum, so every schedule stays close to FP64
    assert max(worst.values()) < 1e-5


def test_tune_batch_schedule_on_a_sample():
    cases = G.batch_cases_2d(6, seed=5, sizes=(64, 96), iter_max=20)
    best, trials = A.tune_batch_schedule(cases, bound=1.0, steps=4, sample=4, schedules=((1, 20), (4, 5)),
                                         cluster=2, threads=512, use_cache=False)
    assert len(trials) == 2 and all(np.isfinite(t["max_rel_l2"]) for t in trials)
    fastest = min(trials, key=lambda t: t["ms"])
    assert best == (fastest["outer"], fastest["inner"])
