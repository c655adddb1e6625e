"""The batched form: a persistent kernel advancing many cases of uneven size.

Every stage of a batched case uses the same per-cell code as the single-case
precision form, so a case must give bit-identical fields alone, in a batch,
in a different mix, order or launch shape."""
import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300._lib import PfError
from pixelflow_gb300.batch import Batch, case_bytes
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


def _cases():
    out = []
    s2 = G.settings_cylinder_2d(iter_max=20, inner_sweeps=5, outer_max=4)
    out.append((s2, (64, 40), G.cylinder_2d(64, 40, radius=0.15, cx=0.6, cy=0.5)))
    out.append((s2, (48, 32), G.cylinder_2d(48, 32, radius=0.2, cx=0.7, cy=0.4)))
    out.append((s2, (33, 17), G.cylinder_2d(33, 17, radius=0.2, cx=0.7, cy=0.5)))  # odd sizes: halo path
    s3 = G.settings_spheres_3d(iter_max=12, inner_sweeps=3, outer_max=4)
    out.append((s3, (20, 16, 12), G.spheres_3d(20, 16, 12, count=3, seed=4)))
    out.append((s3, (17, 15, 13), G.spheres_3d(17, 15, 13, count=2, seed=5)))
    return out


def _single(s, shape, vals, steps):
    with Case(s.replace(precision="mixed"), shape, vals) as c:
        c.initial_conditions()
        c.step(steps)
        return c.get_state(), c.norms()


def _same(a, b):
    """Bit-identical and finite (a NaN field would "equal" a NaN field)."""
    return all(np.isfinite(a[k]).all() and np.array_equal(a[k], b[k]) for k in a)


@pytest.mark.parametrize("cluster,threads,global_passes", [(4, 512, False), (1, 256, False), (2, 1024, True),
                                                          (8, 512, True), (8, 256, False), (16, 256, False)])
def test_batch_matches_single_cases_bitwise(cluster, threads, global_passes):
    """2D cases keep their correction in shared memory unless global_passes;
    both paths, every launch shape, must equal the single-case runs."""
    cases = _cases()
    steps = 4
    ref = [_single(s, shape, vals, steps) for (s, shape, vals) in cases]
    with Batch(cluster=cluster, threads=threads, global_passes=global_passes) as b:
        slots = [b.add(s, shape, vals) for (s, shape, vals) in cases]
        try:
            b.step(steps)
        except PfError as exc:
            if cluster == 16 and "scheduled" in str(exc):
                pytest.skip("clusters of 16 CTAs cannot be scheduled on this device")
            raise
        for k, sl in enumerate(slots):
            got = b.get_state(sl)
            assert _same(got, ref[k][0]), (k, cases[k][1])
            assert np.array_equal(np.array(b.norms(sl)), np.array(ref[k][1]))


def test_large_cases_on_own_streams_match_single_cases():
    """With large_cells small, all but the smallest 2D case run full-GPU step
    graphs on their own streams beside the persistent kernel: the fields are
    still those of the single-case runs, and the launch count covers both."""
    cases = _cases()
    steps = 3
    ref = [_single(s, shape, vals, steps) for (s, shape, vals) in cases]
    with Batch(cluster=2, threads=512, large_cells=1000) as b:
        slots = [b.add(s, shape, vals) for (s, shape, vals) in cases]
        n0 = b.kernel_launches()
        b.step(steps)
        assert b.kernel_launches() - n0 > 2
        for k, sl in enumerate(slots):
            assert _same(b.get_state(sl), ref[k][0]), (k, cases[k][1])
            assert np.array_equal(np.array(b.norms(sl)), np.array(ref[k][1]))


def test_batch_uneven_steps_and_mix_order():
    """Per-case step counts in one launch, cases added in another order and
    advanced in two launches: each still equals its single-case run."""
    cases = _cases()
    want_steps = [3, 5, 0, 2, 4]
    ref = [_single(s, shape, vals, n) for (s, shape, vals), n in zip(cases, want_steps)]
    with Batch(cluster=2, threads=512) as b:
        order = [4, 2, 0, 3, 1]
        slots = {k: b.add(*cases[k]) for k in order}
        first = [min(2, n) for n in want_steps]
        b.step_slots([slots[k] for k in range(5)], first)
        b.step_slots([slots[k] for k in range(5)], [n - f for n, f in zip(want_steps, first)])
        for k in range(5):
            assert _same(b.get_state(slots[k]), ref[k][0]), k


def test_batch_admission_by_budget_and_slot_reuse():
    s, shape, vals = _cases()[0]
    need = case_bytes(s, shape)
    with Batch(hbm_budget_bytes=int(need * 1.5), max_cases=4) as b:
        a = b.add(s, shape, vals)
        with pytest.raises(PfError) as ei:
            b.add(s, shape, vals)
        assert ei.value.code == -3  # PF_E_NOMEM: admitted only once memory frees up
        used, budget = b.memory()
        assert 0 < used <= budget
        b.remove(a)
        c = b.add(s, shape, vals)
        b.step(2)
        got = b.get_state(c)
    ref = _single(s, shape, vals, 2)[0]
    assert _same(got, ref)


def test_batch_launch_is_persistent_one_per_dimension():
    cases = _cases()
    with Batch() as b:
        for c in cases:
            b.add(*c)
        n0 = b.kernel_launches()
        b.step(3)
        assert b.kernel_launches() - n0 == 2  # one 2D launch + one 3D launch for 3 steps of 5 cases


def test_persistent_launch_graph_replays_match_plain_launches():
    """The persistent part of a call runs as a CUDA graph captured per
    composition: repeated calls of the same composition replay it (the
    descriptors, which change between calls, are read from the pinned
    staging when the graph runs), a new composition or launch shape captures
    again, and the fields equal those of plain launches bit for bit."""
    cases = _cases()
    plan = [([0, 1, 2, 3, 4], [2, 2, 2, 2, 2]), ([0, 1, 2, 3, 4], [1, 3, 2, 1, 2]), ([0, 1, 2, 3, 4], [2] * 5),
            ([0, 2, 4], [1, 1, 1]), ([0, 1, 2, 3, 4], [1] * 5)]
    outs = []
    for graph in (True, False):
        with Batch(cluster=2, threads=512, use_graph=graph) as b:
            slots = [b.add(*c) for c in cases]
            for k, (which, steps) in enumerate(plan):
                if k == 3:
                    b.configure(4, 256)
                b.step_slots([slots[i] for i in which], steps)
            outs.append(([b.get_state(sl) for sl in slots], [b.norms(sl) for sl in slots]))
            captured, replays = b.graph_stats()
            if graph:
                # plan[1] and plan[2] have plan[0]'s composition; plan[3] differs; plan[4] has a new shape
                assert captured == 3 and replays == 2, (captured, replays)
            else:
                assert captured == 0 and replays == 0
    for k in range(len(cases)):
        assert _same(outs[0][0][k], outs[1][0][k]), k
        assert outs[0][1][k] == outs[1][1][k]


def test_admission_bytes_equal_the_allocation():
    """The admission estimate (pf_case_bytes through case_bytes) is the
    allocation a batch makes for the case, for small cases (stepped by the
    persistent kernel, split sweep) and large ones (own step graphs)."""
    for (s, shape, vals) in _cases():
        for large in (300000, 100):
            with Batch(max_cases=2, large_cells=large) as b:
                b.add(s, shape, vals)
                assert b.memory()[0] == case_bytes(s, shape, large_cells=large), (shape, large)
