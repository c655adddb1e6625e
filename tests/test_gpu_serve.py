"""The serving form: requests admitted by HBM budget into one resident batch,
advanced together, each result identical (bit for bit) to running the case
alone."""
import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300.batch import case_bytes
from pixelflow_gb300.serve import Server, summarize
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


def _small_requests():
    reqs = G.serving_requests(count=8, rate=400.0, seed=3, sizes_2d=(64, 96, 128), sizes_3d=(24, 32),
                              steps_range=(6, 20))
    for r in reqs:  # a short inner schedule keeps the test quick
        r.settings = r.settings.replace(iter_max=20, outer_max=4, inner_sweeps=5)
    return reqs


def test_gpu_shapes_match_host_generator():
    s = G.settings_cylinder_2d()
    shapes = [(0.5, 0.5, 0.05, 0.05, 0.0), (1.2, 0.4, 0.08, 0.03, 0.7)]
    host = G.obstacles_2d(128, 64, 2.0, 1.0, shapes)
    with Case.from_shapes(s, (128, 64), shapes) as c:
        dev = c.porosity()
    ref = Case(s, (128, 64), host)
    np.testing.assert_allclose(dev, ref.porosity(), rtol=0, atol=1e-12)
    ref.close()


@pytest.mark.parametrize("policy", ["rr", "srpt", "srpt_fill"])
def test_served_results_equal_single_runs(policy):
    reqs = _small_requests()
    # budget for ~2 of the requests at a time forces queueing and slot reuse;
    # srpt_fill's 2 ms rounds split every request over several rounds
    budget = int(2.2 * max(case_bytes(r.settings, r.shape) for r in reqs))
    with Server(hbm_budget_bytes=budget, chunk=4, policy=policy, round_cells=20_000, round_ms=2.0) as srv:
        res = srv.run(reqs, realtime=True)
        assert srv.peak_bytes <= budget
    assert [r.rid for r in res] == [r.rid for r in reqs]
    for r, q in zip(res, reqs):
        assert r.done_s >= r.admitted_s >= 0
        with Case.from_shapes(q.settings.replace(precision="mixed"), q.shape, q.shapes) as c:
            c.initial_conditions()
            c.step(q.steps)
            alone = c.get_state()
            assert np.array_equal(np.array(c.norms()), np.array([r.max_div, r.sor_error]))
        assert np.isfinite(r.max_div) and np.isfinite(r.sor_error), q.rid
        for k in alone:
            assert np.isfinite(r.state[k]).all(), (q.rid, k)
            assert np.array_equal(alone[k], r.state[k]), (q.rid, k)
    summ = summarize(res, max(r.done_s for r in res))
    assert summ["requests"] == len(reqs) and summ["p99_latency_s"] >= summ["p50_latency_s"]


def test_tuned_schedules_apply_to_admissions():
    """tune_schedules picks an outer x inner schedule per grid size, 2D and
    3D; every served result then equals the single run under the tuned
    schedule, bit for bit."""
    reqs = _small_requests()
    cands = ((1, 20), (2, 10), (4, 5))
    with Server(chunk=4, policy="srpt_fill", round_cells=20_000, round_ms=2.0) as srv:
        tuned = srv.tune_schedules(reqs, bound=1e-2, steps=3, schedules=cands, use_cache=False)
        sizes = {(q.dim, tuple(q.shape)) for q in reqs}
        assert {d for d, _ in sizes} == {2, 3} and set(srv.schedules) == sizes
        assert all(v in cands for v in srv.schedules.values())
        assert len(tuned) == len(sizes)
        res = srv.run(reqs, realtime=False)
        chosen = dict(srv.schedules)
    for r, q in zip(res, reqs):
        o, i = chosen[(q.dim, tuple(q.shape))]
        s = q.settings.replace(outer_max=o, inner_sweeps=i)
        with Case.from_shapes(s, q.shape, q.shapes) as c:
            c.initial_conditions()
            c.step(q.steps)
            alone = c.get_state()
        for k in alone:
            assert np.array_equal(alone[k], r.state[k]), (q.rid, k)
