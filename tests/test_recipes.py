"""The synthetic batch and serving recipes (CPU): the stability choices are
the documented ones, and the generator is deterministic in its seed."""
from pixelflow_gb300 import geometry as G


def test_batch_recipe_defaults():
    cases = G.batch_cases_2d(40, seed=0)
    for c in cases:
        s = c.settings
        h = 1.0 / (c.n - 1)
        assert s.threshold == 0.1
        assert 1.0 * h / s.xnue <= 2.0 + 1e-12          # cell Reynolds number capped at 2
        dt = s.time / s.istep_max
        assert abs(dt - G.cfl_dt(h, s.xnue, 1.0, 2)) <= 1e-15
        assert s.precision == "mixed" and s.istep_max == 500
    again = G.batch_cases_2d(40, seed=0)
    assert [(c.m, c.n, c.shapes) for c in cases] == [(c.m, c.n, c.shapes) for c in again]


def test_batch_recipe_knobs():
    lit = G.batch_cases_2d(10, seed=0, threshold=1e-6, cell_re=None, dt_rule="cfl")
    for c in lit:
        h = 1.0 / (c.n - 1)
        assert c.settings.threshold == 1e-6
        assert abs(c.settings.time / c.settings.istep_max - 0.2 * h) <= 1e-15


def test_serving_recipe_threshold():
    reqs = G.serving_requests(count=20, seed=1)
    assert all(r.settings.threshold == 0.1 for r in reqs)
    assert {r.dim for r in reqs} == {2, 3}
