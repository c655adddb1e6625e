"""The profiling mode's stage times (pf_profile_stages): four CUDA-event
intervals that partition each profiled step."""
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_profile_stages_partition_the_step(precision):
    s = G.settings_spheres_3d(iter_max=20, precision=precision, outer_max=2, inner_sweeps=10)
    shape = (48, 40, 32)
    with Case(s, shape, G.spheres_3d(*shape, count=3, seed=1)) as c:
        c.initial_conditions()
        c.step(1)
        c.profile_begin()
        c.step(3)
        prof = c.profile_end()
        st = c.profile_stages()
    assert set(st) == {"predictor", "rhs", "sor", "projection_boundary"}
    assert all(v > 0 for v in st.values()), st
    assert st["sor"] == pytest.approx(prof["sor_ms"], rel=1e-9)
    # event times are floats in ms with about half a microsecond of resolution
    assert abs(sum(st.values()) - prof["step_ms"]) <= 1e-3 * prof["step_ms"] + 0.01, (st, prof)
    assert st["sor"] > st["rhs"]
