"""pf_step_host (one step from host fields to host fields) against the three
calls it stands for, pf_set_state + pf_step(1) + pf_get_state.  In the 3D
periodic plain-FP64 form the input copies run in slabs of planes beside the
divergence and the predictor of the planes already in place; each cell's
arithmetic is the step's own, so every field must agree bit for bit, for
ragged slabs, with and without graphs and error tracking, over several
steps that feed their result back as the next input."""
import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


def _same(a, b):
    return all(np.array_equal(a[k], b[k]) for k in a)


def _start_state(c, warm):
    c.initial_conditions()
    c.step(warm)
    return c.get_state()


def _three_calls(c, state):
    c.set_state(state["u"], state["v"], state["p"], state.get("w"))
    c.step(1)
    return c.get_state()


SHAPES = [
    (24, 20, 3),    # fewest planes: three slabs of two planes
    (40, 24, 37),   # ragged last slab
    (33, 18, 64),   # odd m, more planes than slabs
]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("use_graph", [True, False])
def test_step_host_matches_three_calls(shape, use_graph):
    s = G.settings_spheres_3d(iter_max=30)
    vals = G.spheres_3d(*shape, count=5, seed=7)
    with Case(s, shape, vals, use_graph=use_graph) as a, Case(s, shape, vals, use_graph=use_graph) as b:
        state = _start_state(a, 3)
        _start_state(b, 3)
        for _ in range(3):  # the result of one step is the input of the next
            ref = _three_calls(a, state)
            got = b.step_host(state)
            assert _same(got, ref)
            assert b.norms() == a.norms()  # max|div u| and the tracked SOR error
            state = ref


def test_step_host_in_place():
    shape = (28, 20, 26)
    s = G.settings_spheres_3d(iter_max=15)
    vals = G.spheres_3d(*shape, count=3, seed=11)
    with Case(s, shape, vals) as a, Case(s, shape, vals) as b:
        state = _start_state(a, 2)
        _start_state(b, 2)
        ref = _three_calls(a, state)
        got = b.step_host(state, state)  # the output overwrites the input arrays
        assert got is state and _same(state, ref)


def test_step_host_untracked_and_resident_run():
    shape = (36, 28, 22)
    s = G.settings_spheres_3d(iter_max=25, track_sor_error=0)
    vals = G.spheres_3d(*shape, count=4, seed=8)
    with Case(s, shape, vals) as a, Case(s, shape, vals) as b:
        state = _start_state(a, 2)
        _start_state(b, 2)
        a.step(4)  # the fields stay on the device
        ref = a.get_state()
        for _ in range(4):
            state = b.step_host(state)
        assert _same(state, ref)


@pytest.mark.parametrize("form", ["2d", "mixed", "pitched"])
def test_step_host_other_forms_make_the_three_calls(form):
    if form == "2d":
        shape, s = (48, 24), G.settings_cylinder_2d(iter_max=20)
        vals = G.cylinder_2d(*shape)
    else:
        shape = (30, 20, 16)
        s = G.settings_spheres_3d(iter_max=20, **({"precision": "mixed"} if form == "mixed" else {}))
        vals = G.spheres_3d(*shape, count=3, seed=9)
    with Case(s, shape, vals) as a, Case(s, shape, vals) as b:
        state = _start_state(a, 2)
        _start_state(b, 2)
        if form == "pitched":  # leading dimensions wider than m+2: host rows are not contiguous
            wide = {k: np.zeros(v.shape[:-1] + (v.shape[-1] + 5,)) for k, v in state.items()}
            for k in state:
                wide[k][..., : state[k].shape[-1]] = state[k]
            ref = {k: np.zeros_like(v) for k, v in wide.items()}
            a.set_state(wide["u"], wide["v"], wide["p"], wide.get("w"))
            a.step(1)
            a.get_state(ref)
            got = b.step_host(wide, {k: np.zeros_like(v) for k, v in wide.items()})
        else:
            ref = _three_calls(a, state)
            got = b.step_host(state)
        assert _same(got, ref)


def test_step_host_staging_is_counted():
    shape = (32, 24, 20)
    s = G.settings_spheres_3d(iter_max=10)
    vals = G.spheres_3d(*shape, count=3, seed=10)
    with Case(s, shape, vals) as c:
        state = _start_state(c, 1)
        before = c.memory_bytes()
        c.step_host(state)
        field = (shape[0] + 2) * (shape[1] + 2) * (shape[2] + 2) * 8
        assert c.memory_bytes() == before + 3 * field


@pytest.mark.parametrize("use_graph", [True, False])
def test_step_host_between_resident_steps(use_graph):
    """Host steps and resident steps interleaved on one case (the two step
    graphs of each buffer parity, the buffer swap) equal the three-call
    sequence interleaved the same way."""
    shape = (30, 22, 19)
    s = G.settings_spheres_3d(iter_max=12)
    vals = G.spheres_3d(*shape, count=3, seed=12)
    with Case(s, shape, vals, use_graph=use_graph) as a, Case(s, shape, vals, use_graph=use_graph) as b:
        state = _start_state(a, 1)
        _start_state(b, 1)
        for resident in (1, 2, 3):
            ref = _three_calls(a, state)
            got = b.step_host(state)
            assert _same(got, ref)
            a.step(resident)
            b.step(resident)
            state = a.get_state()
            assert _same(b.get_state(), state)
