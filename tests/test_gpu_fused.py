"""The fused FP32 sweep of the precision form (both colours of one sweep in
one launch, 3D with even n and l) against the two-launch sweep: the same
operands reach the same per-cell arithmetic, so every field must agree bit
for bit after whole steps, for any tile shape, with and without graphs,
error tracking or the early stop of the defect correction."""
import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


def _run(s, shape, vals, steps, use_graph=True):
    with Case(s, shape, vals, use_graph=use_graph) as c:
        c.initial_conditions()
        c.step(steps)
        st = c.get_state()
        norms = c.norms()
        launches = c.kernel_launches()
        mem = c.memory_bytes()
    return st, norms, launches, mem


def _same(a, b):
    return all(np.array_equal(a[k], b[k]) for k in a)


SHAPES = [
    (32, 32, 32),   # tiles divide the grid
    (40, 36, 30),   # ragged last tile in y and z
    (31, 20, 18),   # odd m: the outlet lane falls on the last chunk
    (66, 4, 4),     # four rows and planes: every halo is a periodic image
    (24, 10, 48),   # more planes than rows
]


@pytest.mark.parametrize("shape", SHAPES)
def test_fused_sweep_matches_split_bit_for_bit(shape):
    s = G.settings_spheres_3d(precision="mixed", outer_max=2, inner_sweeps=5)
    vals = G.spheres_3d(*shape, count=6, seed=3)
    split, nsplit, lsplit, msplit = _run(s.replace(sweep_form="split"), shape, vals, 4)
    fused, nfused, lfused, mfused = _run(s.replace(sweep_form="fused"), shape, vals, 4)
    assert _same(fused, split)
    assert nfused == nsplit  # max|div u| and the tracked SOR error
    # one launch per sweep instead of one per colour; two more packed FP32 arrays
    assert lfused < lsplit
    assert mfused > msplit


@pytest.mark.parametrize("rows,planes", [(1, 1), (3, 5), (7, 2), (16, 40)])
def test_fused_tile_shapes_agree(rows, planes):
    shape = (36, 28, 22)
    s = G.settings_spheres_3d(precision="mixed", outer_max=2, inner_sweeps=4)
    vals = G.spheres_3d(*shape, count=5, seed=4)
    ref, nref, _, _ = _run(s.replace(sweep_form="split"), shape, vals, 3)
    got, ngot, _, _ = _run(s.replace(sweep_form="fused", fused_rows=rows, fused_planes=planes), shape, vals, 3)
    assert _same(got, ref)
    assert ngot == nref


def test_fused_eager_early_stop_and_untracked():
    """Eager launches, the defect correction's early stop (dc_tol) and error
    tracking off: still the split sweep's bits; an even inner_sweeps count
    leaves the correction in the first buffer."""
    shape = (30, 24, 26)
    vals = G.spheres_3d(*shape, count=4, seed=5)
    for kw in (dict(dc_tol=1e-3), dict(track_sor_error=False), dict(inner_sweeps=6)):
        s = G.settings_spheres_3d(precision="mixed", sweep_form="fused", outer_max=3,
                                  inner_sweeps=kw.pop("inner_sweeps", 5), **kw)
        ref = _run(s.replace(sweep_form="split"), shape, vals, 3, use_graph=False)[0]
        assert _same(_run(s, shape, vals, 3, use_graph=False)[0], ref), kw
        assert _same(_run(s, shape, vals, 3, use_graph=True)[0], ref), kw


def test_fused_not_used_for_odd_periodic_sizes():
    """Odd n or l needs the ghost-row refresh between colours: the case keeps
    the two-launch sweep (same memory and launches as asking for it)."""
    shape = (24, 21, 16)
    s = G.settings_spheres_3d(precision="mixed", sweep_form="fused", outer_max=1, inner_sweeps=3)
    vals = G.spheres_3d(*shape, count=3, seed=6)
    a = _run(s, shape, vals, 2)
    b = _run(s.replace(sweep_form="split"), shape, vals, 2)
    assert _same(a[0], b[0]) and a[2] == b[2] and a[3] == b[3]


def test_fused_case_bytes_match_allocation():
    from pixelflow_gb300 import _lib
    from pixelflow_gb300.solver import make_options, make_params
    import ctypes
    shape = (40, 32, 24)
    s = G.settings_spheres_3d(precision="mixed")
    vals = G.spheres_3d(*shape, count=3, seed=7)
    L = _lib.load()
    for form in ("auto", "fused", "split"):
        ss = s.replace(sweep_form=form)
        need = ctypes.c_size_t()
        prm, opt = make_params(ss, shape), make_options(ss)
        _lib.check(L.pf_case_bytes(ctypes.byref(prm), ctypes.byref(opt), ctypes.byref(need)))
        with Case(ss, shape, vals) as c:
            assert c.memory_bytes() == need.value, form


def test_bad_sweep_options_rejected():
    s = G.settings_spheres_3d(precision="mixed")
    vals = G.spheres_3d(8, 8, 8, count=1)
    with pytest.raises(ValueError):
        Case(s.replace(sweep_form="diagonal"), (8, 8, 8), vals)
    with pytest.raises(Exception):
        Case(s.replace(fused_rows=-1), (8, 8, 8), vals)


def test_fused_staging_timeout_reported_context_usable():
    """The bounded staging wait of the fused sweep: with one stage never
    issued, every CTA's wait runs out (0.2 s), each drains its own copies
    and leaves, and the host sees PF_E_TIMEOUT from then on; the GPU context
    stays usable -- a new case steps and matches the split sweep bit for bit."""
    from pixelflow_gb300 import _lib
    from pixelflow_gb300._lib import PfError
    shape = (32, 16, 16)
    s = G.settings_spheres_3d(precision="mixed", sweep_form="fused", outer_max=1, inner_sweeps=2)
    vals = G.spheres_3d(*shape, count=3, seed=8)
    L = _lib.load()
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        c.step(1)
        c.synchronize()
        _lib.check(L.pf_debug_fused_drop_stage(c.h, 1))
        c.step(1)
        with pytest.raises(PfError) as ei:
            c.synchronize()
        assert ei.value.code == -5  # PF_E_TIMEOUT
        with pytest.raises(PfError):
            c.get_state()
    with Case(s.replace(sweep_form="split"), shape, vals) as c:
        with pytest.raises(PfError) as ei:
            _lib.check(L.pf_debug_fused_drop_stage(c.h, 1))
        assert ei.value.code == -6  # PF_E_STATE: no fused sweep in this case
    a = _run(s, shape, vals, 2)[0]
    b = _run(s.replace(sweep_form="split"), shape, vals, 2)[0]
    assert _same(a, b)


@pytest.mark.parametrize("shape", [(40, 32, 24), (24, 21, 16)])
def test_auto_sweep_form_choice(shape):
    """PF_SWEEP_AUTO times both forms at creation on zero residual and
    correction (the state is untouched: same bits as the split run from the
    start) and keeps the faster; odd sizes measure nothing and keep split."""
    s = G.settings_spheres_3d(precision="mixed", outer_max=2, inner_sweeps=3)
    vals = G.spheres_3d(*shape, count=3, seed=9)
    with Case(s, shape, vals) as c:
        info = c.sweep_info()
        c.initial_conditions()
        c.step(2)
        got = c.get_state()
    if shape[1] % 2 == 0:
        assert info["split_ms"] > 0 and info["fused_ms"] > 0
        assert info["form"] == ("fused" if info["fused_ms"] < info["split_ms"] else "split")
    else:
        assert info == {"form": "split", "split_ms": 0.0, "fused_ms": 0.0}
    ref = _run(s.replace(sweep_form="split"), shape, vals, 2)[0]
    assert _same(got, ref)


def test_chunk_list_sweep_matches_fused_bit_for_bit():
    """On grids of more than one wave of CTAs the split FP32 sweep walks
    chunk lists (pf_dc_list.cu): the all-fluid chunks in warps of their own,
    their porosity taken as 1.0f without loads.  Every field must still equal
    the fused sweep's (which loads every operand) bit for bit, odd m
    included (the last chunk of a row holds the outlet lane), and the bytes
    must match the admission count."""
    from pixelflow_gb300 import _lib
    from pixelflow_gb300.solver import make_options, make_params
    import ctypes
    shape = (131, 128, 96)
    vals = G.spheres_3d(*shape, count=4, seed=11)
    s = G.settings_spheres_3d(precision="mixed", outer_max=2, inner_sweeps=5)
    L = _lib.load()
    for path in ("auto", "cells"):
        ss = s.replace(sweep_form="split", sor_path=path)
        with Case(ss, shape, vals) as c:
            info = c.dc_list_info()
            need = ctypes.c_size_t()
            _lib.check(L.pf_case_bytes(ctypes.byref(make_params(ss, shape)), ctypes.byref(make_options(ss)),
                                       ctypes.byref(need)))
            assert c.memory_bytes() == need.value, path
        assert info["listed"] == (path == "auto"), info
    chunks = (131 // 2 // 4 + 1) * 128 * 96
    with Case(s.replace(sweep_form="split"), shape, vals) as c:
        info = c.dc_list_info()
    for col in (0, 1):
        assert 0.3 * chunks < info["fluid"][col] < info["total"][col] <= chunks, info
    split, nsplit, _, _ = _run(s.replace(sweep_form="split"), shape, vals, 2)
    fused, nfused, _, _ = _run(s.replace(sweep_form="fused"), shape, vals, 2)
    assert _same(fused, split)
    assert nfused == nsplit
    eager, neager, _, _ = _run(s.replace(sweep_form="split"), shape, vals, 2, use_graph=False)
    assert _same(eager, split) and neager == nsplit
