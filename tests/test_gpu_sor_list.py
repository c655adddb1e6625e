"""The plain 3D sweep driven by cell lists (pf_sor_list.cu): the pure-fluid
cells (porosity 1 at the cell and its six neighbours) take the exact
six-neighbour sum and the one fluid constant, every other cell its own
stored coefficients.

* the exact sum against rational arithmetic (fractions.Fraction rounds to
  the nearest double): correctly rounded whenever the six exponents lie
  within the 7 guard bits, otherwise within 1 ulp of the sum plus 6 * 2^-7
  ulp of the largest term;
* the classification: the count of fluid cells per colour against a count
  from the porosity on the host;
* the list path against the oracle (the same bounds as the per-cell path)
  and against the per-cell path (the iterates differ only by the rounding
  of the fluid cells' neighbour sum).
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

from pixelflow_gb300 import _lib
from pixelflow_gb300 import geometry as G
from pixelflow_gb300.solver import Case
from oracle.oracle import OracleCase
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _sum6(x):
    L = _lib.load()
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 6)
    out = np.zeros(len(x))
    ok = np.zeros(len(x), dtype=np.int32)
    _lib.check(L.pf_debug_sum6(x.ctypes.data_as(ctypes.c_void_p), len(x), out.ctypes.data_as(ctypes.c_void_p),
                               ok.ctypes.data_as(ctypes.c_void_p)))
    return out, ok


def _exact(row):
    return float(sum((Fraction(float(v)) for v in row), Fraction(0)))


def test_sum6_correctly_rounded_near_exponents():
    rng = np.random.default_rng(1)
    n = 20000
    base = rng.uniform(-3, 3, size=(n, 1)) * 10.0 ** rng.integers(-20, 20, size=(n, 1))
    x = base * (1 + rng.uniform(-0.9, 0.9, size=(n, 6)))  # exponents within a few binades
    x[::7, 3] = -x[::7, 0]  # cancellations
    x[::11] = np.round(x[::11], 3)
    x[::13, :] = x[::13, :1]  # equal terms
    x[::17, 2] = 0.0
    out, ok = _sum6(x)
    assert ok.all()
    for i in range(n):
        row = x[i]
        e = np.frexp(row[row != 0])[1]
        if e.size and e.max() - e.min() <= 7:
            assert out[i] == _exact(row), (row.tolist(), out[i], _exact(row))


def test_sum6_error_bound_any_exponents_and_special_values():
    """Terms more than 7 binades below the largest are truncated to its scale
    2^-7 ulp: |sum - exact| <= 1 ulp(exact) + 6 * 2^-7 ulp(max|x|), far below
    the bound of a sequential FP64 sum, 5 * 2^-53 * sum|x|."""
    rng = np.random.default_rng(2)
    n = 20000
    x = rng.standard_normal((n, 6)) * 10.0 ** rng.integers(-30, 30, size=(n, 6))
    x[::5, 1] = -x[::5, 0]  # the largest terms cancel
    out, ok = _sum6(x)
    assert ok.all()
    for i in range(n):
        ex = _exact(x[i])
        bound = np.spacing(abs(ex)) + 6 * 2.0 ** -7 * np.spacing(np.max(np.abs(x[i])))
        assert abs(out[i] - ex) <= bound, (x[i].tolist(), out[i], ex)
    special = np.array([[0.0] * 6, [-0.0] * 6, [1.0, -1.0, 2.0, -2.0, 0.0, 0.0],
                        [np.inf, 1, 2, 3, 4, 5], [np.nan, 1, 2, 3, 4, 5], [5e-324, 5e-324, 0, 0, 0, 0],
                        [1.7e308, 1.7e308, 0, 0, 0, 0], [1e-300, -1e-300 * (1 - 2 ** -52), 0, 0, 0, 0]])
    out, ok = _sum6(special)
    assert ok[0] and out[0] == 0.0 and ok[1] and out[1] == 0.0 and ok[2] and out[2] == 0.0
    assert not ok[3] and not ok[4]  # Inf / NaN: the sweep adds in FP64 instead
    assert not ok[5]                # subnormal result
    assert not ok[6]                # overflow
    assert not ok[7]                # result below the normal range


def _fluid_counts(s, vals, shape):
    """Pure-fluid cells per colour from the porosity: the six normalised
    coefficients a_d * omega/ap, with a_d = dt*max(1e-6, (eps_c + eps_nb)*0.5)
    /h/h and ap = -a_e - a_w - a_n - a_s - a_t - a_b, evaluated in IEEE double
    in the library's order, equal those of a cell whose neighbourhood has
    porosity exactly 1 (a neighbour of 1 - 2^-53 can still round to the same
    coefficient), at interior i = 2 .. m-1 (the inlet and outlet rows carry
    the matrix edits).  Porosity ghosts: x copies, y/z periodic."""
    m, n, l = shape
    dx, dy, dz = s.width / (m - 1), s.height / (n - 1), s.depth / (l - 1)
    dt = s.time / s.istep_max
    e = np.pad(np.maximum(vals, s.threshold), 1, mode="wrap")
    e[:, :, 0] = e[:, :, 1]
    e[:, :, -1] = e[:, :, -2]
    c = e[1:-1, 1:-1, 1:-1]
    nbs = [(e[1:-1, 1:-1, 2:], dx), (e[1:-1, 1:-1, :-2], dx), (e[1:-1, 2:, 1:-1], dy), (e[1:-1, :-2, 1:-1], dy),
           (e[2:, 1:-1, 1:-1], dz), (e[:-2, 1:-1, 1:-1], dz)]

    def coefs(cc, nb_list):
        a = [dt * np.maximum(1e-6, (nb + cc) * 0.5 if d % 2 == 0 else (cc + nb) * 0.5) / h / h
             for d, (nb, h) in enumerate(nb_list)]
        ap = -a[0] - a[1] - a[2] - a[3] - a[4] - a[5]
        wap = s.relux_factor / ap
        return [x * wap for x in a]

    got = coefs(c, nbs)
    one = np.ones(1)
    ref = coefs(one, [(one, h) for _, h in nbs])
    fl = np.ones(c.shape, bool)
    for x, r in zip(got, ref):
        fl &= x == r[0]
    fl[:, :, 0] = False
    fl[:, :, -1] = False
    k, j, i = np.meshgrid(np.arange(1, l + 1), np.arange(1, n + 1), np.arange(1, m + 1), indexing="ij")
    colour = (i + j + k) & 1
    return [int(np.sum(fl & (colour == q))) for q in (0, 1)], [int(np.sum(colour == q)) for q in (0, 1)]


@pytest.mark.parametrize("shape", [(48, 40, 36), (47, 41, 35), (64, 64, 64)])
def test_list_classification_matches_host_count(shape):
    s = G.settings_spheres_3d(iter_max=2)
    vals = G.spheres_3d(*shape, count=6, seed=4)
    with Case(s, shape, vals) as c:
        info = c.sor_info()
    fluid, total = _fluid_counts(s, vals, shape)
    assert info["listed"]
    assert info["fluid"] == fluid and info["total"] == total, (info, fluid, total)
    assert 0 < fluid[0] < total[0]


@pytest.mark.parametrize("shape,steps", [((48, 40, 36), 12), ((47, 41, 35), 10), ((40, 32, 48), 10)])
def test_list_path_against_oracle_and_cells_path(shape, steps):
    s = G.settings_spheres_3d(iter_max=30)
    vals = G.spheres_3d(*shape, count=5, seed=9)
    ref = OracleCase(s, shape, vals)
    ref.initialize()
    e_ref = ref.step(steps)
    out = {}
    for path in ("auto", "cells"):
        with Case(s.replace(sor_path=path), shape, vals) as c:
            assert c.sor_info()["listed"] == (path == "auto")
            c.initial_conditions()
            c.step(steps)
            out[path] = (c.get_state(), c.norms())
    for path, (st, (md, se)) in out.items():
        for f in ("u", "v", "w", "p"):
            assert rel_l2(st[f], getattr(ref, f)) < 1e-11, (path, f)
        assert abs(se - e_ref) <= 1e-8 * abs(e_ref)
        assert abs(md - ref.divergence_diag()) <= 1e-8 * ref.divergence_diag()
    for f in ("u", "v", "w", "p"):
        assert rel_l2(out["auto"][0][f], out["cells"][0][f]) < 1e-12, f


def test_list_path_graph_and_eager_agree():
    s = G.settings_spheres_3d(iter_max=12)
    shape = (32, 30, 28)
    vals = G.spheres_3d(*shape, count=3, seed=2)
    outs = []
    for graph in (True, False):
        with Case(s, shape, vals, use_graph=graph) as c:
            c.initial_conditions()
            c.step(6)
            outs.append(c.get_state())
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(outs[0][f], outs[1][f]), f


def test_mixed_form_residual_over_lists():
    """The precision form's FP64 residual walks the same lists (3D): against
    the per-cell residual the FP32 right-hand side can differ in its last bit,
    so the two runs agree to FP32 level, and both stay within the form's
    bound against the plain FP64 step."""
    s = G.settings_spheres_3d(iter_max=20, outer_max=4, inner_sweeps=5)
    shape = (48, 40, 36)
    vals = G.spheres_3d(*shape, count=5, seed=9)
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        c.step(6)
        ref = c.get_state()
    out = {}
    for path in ("auto", "cells"):
        with Case(s.replace(precision="mixed", sor_path=path), shape, vals) as c:
            assert c.sor_info()["listed"] == (path == "auto")
            c.initial_conditions()
            c.step(6)
            out[path] = c.get_state()
    for f in ("u", "v", "w", "p"):
        assert rel_l2(out["auto"][f], out["cells"][f]) < 1e-6, f
        for path in out:
            assert rel_l2(out[path][f], ref[f]) < 1e-4, (path, f)


@pytest.mark.parametrize("shape", [(133, 129, 99), (130, 131, 97)])
def test_mixed_chunk_lists_odd_periodic_sizes(shape):
    """The precision form's FP32 sweep over chunk lists (pf_dc_list.cu) with
    odd n or l: the periodic neighbours are ghost rows/planes refreshed before
    each colour.  Against the per-cell sweep (sor_path "cells", whose FP64
    residual rounds the fluid cells' neighbour sum differently) the fields
    agree to FP32 level; both stay within the form's bound of the plain FP64
    step; the lists are used and hold most chunks as all-fluid."""
    s = G.settings_spheres_3d(iter_max=20, outer_max=4, inner_sweeps=5)
    vals = G.spheres_3d(*shape, count=4, seed=13)
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        c.step(4)
        ref = c.get_state()
    out = {}
    for path in ("auto", "cells"):
        with Case(s.replace(precision="mixed", sor_path=path, sweep_form="split"), shape, vals) as c:
            info = c.dc_list_info()
            assert info["listed"] == (path == "auto"), info
            if path == "auto":
                assert all(0.3 * t < f < t for f, t in zip(info["fluid"], info["total"])), info
            c.initial_conditions()
            c.step(4)
            out[path] = c.get_state()
    for f in ("u", "v", "w", "p"):
        assert rel_l2(out["auto"][f], out["cells"][f]) < 1e-6, f
        for path in out:
            assert rel_l2(out[path][f], ref[f]) < 1e-4, (path, f)
