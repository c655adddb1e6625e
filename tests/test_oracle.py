"""The oracle (C restatement of the reference step) against an independent
numpy restatement, the reference's colour mapping, physical invariants and
the committed golden vectors.  CPU only."""
import itertools
import os

import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from oracle.np_oracle import NpCase
from oracle.oracle import OracleCase

from tests.golden.make_golden import CASES as GOLDEN_CASES

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _case2d(shape, iters=7, dtype=np.float64):
    m, n = shape
    s = G.settings_cylinder_2d(iter_max=iters)
    return s, G.cylinder_2d(m, n, radius=0.2, cx=0.6, cy=0.45)


def _case3d(shape, iters=5):
    m, n, l = shape
    s = G.settings_spheres_3d(iter_max=iters)
    sph = np.array([[0.4, 0.5, 0.5, 0.2], [0.7, 0.3, 0.6, 0.15]])
    return s, G.spheres_3d(m, n, l, spheres=sph)


@pytest.mark.parametrize("shape", [(8, 6), (9, 6), (8, 7), (9, 7), (16, 12)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_c_oracle_matches_numpy_restatement_2d(shape, dtype):
    s, vals = _case2d(shape)
    a, b = OracleCase(s, shape, vals, dtype), NpCase(s, shape, vals, dtype)
    a.initialize()
    b.initialize()
    assert np.array_equal(a.poro, b.poro)
    for _ in range(3):
        assert a.step(1) == b.step(1)
        for f in ("u", "v", "p"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.divergence_diag() == b.divergence_diag()[0]


@pytest.mark.parametrize("shape", [(6, 6, 6), (7, 6, 6), (6, 7, 6), (7, 7, 5), (6, 5, 7), (8, 6, 4)])
def test_c_oracle_matches_numpy_restatement_3d(shape):
    s, vals = _case3d(shape)
    a, b = OracleCase(s, shape, vals), NpCase(s, shape, vals)
    a.initialize()
    b.initialize()
    for _ in range(2):
        assert a.step(1) == b.step(1)
        for f in ("u", "v", "w", "p"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), f


def _ref_colours_2d(m, n):
    """The reference's linear-index mapping (ibm_2d_uniform_omp_cpu.f90:339-344, 373-378)."""
    first, second = [], []
    for k in range(2, m * n + 1, 2):
        j = (k - 1) // m + 1
        i = k - (j - 1) * m
        if m % 2 == 0 and j % 2 == 0:
            i -= 1
        first.append((i, j))
    for k in range(1, m * n + 1, 2):
        j = (k - 1) // m + 1
        i = k - (j - 1) * m
        if m % 2 == 0 and j % 2 == 0:
            i += 1
        second.append((i, j))
    return first, second


def _ref_colours_3d(m, n, l):
    """ibm_3d_uniform_omp_cpu.f90:493-508, 550-565."""
    out = []
    for start, sign in ((2, -1), (1, +1)):
        cells = []
        for ii in range(start, m * n * l + 1, 2):
            k = (ii - 1) // (m * n) + 1
            j = ((ii - 1) // m + 1) - (k - 1) * n
            i = (ii - (j - 1) * m) - (k - 1) * m * n
            if m % 2 != 0 and n % 2 == 0 and k % 2 == 0:
                j = j + sign if i % 2 != 0 else j - sign
            elif m % 2 == 0 and (j % 2 + k % 2 == 1):
                i = i + sign
            cells.append((i, j, k))
        out.append(cells)
    return out


@pytest.mark.parametrize("m,n", list(itertools.product(range(2, 9), range(2, 9))))
def test_colour_order_2d(m, n):
    first, second = _ref_colours_2d(m, n)
    allc = {(i, j) for i in range(1, m + 1) for j in range(1, n + 1)}
    assert len(set(first)) == len(first) and len(set(second)) == len(second)
    assert set(first) | set(second) == allc and not set(first) & set(second)
    assert set(first) == {(i, j) for (i, j) in allc if (i + j) % 2 == 1}
    # the GPU colour function: colour 0 sweeps first, colour = (i + j + 1) & 1
    assert all(((i + j + 1) & 1) == 0 for (i, j) in first)


@pytest.mark.parametrize("m,n,l", list(itertools.product(range(2, 7), range(2, 7), range(2, 6))))
def test_colour_order_3d(m, n, l):
    first, second = _ref_colours_3d(m, n, l)
    allc = {(i, j, k) for i in range(1, m + 1) for j in range(1, n + 1) for k in range(1, l + 1)}
    assert set(first) | set(second) == allc and not set(first) & set(second)
    assert len(first) == len(set(first))
    assert all(((i + j + k) & 1) == 0 for (i, j, k) in first)


def test_uniform_flow_is_steady():
    """Porosity 1 everywhere, AoA 0: u = U, v = 0, p = p_out stay exact."""
    s = G.settings_cylinder_2d(iter_max=10)
    shape = (16, 10)
    c = OracleCase(s, shape, np.ones((10, 16)))
    c.initialize()
    c.step(5)
    assert np.all(c.u == 1.0) and np.all(c.v == 0.0) and np.all(c.p == 0.0)
    s3 = G.settings_spheres_3d(iter_max=4)
    c3 = OracleCase(s3, (8, 6, 6), np.ones((6, 6, 8)))
    c3.initialize()
    c3.step(3)
    assert np.all(c3.u == 1.0) and np.all(c3.v == 0.0) and np.all(c3.w == 0.0) and np.all(c3.p == 0.0)


def test_periodic_shift_and_lagged_ghost_quirk():
    """Without pressure (iter_max=0) a shift of the geometry by an even number
    of rows shifts the solution bit for bit.  With the SOR running it does
    not: bb at the rows next to the periodic boundary reads the ghost
    velocities left by the previous step's boundary call instead of the new
    predictor values (ibm_2d_uniform_omp_cpu.f90:271-274), so the first
    difference appears in bb on the periodic rows of the second step."""
    m, n, shift = 20, 12, 4
    vals = G.cylinder_2d(m, n, radius=0.25, cx=0.8, cy=0.4)
    R = lambda x: np.roll(x[1:-1], shift, axis=0)
    s0 = G.settings_cylinder_2d(iter_max=0)
    a, b = OracleCase(s0, (m, n), vals), OracleCase(s0, (m, n), np.roll(vals, shift, axis=0))
    a.initialize(); b.initialize()
    a.step(3); b.step(3)
    for f in ("u", "v", "p"):
        assert np.array_equal(R(getattr(a, f)), getattr(b, f)[1:-1]), f
    s1 = G.settings_cylinder_2d(iter_max=1)
    a, b = OracleCase(s1, (m, n), vals), OracleCase(s1, (m, n), np.roll(vals, shift, axis=0))
    a.initialize(); b.initialize()
    a.step(1); b.step(1)
    assert np.array_equal(R(a.p), b.p[1:-1])
    for c in (a, b):
        c.copy_old(); c.divergence(); c.predictor(); c.coefficients()
    assert np.array_equal(R(a.u), b.u[1:-1])
    d = np.abs(R(a.work("bb")) - b.work("bb")[1:-1])
    rows = set(np.nonzero(d)[0].tolist())
    # b's periodic rows (0, n-1) and a's, which the shift moves to (shift, shift-1)
    assert rows and rows <= {0, n - 1, shift - 1, shift}


def test_sor_error_semantics():
    """2D error is the running max over both half-sweeps, 3D over the
    second half-sweep only; both are non-negative and finite."""
    s, vals = _case2d((10, 8), iters=3)
    a = OracleCase(s, (10, 8), vals)
    a.initialize()
    e = a.step(1)
    assert np.isfinite(e) and e > 0


@pytest.mark.parametrize("name", sorted(f + ".npz" for f in GOLDEN_CASES))
def test_oracle_reproduces_golden(name):
    from tests.golden.make_golden import CASES, run_oracle
    spec = CASES[name[:-4]]
    out = run_oracle(spec)
    ref = np.load(os.path.join(GOLDEN, name))
    for k in ref.files:
        assert np.array_equal(out[k], ref[k]), k


@pytest.mark.parametrize("dim", [2, 3])
def test_force_log_c_matches_numpy(dim):
    """The force sums of output_force_log_2d/_3d: the C restatement (loop
    order) and the vectorised one agree to rounding of the sum order."""
    from oracle import np_oracle
    s, vals = _case2d((24, 16)) if dim == 2 else _case3d((10, 9, 8))
    shape = (24, 16) if dim == 2 else (10, 9, 8)
    a = OracleCase(s, shape, vals)
    a.initialize()
    a.step(2)
    fp, fv = a.forces()
    sc = a.scalars()
    bp, bv, mag = np_oracle.forces(a.poro, a.p, a.u, a.v, a.w, sc["dx"], sc["dy"], sc["dz"], s.thickness,
                                   s.density, s.xnue)
    assert np.all(np.abs(np.r_[fp - bp, fv - bv]) <= 1e-13 * np.maximum(mag, 1e-300))
    assert abs(fp[0]) > 0 and abs(fv[0]) > 0
    if dim == 2:
        assert fp[2] == 0 and fv[2] == 0


@pytest.mark.parametrize("shape", [(12, 8), (9, 7), (7, 6, 5)])
def test_backstep_inflow_c_matches_numpy(shape):
    """The backstep program's boundary and initial conditions (inflow and
    initial velocity times porosity, ibm_2d_backstep_omp_cpu.f90:533-534,
    615-618): both restatements agree bit for bit, and the inlet column holds
    U * porosity."""
    if len(shape) == 2:
        s, vals = _case2d(shape)
        # an obstacle touching the inlet, so the inflow profile is not uniform
        vals = np.minimum(vals, G.cylinder_2d(shape[0], shape[1], radius=0.3, cx=0.0, cy=0.5))
    else:
        s, vals = _case3d(shape)
    s = s.replace(inflow_porosity=True)
    a, b = OracleCase(s, shape, vals), NpCase(s, shape, vals)
    a.initialize()
    b.initialize()
    inlet = (slice(1, -1), 1) if len(shape) == 2 else (slice(1, -1), slice(1, -1), 1)
    assert np.array_equal(a.u[inlet], s.inlet_velocity * a.poro[inlet])
    for _ in range(2):
        assert a.step(1) == b.step(1)
        for f in ("u", "v", "p") + (("w",) if len(shape) == 3 else ()):
            assert np.array_equal(getattr(a, f), getattr(b, f)), f
    plain = OracleCase(s.replace(inflow_porosity=False), shape, vals)
    plain.initialize()
    assert not np.array_equal(plain.u, a.u)


@pytest.mark.parametrize("shape", [(12, 8), (9, 7), (10, 3)])
def test_slip_rows_c_matches_numpy(shape):
    """The 2D symmetry rows the reference keeps commented out
    (ibm_2d_uniform_omp_cpu.f90:440-450, 512-526): both restatements agree
    bit for bit; after a step v is 0 on rows 1 and n, the ghost rows mirror
    u and p and negate v, and the run differs from the periodic one."""
    s, vals = _case2d(shape)
    s = s.replace(slip_y=True)
    a, b = OracleCase(s, shape, vals), NpCase(s, shape, vals)
    a.initialize()
    b.initialize()
    m, n = shape
    I = slice(1, m + 1)
    for _ in range(3):
        assert a.step(1) == b.step(1)
        for f in ("u", "v", "p"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), f
        assert not a.v[1, I].any() and not a.v[n, I].any()
        assert np.array_equal(a.u[0, I], a.u[2, I]) and np.array_equal(a.u[n + 1, I], a.u[n - 1, I])
        assert np.array_equal(a.v[0, I], -a.v[2, I]) and np.array_equal(a.p[n + 1, I], a.p[n - 1, I])
    periodic = OracleCase(s.replace(slip_y=False), shape, vals)
    periodic.initialize()
    periodic.step(3)
    assert not np.array_equal(periodic.p, a.p)


AIR_CONDITION_TABLE = (1, 0, 0, 0, 0, 2)  # ibm_3d_air_condition_omp_cpu.f90:10-15


def _room(shape):
    """A room with an opening in the ceiling (inlet) and one in the south wall
    (outlet), an obstacle inside: porosity 1 in the openings, low elsewhere
    on those faces."""
    m, n, l = shape
    s = G.settings_spheres_3d(iter_max=6, walls=AIR_CONDITION_TABLE, inlet_velocity=0.5)
    vals = G.spheres_3d(m, n, l, spheres=np.array([[0.5, 0.5, 0.4, 0.2]]))
    vals[-1, : n // 2, : m // 2] = 0.05   # ceiling: inlet only over part of it
    vals[:, 0, m // 2:] = 0.05            # south wall: outlet only on one side
    return s, vals


@pytest.mark.parametrize("shape", [(8, 7, 6), (7, 8, 7), (9, 6, 8)])
@pytest.mark.parametrize("table", [AIR_CONDITION_TABLE, (2, 1, 0, 1, 2, 0), (0, 2, 2, 0, 1, 1)])
def test_air_condition_c_matches_numpy(shape, table):
    """The air-condition program (wall table, non-periodic ghosts): the C and
    numpy restatements agree bit for bit over several steps, for the
    reference's table and for tables exercising every face type."""
    s, vals = _room(shape)
    s = s.replace(walls=table)
    a, b = OracleCase(s, shape, vals), NpCase(s, shape, vals)
    assert np.array_equal(a.poro, b.poro)
    a.initialize()
    b.initialize()
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), ("init", f)
    for it in range(3):
        assert a.step(1) == b.step(1)
        for f in ("u", "v", "w", "p"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), (it, f)
    assert np.isfinite(a.p).all() and np.abs(a.w).max() > 0


def test_air_condition_walls_hold():
    """Wall faces keep zero velocity, the inlet opening carries the inflow,
    the outlet ghosts hold the outlet pressure."""
    shape = (10, 9, 8)
    s, vals = _room(shape)
    a = OracleCase(s, shape, vals)
    a.initialize()
    a.step(2)
    m, n, l = shape
    po = a.poro
    # away from the edges the later faces (west, east, north, south) overwrite
    top = a.w[l, 2:n, 2:m]
    open_top = po[l, 2:n, 2:m] >= 0.9
    assert open_top.any() and (~open_top).any()
    assert np.all(top[open_top] == -s.inlet_velocity) and np.all(top[~open_top] == 0)
    assert np.all(a.u[1:l + 1, 1:n + 1, 1] == 0) and np.all(a.u[1:l + 1, 1:n + 1, m] == 0)
    south_open = po[1:l + 1, 1, 1:m + 1] >= 0.9
    assert np.all(a.p[1:l + 1, 0, 1:m + 1][south_open] == s.outlet_pressure)
