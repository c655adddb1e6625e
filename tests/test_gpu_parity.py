"""GPU parity: the CUDA step through the C ABI against the oracle (the C
restatement of the reference's OpenMP step) and the golden vectors.

Tolerances (relative L2 over the whole field incl. ghosts; velocity is
measured as the vector field (u, v[, w]) and pressure on its own):
  * a few steps / single stages: 1e-12 -- the GPU reorders the floating point
    operations of each expression (reciprocal multiplies, FMAs), so it is not
    bit-identical, but every stage agrees to a few ulp;
  * long runs: 1e-10 after 1000 steps (the parity bar for the plain FP64 step),
    asserted for u, v[, w] and p each on its own as well: the 2D cylinder for
    its 1000 steps, the 3D geometry at 64^3 for 60 steps, and the benchmarked
    256^3 case for the 25 steps the benchmark runs.
"""
import ctypes
import os

import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300.solver import Case
from oracle.oracle import OracleCase
from tests.conftest import rel_l2, rel_vel
from tests.golden.make_golden import CASES, case_inputs
from tests.golden.make_reference_pin import CASES as REFPIN_CASES, case_inputs as refpin_inputs

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS2, FIELDS3 = ("u", "v", "p"), ("u", "v", "w", "p")


def fields(dim):
    return FIELDS2 if dim == 2 else FIELDS3


def errors(got, ref, dim):
    """{'vel': vector relative L2, 'p': pressure relative L2, 'fields': {f:
    relative L2 of each field u, v[, w], p on its own}}"""
    r = ref if isinstance(ref, dict) else {f: getattr(ref, f) for f in fields(dim)}
    return {"vel": rel_vel(got, r, dim), "p": rel_l2(got["p"], r["p"]),
            "fields": {f: rel_l2(got[f], r[f]) for f in fields(dim)}}


def assert_each_field(errs, bound):
    """Every field within `bound` on its own: a small component (v, w beside
    the inflow u) must not hide inside the vector norm."""
    bad = {f: e for f, e in errs["fields"].items() if not e < bound}
    assert not bad, (bound, errs)


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(name):
    spec = CASES[name]
    s, vals = case_inputs(spec)
    ref = np.load(os.path.join(GOLDEN, name + ".npz"))
    with Case(s, spec["shape"], vals) as c:
        assert np.array_equal(c.porosity(), ref["poro"])
        c.initial_conditions()
        c.step(spec["steps"])
        got = c.get_state()
        max_div, sor_err = c.norms()
    e = errors(got, {f: ref[f] for f in fields(spec["dim"])}, spec["dim"])
    assert e["vel"] < 1e-12 and e["p"] < 1e-12, e
    assert abs(sor_err - float(ref["sor_error"])) <= 1e-9 * abs(float(ref["sor_error"]))
    assert abs(max_div - float(ref["max_div"])) <= 1e-9 * abs(float(ref["max_div"]))


def _pair(s, shape, vals, **kw):
    ref = OracleCase(s, shape, vals)
    ref.initialize()
    return ref, Case(s, shape, vals, **kw)


@pytest.mark.parametrize("shape", [(40, 20), (41, 21), (33, 18)])
def test_predictor_and_rhs_stage(shape):
    """solve_p with iter_max=0 leaves p alone and returns u*, v* of the predictor."""
    s = G.settings_cylinder_2d(iter_max=0)
    vals = G.cylinder_2d(*shape, radius=0.2, cx=0.7, cy=0.45)
    ref, c = _pair(s, shape, vals)
    with c:
        c.initial_conditions()
        ref.step(2)
        c.step(2)  # non-trivial state with pressure still 0
        ref.copy_old()
        ref.solve_p()
        c.solve_p()
        got = c.get_state()
    e = errors(got, ref, 2)
    assert e["vel"] < 1e-13, e


@pytest.mark.parametrize("shape", [(24, 16), (25, 15), (16, 11, 9), (15, 12, 10)])
def test_solve_p_projection_boundary_stages(shape):
    dim = len(shape)
    if dim == 2:
        s = G.settings_cylinder_2d(iter_max=3)
        vals = G.cylinder_2d(*shape, radius=0.2, cx=0.7, cy=0.45)
    else:
        s = G.settings_spheres_3d(iter_max=3)
        vals = G.spheres_3d(*shape, spheres=np.array([[0.5, 0.45, 0.5, 0.25]]))
    ref, c = _pair(s, shape, vals)
    with c:
        c.initial_conditions()
        ref.step(2)
        st = ref.state()
        c.set_state(st["u"], st["v"], st["p"], st.get("w"))
        ref.copy_old()
        ref.solve_p()
        c.solve_p()
        got = c.get_state()
        e = errors(got, ref, dim)
        assert e["vel"] < 1e-12 and e["p"] < 1e-12, ("solve_p", e)
        ref.projection()
        c.projection()
        ref.boundary()
        c.boundary()
        got = c.get_state()
        e = errors(got, ref, dim)
        assert e["vel"] < 1e-12 and e["p"] < 1e-12, ("projection+boundary", e)


def test_state_roundtrip_fortran_leading_dims():
    """pf_set_state / pf_get_state with the caller's static (0:md,0:nd) arrays."""
    s = G.settings_spheres_3d(iter_max=2)
    m, n, l = 13, 9, 6
    vals = G.spheres_3d(m, n, l, count=2, seed=1)
    with Case(s, (m, n, l), vals) as c:
        md1, nd1 = m + 7, n + 4
        rng = np.random.default_rng(0)
        src = {f: rng.standard_normal((l + 2, nd1, md1)) for f in FIELDS3}
        c.set_state(src["u"], src["v"], src["p"], src["w"])
        out = {f: np.zeros((l + 2, nd1, md1)) for f in FIELDS3}
        c.get_state(out)
        for f in FIELDS3:
            assert np.array_equal(out[f][:, : n + 2, : m + 2], src[f][:, : n + 2, : m + 2]), f
            assert not out[f][:, n + 2:, :].any() and not out[f][:, :, m + 2:].any()


@pytest.mark.parametrize("dim", [2, 3])
def test_padded_get_state_right_after_steps(dim):
    """pf_get_state into padded (pageable, strided) arrays called straight
    after steps are enqueued returns the finished step: the same bits as the
    dense read of the same state."""
    if dim == 2:
        s, shape = G.settings_cylinder_2d(iter_max=40), (200, 96)
        vals = G.cylinder_2d(*shape, radius=0.15, cx=0.6, cy=0.5)
    else:
        s, shape = G.settings_spheres_3d(iter_max=40), (64, 48, 40)
        vals = G.spheres_3d(*shape, count=4, seed=3)
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        fs = c.field_shape
        pad = fs[:-2] + (fs[-2] + 5, fs[-1] + 9)
        for _ in range(2):
            c.step(4)  # asynchronous: still running when get_state is called
            out = {f: np.full(pad, np.nan) for f in fields(dim)}
            c.get_state(out)
            dense = c.get_state()
            for f in fields(dim):
                got = out[f][..., : fs[-2], : fs[-1]]
                assert np.array_equal(got, dense[f]), f
                assert np.isnan(out[f][..., fs[-2]:, :]).all() and np.isnan(out[f][..., :, fs[-1]:]).all()


@pytest.mark.parametrize("dim", [2, 3])
def test_graph_replay_matches_eager_launches(dim):
    if dim == 2:
        s, shape = G.settings_cylinder_2d(iter_max=15), (48, 30)
        vals = G.cylinder_2d(*shape, radius=0.2, cx=0.6, cy=0.5)
    else:
        s, shape = G.settings_spheres_3d(iter_max=8), (20, 16, 14)
        vals = G.spheres_3d(*shape, count=3, seed=2)
    outs = []
    for graph in (True, False):
        with Case(s, shape, vals, use_graph=graph) as c:
            c.initial_conditions()
            c.step(7)
            outs.append((c.get_state(), c.norms()))
    for f in fields(dim):
        assert np.array_equal(outs[0][0][f], outs[1][0][f]), f
    assert outs[0][1] == outs[1][1]


@pytest.mark.parametrize("shape,steps", [((64, 32), 40), ((63, 33), 30), ((30, 24, 20), 12),
                                         ((29, 23, 21), 10), ((24, 25, 18), 10)])
def test_multi_step_parity(shape, steps):
    dim = len(shape)
    if dim == 2:
        s = G.settings_cylinder_2d(iter_max=30)
        vals = G.cylinder_2d(*shape, radius=0.15, cx=0.6, cy=0.5)
    else:
        s = G.settings_spheres_3d(iter_max=20)
        vals = G.spheres_3d(*shape, count=4, seed=5)
    ref, c = _pair(s, shape, vals)
    with c:
        c.initial_conditions()
        c.step(steps)
        got = c.get_state()
        max_div, sor_err = c.norms()
    e_ref = ref.step(steps)
    e = errors(got, ref, dim)
    assert e["vel"] < 1e-11 and e["p"] < 1e-11, e
    assert abs(sor_err - e_ref) <= 1e-8 * abs(e_ref)
    assert abs(max_div - ref.divergence_diag()) <= 1e-8 * ref.divergence_diag()


def test_uniform_flow_stays_exact():
    s = G.settings_spheres_3d(iter_max=10)
    with Case(s, (16, 12, 10), np.ones((10, 12, 16))) as c:
        c.initial_conditions()
        c.step(5)
        st = c.get_state()
    assert np.all(st["u"] == 1.0) and not st["v"].any() and not st["w"].any() and not st["p"].any()


def test_nonfinite_fields_are_reported():
    """A run that diverges (wide porosity tail, see geometry.py) is reported by
    pf_norms as PF_E_NONFINITE instead of returning garbage silently."""
    s = G.settings_cylinder_2d(iter_max=100)
    vals = G.cylinder_2d(512, 256, edge=2.0)
    with Case(s, (512, 256), vals) as c:
        c.initial_conditions()
        c.step(120)
        md = ctypes.c_double()
        se = ctypes.c_double()
        rc = c.L.pf_norms(c.h, ctypes.byref(md), ctypes.byref(se))
    assert rc == -4 and not np.isfinite(md.value)


@pytest.mark.slow
def test_cylinder_512x256_1000_steps_parity():
    """The 2D benchmark case for its full 1000 steps against the oracle:
    u, v, p within 1e-10 relative L2."""
    s = G.settings_cylinder_2d()
    vals = G.cylinder_2d()
    ref, c = _pair(s, (512, 256), vals)
    with c:
        c.initial_conditions()
        c.step(1000)
        got = c.get_state()
        max_div, _ = c.norms()
    ref.step(1000)
    errs = errors(got, ref, 2)
    print("1000-step relative L2 vs oracle:", errs, "max|div|", max_div, ref.divergence_diag())
    assert errs["vel"] < 1e-10 and errs["p"] < 1e-10, errs
    assert_each_field(errs, 1e-10)


@pytest.mark.slow
def test_cylinder_512x256_slip_1000_steps_parity():
    """The 2D benchmark case as configured with slip top and bottom walls
    (the reference's commented symmetry rows, slip_y) for 1000 steps against
    the oracle: u, v, p each within 1e-10 relative L2."""
    s = G.settings_cylinder_2d(slip_y=True)
    vals = G.cylinder_2d()
    ref, c = _pair(s, (512, 256), vals)
    with c:
        c.initial_conditions()
        c.step(1000)
        got = c.get_state()
    ref.step(1000)
    errs = errors(got, ref, 2)
    print("1000-step slip relative L2 vs oracle:", errs)
    assert_each_field(errs, 1e-10)


@pytest.mark.slow
def test_spheres_3d_reduced_parity():
    """The 3D benchmark geometry (32 seeded spheres) on a 64x64x64 grid for
    60 steps with iter_max=100."""
    s = G.settings_spheres_3d()
    shape = (64, 64, 64)
    vals = G.spheres_3d(*shape)
    ref, c = _pair(s, shape, vals)
    with c:
        c.initial_conditions()
        c.step(60)
        got = c.get_state()
    ref.step(60)
    errs = errors(got, ref, 3)
    print("3D 64^3 60-step relative L2 vs oracle:", errs)
    assert errs["vel"] < 1e-10 and errs["p"] < 1e-10, errs
    assert_each_field(errs, 1e-10)


@pytest.mark.slow
def test_spheres_3d_256_benchmark_case_parity():
    """The benchmarked case itself -- 256^3, 32 seeded spheres, iter_max 100,
    omega 1.7, nu 1e-3, dt 1e-4 -- for its first 25 steps (the steps the
    benchmark warms up on and times), GPU against the oracle run on all host
    cores: u, v, w and p each within 1e-10 relative L2, the reference's SOR
    error within 1e-8 and max|div u| within 1e-8 relative."""
    s = G.settings_spheres_3d()
    shape = (256, 256, 256)
    vals = G.spheres_3d(*shape)
    steps = 25
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        c.step(steps)
        got = c.get_state()
        max_div, sor_err = c.norms()
    ref = OracleCase(s, shape, vals)
    ref.initialize()
    e_ref = ref.step(steps)
    errs = errors(got, ref, 3)
    ref_div = ref.divergence_diag()
    print("3D 256^3 25-step relative L2 vs oracle, per field:", errs["fields"], "max|div|", max_div, ref_div,
          "sor error", sor_err, e_ref)
    assert_each_field(errs, 1e-10)
    assert abs(sor_err - e_ref) <= 1e-8 * abs(e_ref)
    assert abs(max_div - ref_div) <= 1e-8 * ref_div


@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_precision_error_against_fp64(dim):
    """FP32 stencils and sweeps inside FP64 defect correction (4 passes x 25
    sweeps) against the plain FP64 step with iter_max = 100, on the benchmark
    geometries.  Stated bounds (relative L2): velocity 1e-7 throughout;
    pressure 1e-6 after the first (impulsive) step, and after 60 steps in 3D;
    5e-5 after 300 steps in 2D, where the FP32 velocity stencils' rounding
    accumulates in smooth pressure modes that 100 SOR sweeps per step never
    damp while the pressure level decays (|p|max 298 -> 1.6); measured
    1.1e-5 there, 1.4e-7 in 3D."""
    if dim == 2:
        s, shape, steps, pbound = G.settings_cylinder_2d(), (512, 256), 300, 5e-5
        vals = G.cylinder_2d()
    else:
        s, shape, steps, pbound = G.settings_spheres_3d(), (64, 64, 64), 60, 1e-6
        vals = G.spheres_3d(*shape)
    cs = {}
    for prec in ("fp64", "mixed"):
        cs[prec] = Case(s.replace(precision=prec), shape, vals)
        cs[prec].initial_conditions()
        cs[prec].step(1)
    e1 = errors(cs["mixed"].get_state(), cs["fp64"].get_state(), dim)
    for c in cs.values():
        c.step(steps - 1)
    e = errors(cs["mixed"].get_state(), cs["fp64"].get_state(), dim)
    for c in cs.values():
        c.close()
    print(f"mixed vs fp64 {dim}D {shape}: after 1 step {e1}, after {steps} steps {e}")
    assert e1["vel"] < 1e-7 and e1["p"] < 1e-6, e1
    assert e["vel"] < 1e-7 and e["p"] < pbound, e


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim", [2, 3])
def test_force_log_matches_oracle(dim, precision):
    """pf_forces against the oracle's force sums on the GPU's own state (so
    only the reduction is compared), to rounding of the summation order, and
    reproducible bit for bit from call to call."""
    from oracle import np_oracle
    if dim == 2:
        s = G.settings_cylinder_2d(iter_max=40, precision=precision)
        shape, vals = (128, 64), G.cylinder_2d(128, 64, radius=0.2, cx=0.6, cy=0.5)
    else:
        s = G.settings_spheres_3d(iter_max=20, precision=precision)
        shape, vals = (40, 36, 32), G.spheres_3d(40, 36, 32, count=4, seed=2)
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        c.step(5)
        f1 = c.forces(radius=0.2)
        f2 = c.forces(radius=0.2)
        st = c.get_state()
        por = c.porosity()
    o = OracleCase(s.replace(precision="fp64"), shape, vals.ravel())
    sc = o.scalars()
    bp, bv, mag = np_oracle.forces(por, st["p"], st["u"], st["v"], st.get("w"), sc["dx"], sc["dy"], sc["dz"],
                                   s.thickness, s.density, s.xnue)
    got = np.r_[f1["Fp"], f1["Fv"]]
    want = np.r_[bp[:dim], bv[:dim]]
    scale = np.r_[mag[:dim], mag[3:3 + dim]]
    assert np.all(np.abs(got - want) <= 1e-12 * np.maximum(scale, 1e-300)), (got, want)
    for k in f1:
        assert np.array_equal(np.asarray(f1[k]), np.asarray(f2[k])), k
    key = "Cd" if dim == 2 else "Cd_x"
    assert np.isfinite(f1[key])


@pytest.mark.parametrize("shape,steps", [((64, 32), 40), ((63, 33), 30), ((24, 20, 16), 10)])
def test_backstep_inflow_parity(shape, steps):
    """The backstep program (inflow and initial velocities times porosity,
    ibm_2d_backstep_omp_cpu.f90:533-534, 615-618) against the oracle, with an
    obstacle across the inlet so the inflow profile is not uniform; the batch
    kernel gives the single-case bits for the same settings."""
    from pixelflow_gb300.batch import Batch
    dim = len(shape)
    if dim == 2:
        s = G.settings_cylinder_2d(iter_max=30, inflow_porosity=True)
        vals = np.minimum(G.cylinder_2d(*shape, radius=0.15, cx=0.6, cy=0.5),
                          G.cylinder_2d(*shape, radius=0.3, cx=0.0, cy=0.3))
    else:
        s = G.settings_spheres_3d(iter_max=20, inflow_porosity=True)
        vals = G.spheres_3d(*shape, spheres=np.array([[0.0, 0.5, 0.5, 0.3], [0.6, 0.4, 0.5, 0.2]]))
    ref, c = _pair(s, shape, vals)
    with c:
        c.initial_conditions()
        u0 = c.get_state()["u"]
        c.step(steps)
        got = c.get_state()
    inlet = (slice(1, -1), 1) if dim == 2 else (slice(1, -1), slice(1, -1), 1)
    assert np.array_equal(u0[inlet], ref.u[inlet])
    ref.step(steps)
    e = errors(got, ref, dim)
    assert e["vel"] < 1e-11 and e["p"] < 1e-11, e
    sm = s.replace(precision="mixed")
    with Case(sm, shape, vals) as one, Batch(cluster=2, threads=256) as b:
        one.initial_conditions()
        one.step(3)
        slot = b.add(sm, shape, vals)
        b.step(3)
        a, bb = one.get_state(), b.get_state(slot)
        assert all(np.array_equal(a[k], bb[k]) for k in a)


@pytest.mark.parametrize("shape,steps", [((64, 32), 60), ((63, 33), 40), ((96, 48), 30)])
def test_slip_rows_parity(shape, steps):
    """The 2D symmetry ("slip") rows at j = 1 and j = n, the option the
    reference keeps commented out (ibm_2d_uniform_omp_cpu.f90:440-450 in
    boundrary_matrix, :512-526 in boundary), against the oracle field by
    field (odd n: the SOR's ghost rows are refreshed and multiplied by the
    zeroed coefficients); v is 0 on both rows; the precision form refuses
    the option."""
    s = G.settings_cylinder_2d(iter_max=30, slip_y=True)
    vals = G.cylinder_2d(*shape, radius=0.15, cx=0.6, cy=0.4)
    ref, c = _pair(s, shape, vals)
    with c:
        c.initial_conditions()
        c.step(steps)
        got = c.get_state()
        md, se = c.norms()
    e_ref = ref.step(steps)
    e = errors(got, ref, 2)
    assert_each_field(e, 1e-11)
    m, n = shape
    assert not got["v"][1, 1:m + 1].any() and not got["v"][n, 1:m + 1].any()
    assert abs(se - e_ref) <= 1e-8 * abs(e_ref)
    assert abs(md - ref.divergence_diag()) <= 1e-8 * ref.divergence_diag()
    with pytest.raises(Exception):
        Case(s.replace(precision="mixed"), shape, vals)
    with pytest.raises(Exception):
        Case(G.settings_spheres_3d(slip_y=True), (16, 12, 10), G.spheres_3d(16, 12, 10, count=1))


@pytest.mark.parametrize("name", sorted(REFPIN_CASES))
def test_gpu_matches_the_reference_programs(name):
    """The fields of PixelFlow's own OpenMP programs, executed from their
    Fortran source (tests/golden/refpin_*.npz, see make_reference_pin.py),
    against the GPU step on the same settings and porosity: every field
    within 1e-12 relative L2 after the programs' few steps, max|div u|
    against the divergence the program writes within 1e-8 relative, and the
    drag program's force log (printed after every step) against pf_forces
    within 1e-10 of the largest component (the GPU sums in another order)."""
    s, shape, _, steps = refpin_inputs(name)
    ref = np.load(os.path.join(GOLDEN, f"refpin_{name}.npz"))
    dim = len(shape)
    fp, fv = [], []
    with Case(s, shape, ref["porosity"]) as c:
        c.initial_conditions()
        if "fp" in ref.files:
            for _ in range(steps):
                c.step(1)
                f = c.forces()
                fp.append(f["Fp"])
                fv.append(f["Fv"])
        else:
            c.step(steps)
        got = c.get_state()
        max_div, _ = c.norms()
    errs = errors(got, {f: ref[f] for f in fields(dim)}, dim)
    assert_each_field(errs, 1e-12)
    want = float(np.abs(ref["div"]).max())
    assert abs(max_div - want) <= 1e-8 * want, (max_div, want)
    if "fp" in ref.files:
        for got_f, want_f in ((np.array(fp), ref["fp"]), (np.array(fv), ref["fv"])):
            scale = np.abs(want_f).max(axis=1, keepdims=True)
            assert np.all(np.abs(got_f - want_f) <= 1e-10 * scale), (got_f, want_f)
