"""The air-condition program (3D, wall table on all six faces, non-periodic
ghosts; ibm_3d_air_condition_omp_cpu.f90) on the GPU against the oracle."""
import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300._lib import PfError
from pixelflow_gb300.solver import Case
from oracle.oracle import OracleCase
from tests.conftest import rel_l2, rel_vel

pytestmark = pytest.mark.gpu

AIR_CONDITION_TABLE = (1, 0, 0, 0, 0, 2)


def _room(shape, table=AIR_CONDITION_TABLE, iters=20):
    m, n, l = shape
    s = G.settings_spheres_3d(iter_max=iters, walls=table, inlet_velocity=0.5)
    vals = G.spheres_3d(m, n, l, spheres=np.array([[0.5, 0.5, 0.4, 0.2]]))
    vals[-1, : n // 2, : m // 2] = 0.05
    vals[:, 0, m // 2:] = 0.05
    return s, vals


def _errs(got, ref):
    r = {f: getattr(ref, f) for f in ("u", "v", "w", "p")}
    return {"vel": rel_vel(got, r, 3), "p": rel_l2(got["p"], r["p"])}


@pytest.mark.parametrize("shape", [(24, 20, 16), (23, 21, 17)])
@pytest.mark.parametrize("table", [AIR_CONDITION_TABLE, (2, 1, 0, 1, 2, 0), (0, 2, 2, 0, 1, 1)])
def test_air_condition_parity(shape, table):
    s, vals = _room(shape, table)
    ref = OracleCase(s, shape, vals)
    ref.initialize()
    with Case(s, shape, vals) as c:
        assert np.array_equal(c.porosity(), ref.poro)
        c.initial_conditions()
        st0 = c.get_state()
        for f in ("u", "v", "w", "p"):
            assert np.array_equal(st0[f], getattr(ref, f)), ("initial + boundary", f)
        c.step(12)
        got = c.get_state()
        max_div, sor_err = c.norms()
    e_ref = ref.step(12)
    e = _errs(got, ref)
    assert e["vel"] < 1e-11 and e["p"] < 1e-11, e
    assert abs(sor_err - e_ref) <= 1e-8 * abs(e_ref)
    assert abs(max_div - ref.divergence_diag()) <= 1e-8 * ref.divergence_diag()


def test_air_condition_from_shapes_and_restrictions():
    shape = (20, 18, 16)
    s, vals = _room(shape)
    sph = [(0.5, 0.5, 0.4, 0.2)]
    with Case.from_shapes(s, shape, sph) as c:
        por = c.porosity()
    want = G.spheres_3d(*shape, spheres=np.array(sph))
    ref = OracleCase(s, shape, want)
    assert np.allclose(por, ref.poro, rtol=0, atol=1e-12)
    with pytest.raises(PfError):
        Case(s.replace(precision="mixed"), shape, vals)
    with pytest.raises(PfError):
        Case(G.settings_cylinder_2d(walls=AIR_CONDITION_TABLE), (16, 8), np.ones((8, 16)))
