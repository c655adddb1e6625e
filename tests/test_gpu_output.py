"""Output at istep_out, the force log of the drag program, and checkpoint /
restart: asynchronous snapshots equal the synchronous state of their step,
the output loop writes the reference's files for the right steps, and a
restart continues bit for bit."""
import numpy as np
import pytest

from pixelflow_gb300 import geometry as G
from pixelflow_gb300._lib import PfError
from pixelflow_gb300.output import run_with_output, vtk_path, write_vtk
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


def _case(dim, precision="fp64"):
    if dim == 2:
        s = G.settings_cylinder_2d(iter_max=20, precision=precision)
        return s, (64, 32), G.cylinder_2d(64, 32, radius=0.2, cx=0.6, cy=0.5)
    s = G.settings_spheres_3d(iter_max=10, precision=precision)
    return s, (20, 18, 16), G.spheres_3d(20, 18, 16, count=3, seed=1)


def _same(a, b):
    return all(np.array_equal(a[k], b[k]) for k in a)


@pytest.mark.parametrize("dim", [2, 3])
def test_snapshot_is_the_state_of_its_step(dim):
    s, shape, vals = _case(dim)
    with Case(s, shape, vals) as a, Case(s, shape, vals) as b:
        a.initial_conditions()
        b.initial_conditions()
        a.step(5)
        a.snapshot_begin()
        with pytest.raises(PfError):
            a.snapshot_begin()  # one snapshot in flight
        a.step(3)  # enqueued while the copy runs
        snap = a.snapshot_wait()
        b.step(5)
        assert _same(snap, b.get_state())
        b.step(3)
        assert _same(a.get_state(), b.get_state())
        with pytest.raises(PfError):
            a.snapshot_wait()  # nothing in flight


def test_output_loop_writes_each_istep_out(tmp_path):
    s, shape, vals = _case(2)
    with Case(s, shape, vals) as a, Case(s, shape, vals) as b:
        a.initial_conditions()
        b.initial_conditions()
        log = run_with_output(a, 10, 4, str(tmp_path / "run"), forces_radius=None)
        assert log == []
        por = b.porosity()
        for istep in (4, 8):
            b.step(4)
            write_vtk(str(tmp_path / "want.vtk"), b.get_state(), por, s)
            got = open(vtk_path(str(tmp_path / "run"), istep)).read()
            assert got == open(tmp_path / "want.vtk").read(), istep
        assert not (tmp_path / "run" / "output_00010.vtk").exists()
        b.step(2)
        assert _same(a.get_state(), b.get_state())


def test_drag_program_force_log(tmp_path):
    s, shape, vals = _case(2)
    with Case(s, shape, vals) as a, Case(s, shape, vals) as b:
        a.initial_conditions()
        b.initial_conditions()
        log = run_with_output(a, 6, 3, str(tmp_path), forces_radius=0.2)
        assert [r["istep"] for r in log] == list(range(1, 7))
        for r in log:
            b.step(1)
            f = b.forces(radius=0.2)
            assert np.array_equal(r["F"], f["F"]) and r["Cd"] == f["Cd"] and r["Cl"] == f["Cl"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim", [2, 3])
def test_checkpoint_restart_is_bit_exact(dim, precision, tmp_path):
    s, shape, vals = _case(dim, precision)
    path = str(tmp_path / "ck.npz")
    with Case(s, shape, vals) as a:
        a.initial_conditions()
        a.step(6)
        a.save_checkpoint(path)
        a.step(4)
        want = a.get_state()
    with Case.from_checkpoint(path) as r:
        assert r.steps_done == 6 and r.settings == s
        r.step(4)
        assert _same(r.get_state(), want)
