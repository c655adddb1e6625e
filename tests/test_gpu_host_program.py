"""The C++ host program (pixelflow_gb300/pf_run) on the GPU: a project
directory run through it gives the same VTK files (step 0 and every istep_out),
the same final state bit for bit, the same max|div u| and SOR error, and the
same force log after every step as the Python host (Case + run_with_output)
on the same library; a run split by --save-state / --restart equals the run
in one piece."""
import os
import re
import subprocess

import numpy as np
import pytest

from pixelflow_gb300 import buildlib
from pixelflow_gb300 import geometry as G
from pixelflow_gb300.output import run_with_output, vtk_path, write_vtk
from pixelflow_gb300.solver import Case
from tests.test_host_program import _project, read_state_file

pytestmark = pytest.mark.gpu


def _pf_run(root, *args):
    buildlib.build()
    r = subprocess.run([buildlib.HOST_BIN, "--project", root, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


CASES = {
    "2d-plain": (G.settings_cylinder_2d(iter_max=20, istep_max=7, istep_out=3), (48, 24),
                 lambda: G.cylinder_2d(48, 24, radius=0.15, cx=0.6, cy=0.5)),
    "3d-mixed": (G.settings_spheres_3d(iter_max=10, istep_max=4, istep_out=2, precision="mixed", outer_max=2,
                                       inner_sweeps=5), (16, 12, 10),
                 lambda: G.spheres_3d(16, 12, 10, spheres=np.array([[0.45, 0.5, 0.5, 0.25]]))),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_pf_run_matches_python_host(tmp_path, name):
    s, shape, make = CASES[name]
    root = _project(str(tmp_path / "proj"), s, porosity=make())
    final = str(tmp_path / "final.bin")
    out = _pf_run(root, "--save-state", final)
    m = re.search(r"# steps (\d+)  max\|div u\| (\S+)  SOR error (\S+)", out)
    assert m and int(m.group(1)) == s.istep_max, out

    py_dir = str(tmp_path / "py")
    os.makedirs(py_dir)
    with Case.from_project(root) as c:
        c.initial_conditions()
        write_vtk(vtk_path(py_dir, 0), c.get_state(), c.porosity(), c.settings)  # the step-0 file
        run_with_output(c, s.istep_max, s.istep_out, py_dir)
        want = c.get_state()
        porosity = c.porosity()
        max_div, sor_err = c.norms()
    got, istep = read_state_file(final)
    assert istep == s.istep_max
    for k in want:
        assert got[k].tobytes() == want[k].tobytes(), k
    assert float(m.group(2)) == max_div and float(m.group(3)) == sor_err

    written = sorted(f for f in os.listdir(os.path.join(root, s.output_folder)) if f.endswith(".vtk"))
    steps = [0] + list(range(s.istep_out, s.istep_max + 1, s.istep_out))
    assert written == sorted([os.path.basename(vtk_path("", k)) for k in steps] + ["output_paraview.vtk"])
    for k in steps:
        a = open(vtk_path(os.path.join(root, s.output_folder), k), "rb").read()
        b = open(vtk_path(py_dir, k), "rb").read()
        assert a == b, k
    # the final file: the same writer on the final state
    write_vtk(os.path.join(py_dir, "final.vtk"), want, porosity, s, final=True)
    assert open(os.path.join(root, s.output_folder, "output_paraview.vtk"), "rb").read() == \
        open(os.path.join(py_dir, "final.vtk"), "rb").read()


def test_pf_run_force_log_matches_pf_forces(tmp_path):
    """--force-log prints the drag program's force log after every step; the
    values equal Case.forces after the same steps (printed with 17 digits)."""
    s, shape, make = CASES["2d-plain"]
    s = s.replace(istep_max=5, istep_out=100)
    root = _project(str(tmp_path / "proj"), s, porosity=make())
    out = _pf_run(root, "--force-log", "--no-vtk")
    lines = [l for l in out.splitlines() if l.startswith("force ")]
    assert len(lines) == 5
    with Case.from_project(root) as c:
        c.initial_conditions()
        for istep, line in enumerate(lines, start=1):
            c.step(1)
            f = c.forces(radius=s.radius)
            rec = dict(kv.split("=") for kv in line.split()[1:])
            assert int(rec["istep"]) == istep
            assert [float(rec["Fpx"]), float(rec["Fpy"])] == list(f["Fp"])
            assert [float(rec["Fvx"]), float(rec["Fvy"])] == list(f["Fv"])
            assert [float(rec["Cx"]), float(rec["Cy"])] == [f["Cd"], f["Cl"]]
    assert not os.path.exists(os.path.join(root, s.output_folder))


@pytest.mark.parametrize("name", sorted(CASES))
def test_pf_run_restart_continues_bit_for_bit(tmp_path, name):
    s, shape, make = CASES[name]
    vals = make()
    whole = _project(str(tmp_path / "whole"), s, porosity=vals)
    split = _project(str(tmp_path / "split"), s, porosity=vals)
    _pf_run(whole, "--save-state", str(tmp_path / "whole.bin"))
    _pf_run(split, "--steps", "3", "--save-state", str(tmp_path / "part.bin"), "--no-vtk")
    assert read_state_file(str(tmp_path / "part.bin"))[1] == 3
    _pf_run(split, "--restart", str(tmp_path / "part.bin"), "--save-state", str(tmp_path / "split.bin"))
    a, ia = read_state_file(str(tmp_path / "whole.bin"))
    b, ib = read_state_file(str(tmp_path / "split.bin"))
    assert ia == ib == s.istep_max
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k
    # the restarted run writes the files of the steps after its first one
    after = [k for k in range(s.istep_out, s.istep_max + 1, s.istep_out) if k > 3]
    assert sorted(os.listdir(os.path.join(split, s.output_folder))) == \
        sorted([os.path.basename(vtk_path("", k)) for k in after] + ["output_paraview.vtk"])
    for k in after:
        assert open(vtk_path(os.path.join(whole, s.output_folder), k), "rb").read() == \
            open(vtk_path(os.path.join(split, s.output_folder), k), "rb").read(), k
