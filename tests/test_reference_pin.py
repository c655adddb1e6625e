"""The oracle pinned to the reference itself.

tests/golden/refpin_*.npz hold the fields PixelFlow's own OpenMP programs
compute (their Fortran source executed by tests/golden/fortran_subset.py,
gfortran plain-FP64 semantics, made by tests/golden/make_reference_pin.py):
the uniform 2D program on even and odd grids (the linear-index colour map's
odd-m shift included), the backstep program, the uniform 3D program on even
and odd grids, the air-condition program with its own wall table and two
others (set through its wall parameters), the drag
program, the uniform 2D program with its commented symmetry ("slip")
rows enabled, and the uniform 2D and 3D programs with the physical
parameters away from the template's defaults (inflow angle, second
viscosity, density, outlet pressure, no damping), with the divergence field
each program writes at the end
(output_divergent_2d/3d) and the drag program's force log after every step
(output_force_log_2d).  The C oracle (oracle/pf_oracle.c), given the same
settings and the porosity the program read, must reproduce every field, the
divergence and the force sums bit for bit.

The fixtures also hold every value the programs' VTK writers wrote for the
final state (output_paraview_temp_2d/_3d at istep_out, output_paraview_2d/_3d
at the end of the run), record by record: pixelflow_gb300.output.write_vtk,
given the program's fields, writes the same records, each value as f16.4."""
import os
import re

import numpy as np
import pytest

from oracle.oracle import OracleCase
from tests.golden.make_reference_pin import CASES, case_inputs

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(HERE, f"refpin_{name}.npz"))


def pinned_vtk_inputs(name):
    """(state, ghosted porosity, settings) the pin run's VTK writers saw:
    the program's final fields, its clamped porosity, and the settings with
    the centre offsets at 0, as the pin run set them."""
    s, shape, _, _ = case_inputs(name)
    ref = load(name)
    s = s.replace(center_x=0.0, center_y=0.0, center_z=0.0)
    state = {f: ref[f] for f in (("u", "v", "w", "p") if len(shape) == 3 else ("u", "v", "p"))}
    raw = ref["porosity"]
    por = np.zeros(tuple(x + 2 for x in raw.shape))
    por[tuple(slice(1, -1) for _ in raw.shape)] = np.where(raw > s.threshold, raw, s.threshold)
    return state, por, s


def check_vtk_records(text, vals, lens):
    """One line per record of the Fortran writer: a record of literal text
    only is a line without values; DIMENSIONS / POINTS / POINT_DATA carry the
    record's integers; every other line is the record's values as f16.4,
    each followed by one blank (format 3(f16.4,1x))."""
    lines = text.split("\n")
    assert lines[-1] == ""
    lines = lines[:-1]
    assert len(lines) == len(lens)
    off = 0
    for q, (line, n) in enumerate(zip(lines, lens)):
        rec = vals[off:off + n]
        off += n
        if n == 0:
            assert re.fullmatch(r"# vtk DataFile Version 3\.0|[23]D flow|[A-Za-z_ ]+", line), (q, line)
        elif line.startswith(("DIMENSIONS", "POINTS", "POINT_DATA")):
            assert [int(t) for t in re.findall(r"\d+", line)] == [int(x) for x in rec], (q, line, rec)
        else:
            assert line == "".join("%16.4f " % x for x in rec), (q, line, rec)
    assert off == len(vals)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_the_reference_bit_for_bit(name):
    s, shape, _, steps = case_inputs(name)
    ref = load(name)
    assert int(ref["steps"]) == steps
    o = OracleCase(s, shape, ref["porosity"])
    o.initialize()
    fp, fv = [], []
    for _ in range(steps):  # the drag program logs the forces after every step
        o.step(1)
        a, b = o.forces()
        fp.append(a[:len(shape)])
        fv.append(b[:len(shape)])
    fields = ("u", "v", "w", "p") if len(shape) == 3 else ("u", "v", "p")
    for f in fields:
        got = getattr(o, f)
        assert got.shape == ref[f].shape, f
        assert np.array_equal(got, ref[f]), (f, float(np.abs(got - ref[f]).max()))
    mx, div = o.divergence_diag(want_field=True)
    interior = div[tuple(slice(1, -1) for _ in shape)]
    assert np.array_equal(interior, ref["div"]), float(np.abs(interior - ref["div"]).max())
    assert mx == np.abs(ref["div"]).max()
    if "fp" in ref.files:
        assert np.array_equal(np.array(fp), ref["fp"]) and np.array_equal(np.array(fv), ref["fv"])


def test_fixture_translator_reproduces_itself():
    """The translator is deterministic Python: when the reference is at hand
    (PF_REFERENCE_DIR), re-running one case gives the committed bits."""
    ref_dir = os.environ.get("PF_REFERENCE_DIR")
    if not ref_dir or not os.path.isdir(ref_dir):
        pytest.skip("PF_REFERENCE_DIR not set to a checkout of the reference")
    from tests.golden.make_reference_pin import run_reference
    _, _, _, _, out = run_reference(ref_dir, "uniform2d_9x8")
    ref = load("uniform2d_9x8")
    assert set(out) == set(ref.files) - {"porosity", "steps"}
    for f, a in out.items():
        assert np.array_equal(a, ref[f]), f


@pytest.mark.parametrize("name", sorted(CASES))
def test_vtk_writer_reproduces_the_reference_records(name, tmp_path):
    from pixelflow_gb300.output import write_vtk
    ref = load(name)
    state, por, s = pinned_vtk_inputs(name)
    for final, key in ((False, "vtk_temp"), (True, "vtk_final")):
        path = str(tmp_path / f"{key}.vtk")
        write_vtk(path, state, por, s, final=final)
        check_vtk_records(open(path).read(), ref[key + "_vals"], ref[key + "_lens"])
