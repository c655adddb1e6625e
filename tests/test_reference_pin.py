"""The oracle pinned to the reference itself.

tests/golden/refpin_*.npz hold the fields PixelFlow's own OpenMP programs
compute (their Fortran source executed by tests/golden/fortran_subset.py,
gfortran plain-FP64 semantics, made by tests/golden/make_reference_pin.py):
the uniform 2D program on even and odd grids (the linear-index colour map's
odd-m shift included), the backstep program, the uniform 3D program on even
and odd grids, the air-condition program with its own wall table and two
others (set through its wall parameters), the drag
program and the uniform 2D program with its commented symmetry ("slip")
rows enabled, with the divergence field each program writes at the end
(output_divergent_2d/3d) and the drag program's force log after every step
(output_force_log_2d).  The C oracle (oracle/pf_oracle.c), given the same
settings and the porosity the program read, must reproduce every field, the
divergence and the force sums bit for bit."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleCase
from tests.golden.make_reference_pin import CASES, case_inputs

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(HERE, f"refpin_{name}.npz"))


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
