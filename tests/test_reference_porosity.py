"""Porosity ingest pinned to the reference's own preprocessing code.

tests/golden/porosity_ref_{2d,3d}.csv were written by the reference's
porosity writer (tools/output/output_porosity.py) from porosity computed by
the reference's cylinder tool (tools/cylinder/make_porosity_2d_cylinder.py:
porosity_func) on the seeded distance fields kept in porosity_ref.npz
(generated by tests/golden/make_reference_porosity.py, which runs that code
unchanged).  Checked here: the reader returns the written values, this
repository's writer produces the same bytes from them, and the geometry's
tanh mapping equals the tool's."""
import os

import numpy as np

from pixelflow_gb300 import config as C
from pixelflow_gb300 import geometry as G

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF = np.load(os.path.join(HERE, "porosity_ref.npz"))


def _as_ours(data):
    """The tools index data[i-1, j-1(, k-1)]; this repository [(k-1,) j-1, i-1]."""
    return np.ascontiguousarray(data.T)


def test_reader_returns_the_reference_writer_values():
    shape, vals = C.read_porosity_csv(os.path.join(HERE, "porosity_ref_2d.csv"))
    assert shape == (14, 9)
    np.testing.assert_allclose(vals, _as_ours(REF["por2"]), rtol=0, atol=5e-11)
    shape, vals = C.read_porosity_csv(os.path.join(HERE, "porosity_ref_3d.csv"))
    assert shape == (6, 5, 4)
    np.testing.assert_allclose(vals, _as_ours(REF["por3"]), rtol=0, atol=5e-11)


def test_writer_bytes_equal_the_reference_writer(tmp_path):
    for name, key in (("porosity_ref_2d.csv", "por2"), ("porosity_ref_3d.csv", "por3")):
        out = tmp_path / name
        C.write_porosity_csv(str(out), _as_ours(REF[key]))
        with open(os.path.join(HERE, name), "rb") as f:
            ref = f.read()
        assert out.read_bytes() == ref, name


def test_tanh_mapping_equals_the_reference_tool():
    """geometry.tanh_porosity(sdf, edge, dx) takes the distance in length
    units and the edge in cells; the tool's porosity_func takes both in
    cells.  With dx = 1 the two are the same expression."""
    t = float(REF["thickness"])
    for sdf, por in ((REF["sdf2"], REF["por2"]), (REF["sdf3"], REF["por3"])):
        np.testing.assert_array_equal(G.tanh_porosity(sdf, t, 1.0), por)
        dx = 0.01
        np.testing.assert_allclose(G.tanh_porosity(sdf * dx, t, dx), por, rtol=0, atol=4e-16)
