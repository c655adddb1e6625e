"""Host-side logic on CPU: namelist and porosity-file readers, the C-ABI
library's exports and its argument checks (no kernel is launched)."""
import ctypes
import os
import re
import zipfile

import numpy as np
import pytest

from pixelflow_gb300 import config as C
from pixelflow_gb300 import geometry as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pixelflow_gpu.h")

TEMPLATE = """!********************************************
&physical
!--- Kinematic viscosity coefficient [m2/s]
xnue = 0.001000
xlambda = 0.000000
density = 1.000000
width   = 1.0000000
height  = 1.0000000
depth   = 1.0000000
time = 1.000000
inlet_velocity = 0.100000
outlet_pressure = 0.000000
AoA = 0.000000
/
&file_control
istep_out = 1001
/
&grid_control
istep_max = 100
/
&porosity_control
thickness = 1.500000
threshold = 1.0e-6
radius = 0.100000
center_x = 0.500000
center_y = 0.500000
center_z = 0.500000
/
&calculation_method
nonslip = .true.
/
&directory_control
output_folder   = "output"
csv_file        = "data/porosity.csv"
/
&solver_control
iter_max        = 100
relux_factor    = 1.700000
/
"""


def test_read_template_controldict(tmp_path):
    p = tmp_path / "controlDict.txt"
    p.write_text(TEMPLATE)
    s = C.read_settings(str(p))
    assert s.xnue == 1e-3 and s.inlet_velocity == 0.1 and s.aoa == 0.0
    assert s.istep_max == 100 and s.iter_max == 100 and s.relux_factor == 1.7
    assert s.nonslip is True and s.csv_file == "data/porosity.csv" and s.threshold == 1e-6
    assert s.precision == "fp64"


def test_gpu_control_group_and_roundtrip(tmp_path):
    s = G.settings_spheres_3d(precision="mixed", outer_max=3, inner_sweeps=20)
    p = tmp_path / "c.txt"
    C.write_settings(str(p), s, gpu_group=True)
    r = C.read_settings(str(p))
    assert r == s


def test_missing_group_is_an_error(tmp_path):
    p = tmp_path / "c.txt"
    p.write_text(TEMPLATE.replace("&solver_control", "&solver_controlx"))
    with pytest.raises(ValueError):
        C.read_settings(str(p))


def test_porosity_csv_roundtrip(tmp_path):
    vals = G.spheres_3d(7, 5, 4, count=2, seed=3)
    p = tmp_path / "poro.csv"
    C.write_porosity_csv(str(p), vals)
    shape, back = C.read_porosity_csv(str(p))
    assert shape == (7, 5, 4)
    np.testing.assert_allclose(back, vals, atol=1e-10)
    v2 = G.cylinder_2d(9, 6)
    C.write_porosity_csv(str(p), v2)
    shape, back = C.read_porosity_csv(str(p))
    assert shape == (9, 6)
    np.testing.assert_allclose(back, v2, atol=1e-10)


# The reference's own example project (test/cylinder-2d.zip of PixelFlow):
# PF_REFERENCE_CYLINDER_ZIP names its path; the test is skipped without it.
REF_ZIP = os.environ.get("PF_REFERENCE_CYLINDER_ZIP", "")


@pytest.mark.skipif(not REF_ZIP or not os.path.exists(REF_ZIP),
                    reason="PF_REFERENCE_CYLINDER_ZIP not set to the reference's test/cylinder-2d.zip")
def test_reference_cylinder_fixture_parses(tmp_path):
    with zipfile.ZipFile(REF_ZIP) as z:
        z.extractall(tmp_path)
    proj = tmp_path / "cylinder-2d"
    s = C.read_settings(str(proj / "config" / "controlDict.txt"))
    assert s.istep_max == 5000 and s.width == 1.023 and s.thickness == 1.5
    shape, vals = C.read_porosity_csv(str(proj / s.csv_file))
    assert shape == (1024, 512) and vals.min() >= 0 and vals.max() <= 1


def _declared_symbols():
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(pf_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from pixelflow_gb300 import _lib
    L = _lib.load()
    declared = _declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert set(_lib.exported_symbols()) >= set(declared)
    assert L.pf_abi_version() == 3


def test_invalid_arguments_fail_before_any_device_work():
    from pixelflow_gb300 import _lib
    L = _lib.load()
    s = G.settings_cylinder_2d()
    from pixelflow_gb300.solver import make_options, make_params
    vals = np.ones((4, 4))
    h = ctypes.c_void_p()
    for bad in (dict(dim=4), dict(m=2), dict(n=1)):
        prm = make_params(s, (4, 4))
        for k, v in bad.items():
            setattr(prm, k, v)
        rc = L.pf_create(ctypes.byref(prm), ctypes.byref(make_options(s)), vals.ctypes.data_as(ctypes.c_void_p),
                         ctypes.byref(h))
        assert rc == -1
        assert L.pf_last_error()
    assert L.pf_create(None, None, None, ctypes.byref(h)) == -1
    assert L.pf_destroy(None) == -1
    assert L.pf_step(None, 1) == -1
    assert L.pf_step_host(None, None, None, None, None, None, None, None, None, 6, 6) == -1
    assert L.pf_strerror(-4) == b"non-finite values in the fields"


def test_step_host_schedule_respects_every_dependency():
    """pf_step_host's slab schedule, replayed on the CPU for every plane count
    up to 300: each divergence plane k finds planes k-1 .. k+1 copied, each
    predictor plane k finds them copied and the divergence of k-1 .. k+1 done
    (plane l: l-1, l and 1; plane 1, issued last: l, 1 and 2), and every
    interior plane is covered exactly once by each kernel."""
    from pixelflow_gb300 import _lib
    L = _lib.load()
    for l in range(3, 301):
        n = L.pf_debug_step_host_plan(l, None, 0)
        assert 1 <= n <= 16
        buf = (ctypes.c_int * (6 * n))()
        assert L.pf_debug_step_host_plan(l, ctypes.cast(buf, ctypes.c_void_p), n) == n
        copied, div, pred = set(), [], []
        expect_k0 = 0
        for b in range(n):
            k0, k1, dlo, dhi, plo, phi = buf[6 * b: 6 * b + 6]
            assert k0 == expect_k0 and k1 >= k0
            expect_k0 = k1 + 1
            copied |= set(range(k0, k1 + 1))
            for k in range(dlo, dhi + 1):
                assert {k - 1, k, k + 1} <= copied
                div.append(k)
            done = set(div)
            for k in range(plo, phi + 1):
                assert k != 1
                assert {k - 1, k, k + 1} <= copied
                assert {k - 1, k, 1 if k == l else k + 1} <= done
                pred.append(k)
        assert expect_k0 == l + 2  # the slabs tile the l+2 planes
        pred.append(1)  # after the last slab
        assert {l, 1, 2} <= set(div)
        assert sorted(div) == list(range(1, l + 1))
        assert sorted(pred) == list(range(1, l + 1))
    assert L.pf_debug_step_host_plan(2, None, 0) == -1
