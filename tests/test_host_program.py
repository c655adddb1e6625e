"""The C++ host program (pixelflow_gb300/pf_run, the reference's main program
over the C ABI) on the CPU: its controlDict and porosity-CSV readers against
the Python readers of pixelflow_gb300.config, its error behaviour, and its VTK
writer against pixelflow_gb300.output.write_vtk byte for byte.  No CUDA call
is made (--print-config and --vtk-from stop before any)."""
import dataclasses
import json
import os
import subprocess

import numpy as np
import pytest

from pixelflow_gb300 import buildlib
from pixelflow_gb300 import geometry as G
from pixelflow_gb300.config import Settings, read_porosity_csv, read_settings, write_porosity_csv, write_settings
from pixelflow_gb300.output import write_vtk


@pytest.fixture(scope="module")
def pf_run():
    buildlib.build()
    return buildlib.HOST_BIN


def _project(root, settings=None, text=None, porosity=None):
    os.makedirs(os.path.join(root, "config"), exist_ok=True)
    path = os.path.join(root, "config", "controlDict.txt")
    if text is not None:
        with open(path, "w") as f:
            f.write(text)
    else:
        write_settings(path, settings, gpu_group=True)
    if porosity is not None:
        csv = os.path.join(root, settings.csv_file if settings is not None else "data/porosity.csv")
        os.makedirs(os.path.dirname(csv), exist_ok=True)
        write_porosity_csv(csv, porosity)
    return root


def _run(binary, *args):
    return subprocess.run([binary, *args], capture_output=True, text=True, timeout=120)


def _config(binary, root):
    r = _run(binary, "--project", root, "--print-config")
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def _same_settings(got, s: Settings, shape):
    want = dataclasses.asdict(s)
    want["walls"] = list(s.walls) if s.walls is not None else None
    for k, v in want.items():
        assert k in got, k
        if isinstance(v, bool) or v is None or isinstance(v, (str, list)):
            assert got[k] == v, (k, got[k], v)
        else:
            assert float(got[k]) == float(v), (k, got[k], v)
    assert got["shape"] == list(shape)


SETTINGS = [
    G.settings_cylinder_2d(istep_max=37, istep_out=5, iter_max=12),
    G.settings_spheres_3d(precision="mixed", outer_max=2, inner_sweeps=9, dc_tol=1.5e-9, sweep_form="split",
                          fused_rows=4, fused_planes=64, sor_path="cells", track_sor_error=False),
    G.settings_spheres_3d(walls=(1, 0, 0, 0, 0, 2), aoa=12.5, xlambda=0.25, threshold=0.1),
    G.settings_cylinder_2d(inflow_porosity=True, slip_y=True, nonslip=False, output_folder="out/run 1",
                           csv_file="grid/poro.csv", density=998.2, time=3.0e-7),
]


@pytest.mark.parametrize("k", range(len(SETTINGS)))
def test_print_config_matches_python_reader(pf_run, tmp_path, k):
    s = SETTINGS[k]
    shape = (9, 7) if k in (0, 3) else (6, 5, 4)
    vals = np.random.default_rng(k).random(shape[::-1])
    root = _project(str(tmp_path), s, porosity=vals)
    py = read_settings(os.path.join(root, "config", "controlDict.txt"))
    _same_settings(_config(pf_run, root), py, shape)


NAMELIST = """! hand-written controlDict: comments, several members per line, commas,
! d exponents, logical spellings, quotes and a trailing slash on a member line
&physical
  xnue = 1.5d-3, xlambda=0.0 ,density = 2
  width = 2.0D0 height=1 depth=1.0e0   ! trailing comment
  time = .25, inlet_velocity = 1, outlet_pressure = -0.5, AoA = 3 /
&file_control istep_out = 4 /
&grid_control
istep_max = 12
/
&porosity_control
  thickness = 2.0, threshold = 1.0E-6, radius = 0.05
  center_x = 0.25, center_y = 0.5, center_z = 0.5
/
&calculation_method
  nonslip = .F.
/
&directory_control
  output_folder = 'results', csv_file = "data/porosity.csv"
/
&solver_control
  iter_max = 25, relux_factor = 1.6
/
&gpu_control
  precision = "mixed", walls = "", track_sor_error = t
/
"""


def test_quotes_hold_comment_and_slash_characters(pf_run, tmp_path):
    """`!` and `/` inside a quoted value are characters of the value; a `/`
    after it on the same line still ends the group."""
    text = NAMELIST.replace("""  output_folder = 'results', csv_file = "data/porosity.csv"
/""", """  output_folder = 'out/run!1', csv_file = "data/porosity.csv" /""")
    root = _project(str(tmp_path), text=text, porosity=np.full((5, 6), 0.5))
    py = read_settings(os.path.join(root, "config", "controlDict.txt"))
    assert py.output_folder == "out/run!1" and py.csv_file == "data/porosity.csv" and py.iter_max == 25
    _same_settings(_config(pf_run, root), py, (6, 5))


def test_print_config_hand_written_namelist(pf_run, tmp_path):
    root = _project(str(tmp_path), text=NAMELIST, porosity=np.full((5, 6), 0.5))
    py = read_settings(os.path.join(root, "config", "controlDict.txt"))
    assert py.xnue == 1.5e-3 and py.nonslip is False and py.output_folder == "results" and py.aoa == 3
    _same_settings(_config(pf_run, root), py, (6, 5))


@pytest.mark.parametrize("shape", [(7, 5), (5, 4, 3)])
def test_porosity_csv_any_record_order(pf_run, tmp_path, shape):
    """The records are stored at their own indices (grid.f90:42, :291), so a
    shuffled file gives the same array; the raw values match the Python
    reader bit for bit."""
    vals = np.random.default_rng(3).random(shape[::-1])
    root = _project(str(tmp_path), G.settings_spheres_3d(), porosity=vals)
    csv = os.path.join(root, "data", "porosity.csv")
    with open(csv) as f:
        head, *recs = f.read().splitlines()
    rng = np.random.default_rng(4)
    with open(csv, "w") as f:
        f.write("\n".join([head] + [recs[i] for i in rng.permutation(len(recs))]) + "\n")
    raw = str(tmp_path / "poro.bin")
    r = _run(pf_run, "--project", root, "--print-config", "--dump-porosity", raw)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(raw, dtype=np.float64)
    _, want = read_porosity_csv(csv)
    assert got.tobytes() == want.ravel().tobytes()
    assert json.loads(r.stdout)["shape"] == list(shape)


@pytest.mark.parametrize("text,needle", [
    (NAMELIST.replace("&grid_control\nistep_max = 12\n/\n", ""), "&grid_control missing"),
    (NAMELIST.replace("radius = 0.05", "radius = 0.05, diameter = 0.1"), "no member 'diameter'"),
    (NAMELIST.replace('walls = ""', 'walls = "1,0,3,0,0,2"'), "walls"),
    (NAMELIST.replace("iter_max = 25", "iter_max = 2x5"), "cannot parse"),
], ids=["missing-group", "unknown-member", "bad-walls", "bad-number"])
def test_bad_settings_are_errors(pf_run, tmp_path, text, needle):
    root = _project(str(tmp_path), text=text, porosity=np.full((5, 6), 0.5))
    r = _run(pf_run, "--project", root, "--print-config")
    assert r.returncode == 1 and needle in r.stderr, r.stderr


@pytest.mark.parametrize("edit,needle", [
    (lambda t: t + "6, 1, 1, 0.5\n", "index out of range"),  # i beyond m = 5
    (lambda t: t + "nan, 1, 1, 0.5\n", "index out of range"),
    (lambda t: t + "1, 1\n", "too few columns"),
    (lambda t: t + "1, 1, 1, x\n", "bad record"),
    (lambda t: "5,4000000,1\n" + t.split("\n", 1)[1], "out of range"),
    (lambda t: "1048576,1048576,1048576\n" + t.split("\n", 1)[1], "grid too large"),
], ids=["index", "nan-index", "columns", "value", "extent", "cells"])
def test_bad_porosity_file_is_an_error(pf_run, tmp_path, edit, needle):
    root = _project(str(tmp_path), G.settings_cylinder_2d(), porosity=np.full((4, 5), 0.5))
    csv = os.path.join(root, "data", "porosity.csv")
    text = open(csv).read()
    with open(csv, "w") as f:
        f.write(edit(text))
    r = _run(pf_run, "--project", root, "--print-config")
    assert r.returncode == 1 and needle in r.stderr, r.stderr


def write_state_file(path, state, shape, istep=0):
    """The host program's state file: "PFSTATE1", int32 dim, m, n, l, int64
    istep, then u, v, [w,] p in the Fortran order with ghosts (what
    --save-state writes)."""
    dim = len(shape)
    hdr = np.array([dim, shape[0], shape[1], shape[2] if dim == 3 else 1], dtype=np.int32)
    with open(path, "wb") as f:
        f.write(b"PFSTATE1" + hdr.tobytes() + np.array([istep], dtype=np.int64).tobytes())
        for k in ("u", "v", "w", "p") if dim == 3 else ("u", "v", "p"):
            f.write(np.ascontiguousarray(state[k], dtype=np.float64).tobytes())


def read_state_file(path):
    """(fields, istep) of a state file."""
    b = open(path, "rb").read()
    assert b[:8] == b"PFSTATE1"
    dim, m, n, l = np.frombuffer(b[8:24], dtype=np.int32)
    istep = int(np.frombuffer(b[24:32], dtype=np.int64)[0])
    shp = (n + 2, m + 2) if dim == 2 else (l + 2, n + 2, m + 2)
    keys = ("u", "v", "p") if dim == 2 else ("u", "v", "w", "p")
    arr = np.frombuffer(b[32:], dtype=np.float64).reshape((len(keys),) + shp)
    return {k: arr[q] for q, k in enumerate(keys)}, istep


def _padded_porosity(vals, threshold):
    """Interior porosity clamped as grid.f90:43 does, in a ghosted array."""
    out = np.zeros(tuple(x + 2 for x in vals.shape))
    inner = tuple(slice(1, x + 1) for x in vals.shape)
    out[inner] = np.where(vals > threshold, vals, threshold)
    return out


@pytest.mark.parametrize("final", [False, True])
@pytest.mark.parametrize("shape", [(11, 7), (6, 5, 4)])
def test_vtk_from_state_matches_python_writer(pf_run, tmp_path, shape, final):
    """--vtk-from writes the same bytes as write_vtk for the same state: the
    coordinates, the seven arrays and their f16.4 text, i fastest; with
    --final the end-of-run file output_paraview.vtk."""
    dim = len(shape)
    s = (G.settings_cylinder_2d(center_x=0.3, inlet_velocity=1.3) if dim == 2
         else G.settings_spheres_3d(center_x=0.5, center_y=0.25, center_z=0.75))
    rng = np.random.default_rng(11)
    vals = rng.random(shape[::-1]) * 1.2 - 0.1  # some values below the threshold
    root = _project(str(tmp_path), s, porosity=vals)
    ghosted = tuple(x + 2 for x in shape[::-1])
    state = {k: rng.standard_normal(ghosted) * 40.0 for k in (("u", "v", "p") if dim == 2 else ("u", "v", "w", "p"))}
    state["u"].flat[5] = -0.0
    state["p"].flat[7] = -1e-7  # prints as -0.0000
    write_state_file(str(tmp_path / "state.bin"), state, shape, istep=42)
    r = _run(pf_run, "--project", root, "--vtk-from", str(tmp_path / "state.bin"),  # the file's own step
             *(["--final"] if final else []))
    assert r.returncode == 0, r.stderr
    name = "output_paraview.vtk" if final else "output_00042.vtk"
    got = open(os.path.join(root, s.output_folder, name), "rb").read()
    s_py = read_settings(os.path.join(root, "config", "controlDict.txt"))
    _, raw = read_porosity_csv(os.path.join(root, s.csv_file))
    want_path = str(tmp_path / "want.vtk")
    write_vtk(want_path, state, _padded_porosity(raw, s_py.threshold), s_py, final=final)
    want = open(want_path, "rb").read()
    assert got == want


@pytest.mark.parametrize("threads", ["1", "3", "8"])
def test_vtk_from_threads_give_the_same_bytes(pf_run, tmp_path, threads):
    """A grid of several formatting blocks (90,000 points, blocks of 65,536
    per thread): the text equals the Python writer's for any thread count."""
    shape = (50, 45, 40)
    s = G.settings_spheres_3d(center_x=0.1)
    rng = np.random.default_rng(5)
    vals = rng.random(shape[::-1])
    root = _project(str(tmp_path), s, porosity=vals)
    state = {k: rng.standard_normal(tuple(x + 2 for x in shape[::-1])) for k in ("u", "v", "w", "p")}
    write_state_file(str(tmp_path / "state.bin"), state, shape, istep=7)
    r = subprocess.run([pf_run, "--project", root, "--vtk-from", str(tmp_path / "state.bin")],
                       capture_output=True, text=True, timeout=300, env={**os.environ, "PF_RUN_THREADS": threads})
    assert r.returncode == 0, r.stderr
    got = open(os.path.join(root, s.output_folder, "output_00007.vtk"), "rb").read()
    _, raw = read_porosity_csv(os.path.join(root, s.csv_file))
    write_vtk(str(tmp_path / "want.vtk"), state, _padded_porosity(raw, s.threshold), read_settings(
        os.path.join(root, "config", "controlDict.txt")))
    assert got == open(tmp_path / "want.vtk", "rb").read()


def test_state_file_round_trip(tmp_path):
    st = {k: np.random.default_rng(1).random((6, 7, 8)) for k in ("u", "v", "w", "p")}
    write_state_file(str(tmp_path / "s.bin"), st, (6, 5, 4), istep=17)
    back, istep = read_state_file(str(tmp_path / "s.bin"))
    assert istep == 17 and all(np.array_equal(back[k], st[k]) for k in st)


def test_state_file_of_another_grid_is_rejected(pf_run, tmp_path):
    root = _project(str(tmp_path), G.settings_spheres_3d(), porosity=np.full((4, 5, 7), 0.5))  # m, n, l = 7, 5, 4
    st = {k: np.zeros((6, 7, 8)) for k in ("u", "v", "w", "p")}
    write_state_file(str(tmp_path / "s.bin"), st, (6, 5, 4))  # m = 6
    r = _run(pf_run, "--project", root, "--vtk-from", str(tmp_path / "s.bin"))
    assert r.returncode == 1 and "does not match" in r.stderr, r.stderr
    with open(tmp_path / "s.bin", "ab") as f:
        f.write(b"\0")
    r = _run(pf_run, "--project", root, "--restart", str(tmp_path / "s.bin"))
    assert r.returncode == 1 and "size does not match" in r.stderr, r.stderr


# The reference's own example project (test/cylinder-2d.zip of PixelFlow):
# PF_REFERENCE_CYLINDER_ZIP names its path; the test is skipped without it.
REF_ZIP = os.environ.get("PF_REFERENCE_CYLINDER_ZIP", "")


@pytest.mark.skipif(not REF_ZIP or not os.path.exists(REF_ZIP),
                    reason="PF_REFERENCE_CYLINDER_ZIP not set to the reference's test/cylinder-2d.zip")
def test_reference_cylinder_project_reads_as_in_python(pf_run, tmp_path):
    """The reference's example project, its controlDict and 1024 x 512
    porosity file as shipped: the same settings and values bit for bit."""
    import zipfile
    with zipfile.ZipFile(REF_ZIP) as z:
        z.extractall(tmp_path)
    proj = str(tmp_path / "cylinder-2d")
    raw = str(tmp_path / "poro.bin")
    r = _run(pf_run, "--project", proj, "--print-config", "--dump-porosity", raw)
    assert r.returncode == 0, r.stderr
    py = read_settings(os.path.join(proj, "config", "controlDict.txt"))
    shape, vals = read_porosity_csv(os.path.join(proj, py.csv_file))
    _same_settings(json.loads(r.stdout), py, shape)
    assert np.fromfile(raw, dtype=np.float64).tobytes() == vals.ravel().tobytes()


def _refpin_cases():
    from tests.golden.make_reference_pin import CASES
    return sorted(CASES)


@pytest.mark.parametrize("name", _refpin_cases())
def test_vtk_from_reproduces_the_reference_records(pf_run, tmp_path, name):
    """The host program's VTK writer against the records the reference's own
    writers produced for the final state of each pinned program run
    (tests/golden/refpin_*.npz): the istep_out file and, with --final, the
    end-of-run file."""
    from tests.test_reference_pin import check_vtk_records, load, pinned_vtk_inputs
    ref = load(name)
    state, _, s = pinned_vtk_inputs(name)
    shape = tuple(reversed(ref["porosity"].shape))
    root = _project(str(tmp_path), s, porosity=ref["porosity"])
    write_state_file(str(tmp_path / "state.bin"), state, shape, istep=int(ref["steps"]))
    for final, key in ((False, "vtk_temp"), (True, "vtk_final")):
        r = _run(pf_run, "--project", root, "--vtk-from", str(tmp_path / "state.bin"), *(["--final"] if final else []))
        assert r.returncode == 0, r.stderr
        out = os.path.join(root, s.output_folder,
                           "output_paraview.vtk" if final else "output_%05d.vtk" % int(ref["steps"]))
        check_vtk_records(open(out).read(), ref[key + "_vals"], ref[key + "_lens"])


@pytest.mark.parametrize("args,needle", [
    (["--steps", "ten"], "--steps needs an integer"),
    (["--steps", "-3"], "--steps out of range"),
    (["--device", "99999999999"], "--device out of range"),
    (["--frobnicate"], "unknown argument"),
    (["--steps"], "missing value after --steps"),
])
def test_bad_arguments_are_errors(pf_run, tmp_path, args, needle):
    root = _project(str(tmp_path), G.settings_cylinder_2d(), porosity=np.full((4, 5), 0.5))
    r = _run(pf_run, "--project", root, *args)
    assert r.returncode == 1 and needle in r.stderr, r.stderr


# The reference's project template (template/config/controlDict.txt of
# PixelFlow): PF_REFERENCE_DIR names a checkout; skipped without it.
REF_DIR = os.environ.get("PF_REFERENCE_DIR", "")


@pytest.mark.skipif(not REF_DIR or not os.path.isfile(os.path.join(REF_DIR, "template", "config", "controlDict.txt")),
                    reason="PF_REFERENCE_DIR not set to a checkout of the reference")
def test_template_controldict_gives_the_defaults(pf_run, tmp_path):
    """The template's namelists read as the Settings defaults, in both
    readers (the defaults the readers fall back on are the template's)."""
    import shutil
    os.makedirs(tmp_path / "config")
    shutil.copy(os.path.join(REF_DIR, "template", "config", "controlDict.txt"), tmp_path / "config")
    root = _project(str(tmp_path), porosity=None, text=open(tmp_path / "config" / "controlDict.txt").read())
    csv = os.path.join(root, "data", "porosity.csv")
    os.makedirs(os.path.dirname(csv))
    write_porosity_csv(csv, np.full((4, 5), 0.5))
    py = read_settings(os.path.join(root, "config", "controlDict.txt"))
    assert py == Settings()
    _same_settings(_config(pf_run, root), Settings(), (5, 4))


def test_porosity_csv_parsed_on_threads_keeps_file_order(pf_run, tmp_path):
    """A file of several megabytes is parsed on several threads: shuffled
    records land at their own indices, a cell listed twice keeps its last
    value, and of two bad lines the first one in the file is reported."""
    shape = (60, 60, 60)
    vals = np.random.default_rng(8).random(shape[::-1])
    root = _project(str(tmp_path), G.settings_spheres_3d(), porosity=vals)
    csv = os.path.join(root, "data", "porosity.csv")
    with open(csv) as f:
        head, *recs = f.read().splitlines()
    order = np.random.default_rng(9).permutation(len(recs))
    lines = [head] + [recs[i] for i in order] + ["1, 1, 1, 0.25"]  # listed twice: the last value counts
    with open(csv, "w") as f:
        f.write("\n".join(lines) + "\n")
    want = vals.copy()
    want[0, 0, 0] = 0.25
    raw = str(tmp_path / "poro.bin")
    env = {**os.environ, "PF_RUN_THREADS": "4"}
    r = subprocess.run([pf_run, "--project", root, "--print-config", "--dump-porosity", raw],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(raw, dtype=np.float64)
    assert got[0] == 0.25 and np.allclose(got, want.ravel(), rtol=0, atol=1e-10)
    _, py = read_porosity_csv(csv)
    assert got.tobytes() == py.ravel().tobytes()
    bad = list(lines)
    bad[len(bad) // 3] = "1, 2, x, 0.5"
    bad[len(bad) - 5] = "1, 2, 3"
    with open(csv, "w") as f:
        f.write("\n".join(bad) + "\n")
    r = subprocess.run([pf_run, "--project", root, "--print-config"], capture_output=True, text=True, timeout=300,
                       env=env)
    assert r.returncode == 1 and "bad record '1, 2, x, 0.5'" in r.stderr, r.stderr
