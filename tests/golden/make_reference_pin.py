"""Golden vectors made by the reference itself: PixelFlow's OpenMP programs
(src/omp_parallel/*.f90 and lib/global.f90, lib/grid.f90, lib/output.f90),
executed from their own source text by tests/golden/fortran_subset.py with
gfortran's plain-FP64 semantics, on small grids for a few steps.

Each case writes tests/golden/refpin_<name>.npz with the porosity values the
program read (its CSV, written by this repository's writer, which produces
the reference writer's bytes), the settings, the fields u, v, [w,] p the
program holds after `steps` time steps (ghost layers included,
[(k,) j, i] order), the porosity-weighted divergence field `div`
([(k,) j, i], interior only) that output_divergent_2d/3d writes at the end
of the run, for the drag program the pressure and friction force sums
`fp`, `fv` (one row per step) that output_force_log_2d prints after every
step, and the records of the two VTK writers on the final state: the
istep_out file of the last step (output_paraview_temp_2d/_3d) and the
end-of-run file (output_paraview_2d/_3d), as `vtk_temp_vals`/`_lens` and
`vtk_final_vals`/`_lens` (every value written, in order, and the number of
values of each record; a record of literal text only has none).  The runs replace only what is not arithmetic: the namelist reader
(`read_settings` returns the settings below), the other file writers,
`get_now_time` and `system`; the static array sizes md, nd, ld are shrunk to
the grid (they size storage only).  The main program, the grid set-up (which
reads the CSV with list-directed input), the initial and boundary
conditions, solve_p, the matrix edits, the SOR, the divergence output and
the force log and the VTK writers run unchanged (istep_out = the run's
steps); their `write` statements are recorded as values rather than
formatted.  The slip cases run the uniform 2D program with the
symmetry rows its source keeps commented out enabled (enable_slip), the
option this repository exposes as `slip_y`.

Run from the repository root (the reference is not needed afterwards):

    PF_REFERENCE_DIR=<reference checkout> python -m tests.golden.make_reference_pin [case ...]
"""
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from pixelflow_gb300 import config as C  # noqa: E402
from pixelflow_gb300 import geometry as G  # noqa: E402
from tests.golden.fortran_subset import Program  # noqa: E402

AIR_CONDITION_TABLE = (1, 0, 0, 0, 0, 2)  # top, bottom, east, west, north, south
# other wall tables of the air-condition program, set through its integer
# parameters top_wall .. north_wall (0 wall, 1 inlet, 2 outlet); the second
# has outlets on the top (its bb starts from plane 1) and west faces and
# inlets on the east and north faces
WALL_TABLES = {"aircon3d_bottom_in_east_out_8x7x6": (0, 1, 2, 0, 0, 0),
               "aircon3d_mixed_faces_9x7x6": (2, 0, 1, 2, 1, 0)}
WALL_PARAMS = ("top_wall", "bottom_wall", "east_wall", "west_wall", "north_wall", "south_wall")

# name -> (program file, dim, shape, settings builder, steps)
CASES = {
    "uniform2d_12x8": ("ibm_2d_uniform_omp_cpu.f90", (12, 8), "cyl", 3),
    "uniform2d_13x9": ("ibm_2d_uniform_omp_cpu.f90", (13, 9), "cyl", 3),
    "uniform2d_9x8": ("ibm_2d_uniform_omp_cpu.f90", (9, 8), "cyl", 3),
    "backstep2d_12x8": ("ibm_2d_backstep_omp_cpu.f90", (12, 8), "step", 3),
    "uniform3d_8x6x5": ("ibm_3d_uniform_omp_cpu.f90", (8, 6, 5), "sph", 3),
    "uniform3d_7x6x5": ("ibm_3d_uniform_omp_cpu.f90", (7, 6, 5), "sph", 3),
    "uniform3d_8x7x6": ("ibm_3d_uniform_omp_cpu.f90", (8, 7, 6), "sph", 2),
    "aircon3d_8x7x6": ("ibm_3d_air_condition_omp_cpu.f90", (8, 7, 6), "room", 3),
    "aircon3d_bottom_in_east_out_8x7x6": ("ibm_3d_air_condition_omp_cpu.f90", (8, 7, 6), "room", 3),
    "aircon3d_mixed_faces_9x7x6": ("ibm_3d_air_condition_omp_cpu.f90", (9, 7, 6), "room", 3),
    "drag2d_12x8": ("ibm_2d_drag_omp_cpu.f90", (12, 8), "cyl", 4),
    # the uniform 2D program with its commented symmetry ("slip") rows enabled
    "slip2d_12x8": ("ibm_2d_uniform_omp_cpu.f90", (12, 8), "cyl_slip", 3),
    "slip2d_13x9": ("ibm_2d_uniform_omp_cpu.f90", (13, 9), "cyl_slip", 3),
    # the physical parameters away from the template's defaults: an inflow
    # angle (2D: AoA/180*pi in boundary and initial_conditions; 3D: AoA/1300*pi
    # in boundary, AoA/360*pi in initial_conditions), the second viscosity,
    # density, outlet pressure, and (2D) no damping term
    "physics2d_12x8": ("ibm_2d_uniform_omp_cpu.f90", (12, 8), "cyl_phys", 3),
    "physics3d_8x6x5": ("ibm_3d_uniform_omp_cpu.f90", (8, 6, 5), "sph_phys", 3),
}
PHYSICS = {"cyl_phys": dict(aoa=10.0, xlambda=0.3, density=1.3, outlet_pressure=0.25, nonslip=False),
           "sph_phys": dict(aoa=25.0, xlambda=0.2, density=0.8, outlet_pressure=-0.5)}

# The commented blocks that make up the 2D symmetry option, by the comment
# line that heads each (ibm_2d_uniform_omp_cpu.f90: boundrary_matrix :440-450,
# boundary :512-526); enable_slip() removes the leading "!" of the block's
# statements.
SLIP_HEADS = ("! symmetry or wall (dp/dy=0. at j=1)", "! symmetry or wall  (dp/dy=0. at j=n)",
              "! option: symmetry (du/dy=0., v=0., dp/dy=0. at j=1)",
              "! option: symmetry  (du/dy=0., v=0., dp/dy=0. at j=n)")

# output routines that run as written (their records are captured)
INTERPRETED = ("output_divergent_2d", "output_divergent_3d", "output_force_log_2d", "output_force_log_3d",
               "output_paraview_temp_2d", "output_paraview_temp_3d", "output_paraview_2d", "output_paraview_3d")
VTK_TEMP_UNIT, VTK_FINAL_UNIT = 65, 50  # output.f90:441, :994 and :323, :816

NAMES = ["xnue", "xlambda", "density", "width", "height", "depth", "time", "inlet_velocity", "outlet_pressure",
         "aoa", "istep_max", "istep_out", "thickness", "threshold", "radius", "center_x", "center_y", "center_z",
         "nonslip", "output_folder", "csv_file", "iter_max", "relux_factor"]


def case_inputs(name):
    """(settings, shape, porosity values before the CSV round trip, steps)."""
    prog, shape, kind, steps = CASES[name]
    if kind in ("cyl", "step", "cyl_slip", "cyl_phys"):
        m, n = shape
        s = G.settings_cylinder_2d(iter_max=7, slip_y=kind == "cyl_slip", **PHYSICS.get(kind, {}))
        vals = G.cylinder_2d(m, n, radius=0.2, cx=0.6, cy=0.45)
        if kind == "step":  # an obstacle across the inlet: a non-uniform inflow profile
            vals = np.minimum(vals, G.cylinder_2d(m, n, radius=0.3, cx=0.0, cy=0.3))
            s = s.replace(inflow_porosity=True)
        dt = 2e-4
    else:
        m, n, l = shape
        if kind == "room":
            s = G.settings_spheres_3d(iter_max=5, walls=WALL_TABLES.get(name, AIR_CONDITION_TABLE),
                                      inlet_velocity=0.5)
            vals = G.spheres_3d(m, n, l, spheres=np.array([[0.5, 0.5, 0.4, 0.2]]))
            vals[-1, : n // 2, : m // 2] = 0.05
            vals[:, 0, m // 2:] = 0.05
        else:
            s = G.settings_spheres_3d(iter_max=5, **PHYSICS.get(kind, {}))
            vals = G.spheres_3d(m, n, l, spheres=np.array([[0.4, 0.5, 0.5, 0.2], [0.7, 0.3, 0.6, 0.15]]))
        dt = 1e-4
    # time / istep_max is dt for the program and the oracle alike
    s = s.replace(time=dt * steps, istep_max=steps)
    return s, shape, vals, steps


def enable_slip(text):
    """The program text with the commented statements under each SLIP_HEADS
    comment enabled (up to the next line that is not a commented statement)."""
    lines = text.splitlines()
    out, on, found = [], False, 0
    for ln in lines:
        st = ln.strip()
        if any(st.startswith(h) for h in SLIP_HEADS):
            on, found = True, found + 1
            out.append(ln)
            continue
        if on and st.startswith("!") and not st.startswith("! -") and len(st) > 1:
            out.append(ln.replace("!", "", 1))
            continue
        on = False
        out.append(ln)
    assert found == len(SLIP_HEADS), found
    return "\n".join(out) + "\n"


def run_reference(ref_dir, name):
    prog, shape, kind, steps = CASES[name]
    s, shape, vals, steps = case_inputs(name)
    src = os.path.join(ref_dir, "src", "omp_parallel")
    files = [os.path.join(src, "lib", f) for f in ("global.f90", "grid.f90", "output.f90")]
    files.append(os.path.join(src, prog))
    texts = [open(f).read() for f in files]
    if kind == "cyl_slip":
        texts[-1] = enable_slip(texts[-1])
    with tempfile.TemporaryDirectory() as tmp:
        csv = os.path.join(tmp, "porosity.csv")
        C.write_porosity_csv(csv, vals)
        csv_text = open(csv).read()
        _, vals_read = C.read_porosity_csv(csv)
    settings = dict(xnue=s.xnue, xlambda=s.xlambda, density=s.density, width=s.width, height=s.height,
                    depth=s.depth, time=s.time, inlet_velocity=s.inlet_velocity, outlet_pressure=s.outlet_pressure,
                    aoa=s.aoa, istep_max=int(s.istep_max), istep_out=int(s.istep_max), thickness=s.thickness,
                    threshold=s.threshold, radius=s.radius, center_x=0.0, center_y=0.0, center_z=0.0,
                    nonslip=bool(s.nonslip), output_folder="out", csv_file="porosity.csv",
                    iter_max=int(s.iter_max), relux_factor=s.relux_factor)

    def read_settings(P, *args):
        return [settings[k] for k in NAMES]

    def noop(P, *args):
        return None

    overrides = _sizes(shape)
    if kind == "room":
        overrides.update(zip(WALL_PARAMS, WALL_TABLES.get(name, AIR_CONDITION_TABLE)))
    called = set(re.findall(r"\bcall\s+(\w+)", "\n".join(t.lower() for t in texts)))
    probe = Program(texts, overrides=overrides)
    stubs = {nm: noop for nm in called - set(probe.subs)}
    stubs.update({nm: noop for nm in called
                  if (nm.startswith("output_") and nm not in INTERPRETED) or nm in ("get_now_time", "system")})
    stubs["read_settings"] = read_settings
    P = Program(texts, overrides=overrides, stubs=stubs)
    P.vfs["porosity.csv"] = csv_text
    # the 3D VTK writers read &directory_control themselves (output.f90:811-814)
    P.nml_values = {"directory_control": {"csv_file": settings["csv_file"],
                                          "output_folder": settings["output_folder"]}}
    S = P.run_main()
    out = {}
    for f in ("u", "v", "w", "p") if len(shape) == 3 else ("u", "v", "p"):
        a = S[f]
        out[f] = np.array(a.data, dtype=np.float64).reshape(a.ext[::-1])
    out["div"] = _divergence_records(P.writes[63 if len(shape) == 2 else 62], shape)
    final = P.writes.get(VTK_FINAL_UNIT, [])
    temp = P.writes.get(VTK_TEMP_UNIT, [])
    if final:  # the VTK records: the end-of-run file and the istep_out file of the last step
        assert len(temp) == 2 * len(final)  # step 0 and step `steps`
        for key, recs in (("vtk_final", final), ("vtk_temp", temp[len(final):])):
            assert all(isinstance(x, (int, float)) for r in recs for x in r)
            out[key + "_vals"] = np.array([x for r in recs for x in r], dtype=np.float64)
            out[key + "_lens"] = np.array([len(r) for r in recs], dtype=np.int64)
    fp = [r[1:] for r in P.writes["*"] if r and r[0] == "Fp ="]
    fv = [r[1:] for r in P.writes["*"] if r and r[0] == "Fv ="]
    if fp:
        out["fp"] = np.array(fp, dtype=np.float64)
        out["fv"] = np.array(fv, dtype=np.float64)
        assert len(fp) == steps
    return s, shape, vals_read, steps, out


def _divergence_records(recs, shape):
    """The rows after the 'divergent velocity' record, one per (k,) j."""
    k = [q for q, r in enumerate(recs) if r == ["divergent velocity"]][-1]
    rows = int(np.prod(shape[1:]))
    body = recs[k + 1:k + 1 + rows]
    assert all(len(r) == shape[0] for r in body)
    return np.array(body, dtype=np.float64).reshape(shape[::-1])


def _sizes(shape):
    if len(shape) == 2:
        return {"md": shape[0] + 1, "nd": shape[1] + 1}
    return {"md": shape[0] + 1, "nd": shape[1] + 1, "ld": shape[2] + 1}


def main():
    ref = os.environ.get("PF_REFERENCE_DIR")
    if not ref:
        raise SystemExit("set PF_REFERENCE_DIR to a checkout of the reference")
    for name in sys.argv[1:] or CASES:  # given names: only those cases
        s, shape, vals_read, steps, out = run_reference(ref, name)
        np.savez_compressed(os.path.join(HERE, f"refpin_{name}.npz"), porosity=vals_read, steps=steps, **out)
        print(name, {k: float(np.abs(v).max()) for k, v in out.items()})


if __name__ == "__main__":
    main()
