"""Field output at istep_out: the reference's legacy-VTK files, fed by
asynchronous snapshots so the GPU keeps stepping while a file is written.

`write_vtk` writes the file `output_paraview_temp_2d` / `_3d` write
(src/omp_parallel/lib/output.f90:421-537, :968-1088): an ASCII STRUCTURED_GRID
of the m x n [x l] interior nodes at x_i = dx (i-1) - width*center_x (and y,
z likewise, lib/grid.f90:81-89, :333-345), with the same arrays in the same
order -- velocity, velocityInFluid, (2D: dimless_v), porosity, pressure,
VelocityDivergent, (2D: abs_dimless_v) -- each value formatted as Fortran
f16.4, records in Fortran order (i fastest).  The file is
``<folder>/output_<istep:05d>.vtk``.

`run_with_output` is the reference's time loop with that output: every
`istep_out` steps it takes a snapshot (pf_snapshot_begin), enqueues the next
steps, and writes the previous snapshot while they run.

Arrays are in the library's Fortran layout with ghosts: (n+2, m+2) in 2D,
(l+2, n+2, m+2) in 3D, a[k, j, i] == a(i, j, k).
"""
from __future__ import annotations

import os
from typing import Dict, List, Optional

import numpy as np

from .config import Settings


def node_coords(settings: Settings, shape) -> List[np.ndarray]:
    """x, y[, z] of nodes 0..m+1 (ghosts included), lib/grid.f90:81-89, :333-345."""
    s = settings
    dim = len(shape)
    lens = [s.width, s.height] + ([s.depth] if dim == 3 else [])
    cents = [s.center_x, s.center_y] + ([s.center_z] if dim == 3 else [])
    out = []
    for count, length, cen in zip(shape, lens, cents):
        d = length / (count - 1)
        out.append(d * (np.arange(count + 2, dtype=np.float64) - 1.0) - length * cen)
    return out


def _f16_4(a: np.ndarray) -> np.ndarray:
    """Fortran f16.4 text of each value (right-aligned in 16 columns)."""
    return np.char.mod("%16.4f", a)


def _rows(cols: List[np.ndarray]) -> str:
    """Records of 3(f16.4,1x): each value, one blank, up to three per line."""
    parts = [_f16_4(np.asarray(c, dtype=np.float64).ravel()) for c in cols]
    line = parts[0]
    for p in parts[1:]:
        line = np.char.add(np.char.add(line, " "), p)
    line = np.char.add(line, " ")
    return "\n".join(line.tolist()) + "\n"


def write_vtk(path: str, state: Dict[str, np.ndarray], porosity: np.ndarray, settings: Settings,
              final: bool = False) -> None:
    """final=True: the file the main programs write at the end of the run,
    output_paraview_2d/_3d (output.f90:307-419, :793-910).  In 2D it is the
    same text; in 3D its porosity section comes after VelocityDivergent
    instead of before pressure."""
    s = settings
    u, v, p = state["u"], state["v"], state["p"]
    dim = u.ndim
    if dim == 2:
        n, m = u.shape[0] - 2, u.shape[1] - 2
        shape = (m, n)
        I = (slice(1, n + 1), slice(1, m + 1))
    else:
        l, n, m = u.shape[0] - 2, u.shape[1] - 2, u.shape[2] - 2
        shape = (m, n, l)
        I = (slice(1, l + 1), slice(1, n + 1), slice(1, m + 1))
    xs = node_coords(s, shape)
    npts = int(np.prod(shape))
    po = porosity[I]
    zero = np.zeros(po.shape)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\n")
        f.write("2D flow\n" if dim == 2 else "3D flow\n")
        f.write("ASCII \n")
        f.write("DATASET STRUCTURED_GRID\n")
        f.write("DIMENSIONS " + "".join(" %4d" % x for x in (shape if dim == 3 else shape + (1,))) + "\n")
        f.write("POINTS %9d float\n" % npts)
        if dim == 2:
            Y, X = np.meshgrid(xs[1][1:n + 1], xs[0][1:m + 1], indexing="ij")
            f.write(_rows([X, Y, zero]))
        else:
            Z, Y, X = np.meshgrid(xs[2][1:l + 1], xs[1][1:n + 1], xs[0][1:m + 1], indexing="ij")
            f.write(_rows([X, Y, Z]))
        f.write("POINT_DATA %9d\n" % npts)
        w = state.get("w")
        f.write("VECTORS velocity float\n")
        f.write(_rows([u[I], v[I], zero if dim == 2 else w[I]]))
        f.write("VECTORS velocityInFluid float\n")
        f.write(_rows([u[I] * po, v[I] * po, zero if dim == 2 else w[I] * po]))
        if dim == 2:
            f.write("VECTORS dimless_v float\n")
            f.write(_rows([u[I] * po / s.inlet_velocity, v[I] * po / s.inlet_velocity, zero]))
        porosity_last = final and dim == 3
        if not porosity_last:
            f.write("SCALARS porosity float\n")
            f.write("LOOKUP_TABLE default\n")
            f.write(_rows([po]))
        f.write("SCALARS pressure float\n")
        f.write("LOOKUP_TABLE default\n")
        f.write(_rows([p[I]]))
        # plain central divergence over the node spacing (output.f90:501-510, :1058-1069)
        if dim == 2:
            x, y = xs
            div = ((u[1:n + 1, 2:] - u[1:n + 1, :-2]) / (x[2:] - x[:-2])[None, :]
                   + (v[2:, 1:m + 1] - v[:-2, 1:m + 1]) / (y[2:] - y[:-2])[:, None])
        else:
            x, y, z = xs
            div = ((u[1:l + 1, 1:n + 1, 2:] - u[1:l + 1, 1:n + 1, :-2]) / (x[2:] - x[:-2])[None, None, :]
                   + (v[1:l + 1, 2:, 1:m + 1] - v[1:l + 1, :-2, 1:m + 1]) / (y[2:] - y[:-2])[None, :, None]
                   + (w[2:, 1:n + 1, 1:m + 1] - w[:-2, 1:n + 1, 1:m + 1]) / (z[2:] - z[:-2])[:, None, None])
        f.write("SCALARS VelocityDivergent float\n")
        f.write("LOOKUP_TABLE default\n")
        f.write(_rows([div]))
        if porosity_last:
            f.write("SCALARS porosity float\n")
            f.write("LOOKUP_TABLE default\n")
            f.write(_rows([po]))
        if dim == 2:
            f.write("SCALARS abs_dimless_v float\n")
            f.write("LOOKUP_TABLE default\n")
            a = np.sqrt((u[I] * po / s.inlet_velocity) ** 2 + (v[I] * po / s.inlet_velocity) ** 2)
            f.write(_rows([a]))


def vtk_path(folder: str, istep: int) -> str:
    return os.path.join(folder, "output_%05d.vtk" % istep)


def run_with_output(case, steps: int, istep_out: int, folder: str, write=None,
                    forces_radius: Optional[float] = None) -> List[dict]:
    """The reference's loop with its periodic output: `steps` steps and a VTK
    file (or `write(istep, state)`) every `istep_out` steps.  A snapshot is
    taken on the device right after its step, the steps of the next interval
    are enqueued, and only then is the previous snapshot written, so the
    device-to-host copy and the file writing overlap the GPU's stepping.
    With `forces_radius` the force log is recorded after every step, as the
    drag program does (ibm_2d_drag_omp_cpu.f90:121); each record waits for
    its step.  Returns the force log."""
    os.makedirs(folder, exist_ok=True)
    porosity = case.porosity()
    if write is None:
        def write(istep, state):
            write_vtk(vtk_path(folder, istep), state, porosity, case.settings)
    log: List[dict] = []

    def advance(k, first):
        if forces_radius is None:
            case.step(k)
            return
        for q in range(k):
            case.step(1)
            rec = case.forces(radius=forces_radius)
            rec["istep"] = first + q
            log.append(rec)

    done, pending, ready = 0, None, None
    while done < steps:
        k = min(istep_out - done % istep_out, steps - done)
        advance(k, done + 1)  # enqueued; without the force log nothing waits here
        done += k
        if ready is not None:  # written while the GPU runs the steps just enqueued
            write(*ready)
            ready = None
        if done % istep_out == 0:
            if pending is not None:
                ready = (pending, case.snapshot_wait())
            case.snapshot_begin()
            pending = done
    if ready is not None:
        write(*ready)
    if pending is not None:
        write(pending, case.snapshot_wait())
    return log
