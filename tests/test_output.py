"""The VTK writer against a line-by-line restatement of the reference's
output_paraview_temp_2d/_3d (lib/output.f90:421-537, :968-1088) on small
synthetic fields.  CPU only."""
import math

import numpy as np
import pytest

from pixelflow_gb300.config import Settings
from pixelflow_gb300.output import node_coords, write_vtk


def _f(x):
    return "%16.4f" % x


def _reference_text(st, po, s, dim, final=False):
    """Loop-by-loop statement of the Fortran writer (records of 3(f16.4,1x)).
    final: output_paraview_2d/_3d (output.f90:307-419, :793-910), the file of
    the end of the run, whose 3D form writes porosity last."""
    u, v, p = st["u"], st["v"], st["p"]
    if dim == 2:
        n, m = u.shape[0] - 2, u.shape[1] - 2
        l = 1
    else:
        l, n, m = u.shape[0] - 2, u.shape[1] - 2, u.shape[2] - 2
    xs = node_coords(s, (m, n) if dim == 2 else (m, n, l))
    U = (lambda a, i, j, k: a[j, i]) if dim == 2 else (lambda a, i, j, k: a[k, j, i])
    ks = [0] if dim == 2 else range(1, l + 1)
    cells = [(i, j, k) for k in ks for j in range(1, n + 1) for i in range(1, m + 1)]
    rec = lambda vals: " ".join(_f(x) for x in vals) + " "
    out = ["# vtk DataFile Version 3.0", "2D flow" if dim == 2 else "3D flow", "ASCII ", "DATASET STRUCTURED_GRID",
           "DIMENSIONS " + "".join(" %4d" % x for x in ((m, n, 1) if dim == 2 else (m, n, l))),
           "POINTS %9d float" % len(cells)]
    for (i, j, k) in cells:
        out.append(rec((xs[0][i], xs[1][j], 0.0 if dim == 2 else xs[2][k])))
    out.append("POINT_DATA %9d" % len(cells))
    w = st.get("w")
    out.append("VECTORS velocity float")
    for c in cells:
        out.append(rec((U(u, *c), U(v, *c), 0.0 if dim == 2 else U(w, *c))))
    out.append("VECTORS velocityInFluid float")
    for c in cells:
        e = U(po, *c)
        out.append(rec((U(u, *c) * e, U(v, *c) * e, 0.0 if dim == 2 else U(w, *c) * e)))
    if dim == 2:
        out.append("VECTORS dimless_v float")
        for c in cells:
            e = U(po, *c)
            out.append(rec((U(u, *c) * e / s.inlet_velocity, U(v, *c) * e / s.inlet_velocity, 0.0)))
    porosity = ["SCALARS porosity float", "LOOKUP_TABLE default"] + [rec((U(po, *c),)) for c in cells]
    if not (final and dim == 3):
        out += porosity
    out += ["SCALARS pressure float", "LOOKUP_TABLE default"] + [rec((U(p, *c),)) for c in cells]
    out += ["SCALARS VelocityDivergent float", "LOOKUP_TABLE default"]
    x, y = xs[0], xs[1]
    for (i, j, k) in cells:
        if dim == 2:
            d = (u[j, i + 1] - u[j, i - 1]) / (x[i + 1] - x[i - 1]) + (v[j + 1, i] - v[j - 1, i]) / (y[j + 1] - y[j - 1])
        else:
            z = xs[2]
            d = ((u[k, j, i + 1] - u[k, j, i - 1]) / (x[i + 1] - x[i - 1])
                 + (v[k, j + 1, i] - v[k, j - 1, i]) / (y[j + 1] - y[j - 1])
                 + (w[k + 1, j, i] - w[k - 1, j, i]) / (z[k + 1] - z[k - 1]))
        out.append(rec((d,)))
    if final and dim == 3:
        out += porosity
    if dim == 2:
        out += ["SCALARS abs_dimless_v float", "LOOKUP_TABLE default"]
        for c in cells:
            e = U(po, *c)
            out.append(rec((math.sqrt((U(u, *c) * e / s.inlet_velocity) ** 2
                                      + (U(v, *c) * e / s.inlet_velocity) ** 2),)))
    return "\n".join(out) + "\n"


@pytest.mark.parametrize("final", [False, True])
@pytest.mark.parametrize("dim", [2, 3])
def test_vtk_writer_matches_reference_layout(dim, final, tmp_path):
    rng = np.random.default_rng(3)
    shape = (5, 4) if dim == 2 else (4, 3, 3)
    fshape = tuple(x + 2 for x in reversed(shape))
    st = {k: rng.normal(size=fshape) * 3 for k in ("u", "v", "p") + (("w",) if dim == 3 else ())}
    po = rng.uniform(0, 1, size=fshape)
    s = Settings(width=2.0, height=1.0, depth=1.5, inlet_velocity=0.7, center_x=0.25, center_y=0.5, center_z=0.4)
    path = tmp_path / "output_00010.vtk"
    write_vtk(str(path), st, po, s, final=final)
    assert path.read_text() == _reference_text(st, po, s, dim, final=final)
