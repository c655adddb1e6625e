"""Generate tests/golden/porosity_ref_2d.csv, porosity_ref_3d.csv and
porosity_ref.npz with the reference's own preprocessing code.

The reference ships a porosity CSV writer (tools/output/output_porosity.py:
write_porosity_2d, write_porosity_3d) and the tanh porosity of its cylinder
tool (tools/cylinder/make_porosity_2d_cylinder.py: porosity_func).  This
script imports both from a checkout of the reference (its path in
PF_REFERENCE_DIR) and runs them unchanged on small seeded signed-distance
fields: porosity_func maps the distances (in cells) to porosity, the writers
write the files the Fortran programs read (grid.f90:36-47, :281-294).  The
cylinder tool's plotting and image imports (matplotlib, cv2, seaborn) are not
installed here and are not used by porosity_func, so they are replaced by
empty modules before the import.  Run from the repository root:

    PF_REFERENCE_DIR=<reference checkout> python -m tests.golden.make_reference_porosity
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    ref = os.environ.get("PF_REFERENCE_DIR")
    if not ref:
        raise SystemExit("set PF_REFERENCE_DIR to a checkout of the reference")
    for name in ("matplotlib", "matplotlib.pyplot", "cv2", "seaborn"):
        sys.modules.setdefault(name, types.ModuleType(name))
    writer = _load(os.path.join(ref, "tools", "output", "output_porosity.py"), "ref_output_porosity")
    cyl = _load(os.path.join(ref, "tools", "cylinder", "make_porosity_2d_cylinder.py"), "ref_cylinder")
    rng = np.random.default_rng(7)
    thickness = 1.5
    # 2D: a circle of radius 3 cells at an off-grid centre, data[i-1, j-1]
    m, n = 14, 9
    ii, jj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    cx, cy = 6.3, 4.1
    sdf2 = np.sqrt((ii - cx) ** 2 + (jj - cy) ** 2) - 3.0
    por2 = cyl.porosity_func(sdf2, thickness=thickness)
    # 3D: a sphere of radius 1.7 cells, plus a seeded perturbation of the distances
    m3, n3, l3 = 6, 5, 4
    i3, j3, k3 = np.meshgrid(np.arange(m3), np.arange(n3), np.arange(l3), indexing="ij")
    sdf3 = np.sqrt((i3 - 2.4) ** 2 + (j3 - 2.2) ** 2 + (k3 - 1.6) ** 2) - 1.7 + rng.normal(0, 0.3, (m3, n3, l3))
    por3 = cyl.porosity_func(sdf3, thickness=thickness)
    cwd = os.getcwd()
    os.chdir(HERE)
    try:
        writer.write_porosity_2d(por2, "porosity_ref_2d.csv")
        writer.write_porosity_3d(por3, "porosity_ref_3d.csv")
    finally:
        os.chdir(cwd)
    np.savez(os.path.join(HERE, "porosity_ref.npz"), sdf2=sdf2, por2=por2, sdf3=sdf3, por3=por3,
             thickness=thickness)


if __name__ == "__main__":
    main()
