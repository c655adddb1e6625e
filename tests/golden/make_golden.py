"""Generate the golden vectors under tests/golden/ from the oracle.

The reference ships no tests or expected outputs and no Fortran compiler is
available to run it, so these vectors come from the oracle (the C
restatement of the reference's OpenMP step, cross-checked bit for bit
against an independent numpy restatement).  They pin the oracle against
regressions and give the GPU tests fixed expected outputs that need no CPU
re-run.  Regenerate with: python -m tests.golden.make_golden
"""
import os

import numpy as np

from pixelflow_gb300 import geometry as G

HERE = os.path.dirname(os.path.abspath(__file__))

# name -> (dim, shape, iter_max, steps, geometry)
CASES = {
    "cyl2d_24x12_it10_s5": dict(dim=2, shape=(24, 12), iter_max=10, steps=5),
    "cyl2d_25x13_it10_s5": dict(dim=2, shape=(25, 13), iter_max=10, steps=5),
    "sph3d_12x10x8_it6_s3": dict(dim=3, shape=(12, 10, 8), iter_max=6, steps=3),
    "sph3d_11x9x7_it6_s3": dict(dim=3, shape=(11, 9, 7), iter_max=6, steps=3),
}


def case_inputs(spec):
    if spec["dim"] == 2:
        m, n = spec["shape"]
        s = G.settings_cylinder_2d(iter_max=spec["iter_max"])
        vals = G.cylinder_2d(m, n, radius=0.2, cx=0.6, cy=0.45)
    else:
        m, n, l = spec["shape"]
        s = G.settings_spheres_3d(iter_max=spec["iter_max"])
        vals = G.spheres_3d(m, n, l, spheres=np.array([[0.4, 0.5, 0.5, 0.2], [0.7, 0.3, 0.6, 0.15]]))
    return s, vals


def run_oracle(spec):
    from oracle.oracle import OracleCase
    s, vals = case_inputs(spec)
    c = OracleCase(s, spec["shape"], vals)
    c.initialize()
    err = c.step(spec["steps"])
    out = dict(u=c.u.copy(), v=c.v.copy(), p=c.p.copy(), poro=c.poro.copy(), porosity_values=vals,
               sor_error=np.array(err), max_div=np.array(c.divergence_diag()))
    if spec["dim"] == 3:
        out["w"] = c.w.copy()
    return out


def main():
    for name, spec in CASES.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **run_oracle(spec))
        print("wrote", name)


if __name__ == "__main__":
    main()
