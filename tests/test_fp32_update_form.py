"""The precision form's FP32 correction sweep, emulated in numpy on the CPU:
why its update is evaluated as e + r + (w/sigma) sum a_f (e_f - e).

One step's pressure solve of a small 3D spheres case: the plain FP64 SOR
(the oracle's, 100 iterations) against 4 defect-correction passes of 25
sweeps whose correction e and operator are held in FP32.  With the update in
the form (1-w) e + r - sum a'_f e_f the operator's rounding shifts its row
sum (the same few 1e-8 at every pure-fluid cell), which acts on the smooth
pressure modes; keeping the row sum (a constant correction maps to e + r
exactly) removes that error.  The emulation rounds the normalised FP64
coefficients to FP32 instead of rebuilding them from FP32 porosity as the
kernels do (pixelflow_gb300/csrc/pf_cells.cuh, dc_cell_faces); the point it
checks is the form of the update."""
import numpy as np

from oracle.np_oracle import NpCase
from pixelflow_gb300 import geometry as G

KEYS = ("ae", "aw", "an", "as", "at", "ab")
OFFS = {"ae": (1, 0, 0), "aw": (-1, 0, 0), "an": (0, 1, 0), "as": (0, -1, 0), "at": (0, 0, 1), "ab": (0, 0, -1)}


def _setup(n=24):
    s = G.settings_spheres_3d(iter_max=100)
    c = NpCase(s, (n, n, n), G.spheres_3d(n, n, n, count=4, seed=1))
    c.initialize()
    c.step(2)
    uo, vo, wo = c.u.copy(), c.v.copy(), c.w.copy()
    c.predictor(uo, vo, wo, c.divergence(uo, vo, wo))
    C = c.coefficients()
    p0 = c.p.copy()
    c.sor(C)
    return c, C, p0, c.p.copy()


def _halo(c, a):
    m, n, l = c.m, c.n, c.l
    a[1:l + 1, 0, 1:m + 1] = a[1:l + 1, n, 1:m + 1]
    a[1:l + 1, n + 1, 1:m + 1] = a[1:l + 1, 1, 1:m + 1]
    a[0, 1:n + 1, 1:m + 1] = a[l, 1:n + 1, 1:m + 1]
    a[l + 1, 1:n + 1, 1:m + 1] = a[1, 1:n + 1, 1:m + 1]


def _dc_error(c, C, p0, pref, rowsum, passes=4, sweeps=25):
    S, I = c._s, c._interior()
    om = float(c.relux)
    wap = om / C["ap"]
    A = {k: C[k] * wap for k in KEYS}
    A32 = {k: A[k].astype(np.float32) for k in KEYS}
    bbn = C["bb"] * wap
    one_m = np.float32(1.0) - np.float32(om)
    outlet = np.zeros(A["ae"].shape, bool)
    outlet[..., -1] = True  # the outlet column keeps (1-w) e + r (no neighbours)
    first, second = c.colour_masks()
    p = p0.copy()
    for _ in range(passes):
        _halo(c, p)
        r = bbn - om * S(p)
        for k in KEYS:
            r = r - A[k] * S(p, *OFFS[k])
        r = r.astype(np.float32)
        e = np.zeros(p.shape, dtype=np.float32)
        for _ in range(sweeps):
            for mask in (first, second):
                _halo(c, e)
                se = S(e)
                plain = one_m * se + r
                for k in KEYS:
                    plain = plain - A32[k] * S(e, *OFFS[k])
                new = plain
                if rowsum:
                    acc = se + r
                    for k in KEYS:
                        acc = acc + A32[k] * (se - S(e, *OFFS[k]))
                    new = np.where(outlet, plain, acc)
                inter = e[I]
                inter[mask] = new[mask]
        p[I] = S(p) + S(e).astype(np.float64)
    d = S(p) - S(pref)
    return float(np.sqrt((d * d).sum() / (S(pref) ** 2).sum()))


def test_rowsum_form_removes_the_operator_rounding_error():
    c, C, p0, pref = _setup()
    plain = _dc_error(c, C, p0, pref, rowsum=False)
    kept = _dc_error(c, C, p0, pref, rowsum=True)
    print(f"pressure after one solve: (1-w) form {plain:.2e}, row-sum form {kept:.2e}")
    assert kept < 1e-6
    assert kept < plain / 20
