"""pf_max_div_noalloc: max|div u| for callers that must not allocate device
memory (cudaMalloc/cudaFree synchronise the device and some programs run under
another allocator's memory budget).  The entry point reduces into scratch
compiled into the library; these tests check it against pf_norms (which uses
the case's own allocated scratch) on two calls in a row.  The device input
arrays here are allocated by the test with torch -- the entry point itself
allocates nothing.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from pixelflow_gb300 import _lib
from pixelflow_gb300 import geometry as G
from pixelflow_gb300.solver import Case

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_max_div_matches_pf_norms(dim):
    import torch
    if dim == 2:
        s, shape = G.settings_cylinder_2d(iter_max=30), (96, 48)
        vals = G.cylinder_2d(*shape, radius=0.15, cx=0.6, cy=0.5)
    else:
        s, shape = G.settings_spheres_3d(iter_max=20), (40, 32, 24)
        vals = G.spheres_3d(*shape, count=4, seed=7)
    L = _lib.load()
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        results = []
        for _ in range(2):  # two calls in a row, the state moving in between
            c.step(3)
            want, _ = c.norms()
            st = c.get_state()
            poro = c.porosity()
            d = {k: _dev(a) for k, a in st.items()}
            dp = _dev(poro)
            out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda:0")
            torch.cuda.synchronize()
            ptr = lambda t: ctypes.c_void_p(t.data_ptr())
            w = ptr(d["w"]) if dim == 3 else None
            rc = L.pf_max_div_noalloc(ctypes.byref(c.params), ptr(d["u"]), ptr(d["v"]), w, ptr(dp),
                                      st["u"].shape[-1], st["u"].shape[-2], ptr(out), None)
            assert rc == 0, L.pf_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            results.append((got, want))
    for got, want in results:
        assert np.isfinite(got) and want > 0
        assert abs(got - want) <= 1e-12 * want, (got, want)
    assert results[0][0] != results[1][0]


def test_noalloc_rejects_sizes_beyond_scratch():
    L = _lib.load()
    s = G.settings_spheres_3d()
    from pixelflow_gb300.solver import make_params
    prm = make_params(s, (8, 1024, 1024))  # n*l = 1048576 rows > 262144
    dummy = ctypes.c_void_p(16)
    rc = L.pf_max_div_noalloc(ctypes.byref(prm), dummy, dummy, dummy, dummy, 10, 1026, dummy, None)
    assert rc == -1
    assert b"PF_NOALLOC_MAX_ROWS" in L.pf_last_error()
