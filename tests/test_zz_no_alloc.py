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


def _padded(a, ld1, ld2):
    """The field in a caller's static array: leading dimensions ld1 >= m+2,
    ld2 >= n+2 (Fortran a(0:md,0:nd[,0:l+1])), the padding filled with NaN
    so that a read outside the case's extent would show in the result."""
    out = np.full(a.shape[:-2] + (ld2, ld1), np.nan)
    out[..., : a.shape[-2], : a.shape[-1]] = a
    return out


@pytest.mark.parametrize("dim,pad", [(2, (0, 0)), (3, (0, 0)), (2, (7, 3)), (3, (5, 4))])
def test_noalloc_max_div_matches_pf_norms(dim, pad):
    import torch
    if dim == 2:
        s, shape = G.settings_cylinder_2d(iter_max=30), (96, 48)
        vals = G.cylinder_2d(*shape, radius=0.15, cx=0.6, cy=0.5)
    else:
        s, shape = G.settings_spheres_3d(iter_max=20), (40, 32, 24)
        vals = G.spheres_3d(*shape, count=4, seed=7)
    L = _lib.load()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    side = torch.cuda.Stream()  # a caller's own stream, not the legacy default one
    with Case(s, shape, vals) as c:
        c.initial_conditions()
        results = []
        for call in range(2):  # two calls in a row, the state moving in between
            c.step(3)
            want, _ = c.norms()
            st = c.get_state()
            ld1, ld2 = st["u"].shape[-1] + pad[0], st["u"].shape[-2] + pad[1]
            d = {k: _dev(_padded(a, ld1, ld2)) for k, a in st.items()}
            dp = _dev(_padded(c.porosity(), ld1, ld2))
            out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda:0")
            w = ptr(d["w"]) if dim == 3 else None
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            rc = L.pf_max_div_noalloc(ctypes.byref(c.params), ptr(d["u"]), ptr(d["v"]), w, ptr(dp),
                                      ld1, ld2, ptr(out), ctypes.c_void_p(side.cuda_stream))
            assert rc == 0, L.pf_last_error()
            side.synchronize()
            free1 = torch.cuda.mem_get_info()[0]
            if call == 1:  # the first call on the device may load the library's kernels
                assert free1 == free0, ("device memory in use changed across the call", free0, free1)
            results.append((float(out.item()), want))
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
