"""The batched form: many independent cases resident on one GPU, advanced by
one persistent kernel (include/pixelflow_gpu.h, pf_batch_*).

Each case runs the precision form (FP32 stencils and sweeps inside FP64
defect correction).  The reference runs one case per process; a `Batch`
holds many of them and advances any subset by per-case step counts in one
launch per dimension.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import PfBatchOptions, check
from .config import Settings
from .solver import make_options, make_params

GIB = 1 << 30


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def case_bytes(settings: Settings, shape: Sequence[int], large_cells: int = 100000) -> int:
    """Device bytes one case of this shape takes in a batch: the allocation
    pf_batch_add makes (precision form; a case the persistent kernel steps,
    at most `large_cells` cells, uses the split FP32 sweep)."""
    L = _lib.load()
    b = ctypes.c_size_t()
    cells = int(np.prod(shape))
    s = settings.replace(precision="mixed")
    if cells <= large_cells:
        s = s.replace(sweep_form="split")
    check(L.pf_case_bytes(ctypes.byref(make_params(s, shape)),
                          ctypes.byref(make_options(s, use_graph=cells > large_cells)), ctypes.byref(b)))
    return b.value


class Batch:
    def __init__(self, cluster: int = 4, threads: int = 512, max_cases: int = 1024,
                 hbm_budget_bytes: int = 150 * GIB, global_passes: bool = False, large_cells: int = 100000,
                 use_graph: bool = True):
        self.L = _lib.load()
        o = PfBatchOptions()
        self.L.pf_batch_default_options(ctypes.byref(o))
        o.cluster, o.threads, o.max_cases, o.hbm_budget_bytes = cluster, threads, max_cases, int(hbm_budget_bytes)
        o.global_passes = 1 if global_passes else 0
        o.large_cells = int(large_cells)
        o.use_graph = 1 if use_graph else 0
        h = ctypes.c_void_p()
        check(self.L.pf_batch_create(ctypes.byref(o), ctypes.byref(h)))
        self.h = h
        self.shapes: Dict[int, Tuple[int, ...]] = {}
        self.params: Dict[int, object] = {}

    def close(self):
        if getattr(self, "h", None):
            check(self.L.pf_batch_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def configure(self, cluster: int, threads: int):
        check(self.L.pf_batch_configure(self.h, int(cluster), int(threads)))

    def add(self, settings: Settings, shape: Sequence[int], porosity_values: np.ndarray) -> int:
        """Add a case; raises PfError(PF_E_NOMEM) if it does not fit the budget now."""
        s = settings.replace(precision="mixed")
        shape = tuple(int(x) for x in shape)
        prm = make_params(s, shape)
        opt = make_options(s, use_graph=False)
        vals = np.ascontiguousarray(porosity_values, dtype=np.float64)
        slot = ctypes.c_int()
        check(self.L.pf_batch_add(self.h, ctypes.byref(prm), ctypes.byref(opt), _ptr(vals), ctypes.byref(slot)))
        self.shapes[slot.value] = shape
        self.params[slot.value] = prm
        return slot.value

    def add_shapes(self, settings: Settings, shape: Sequence[int], shapes, edge: float = 1.0) -> int:
        """Add a case whose porosity is generated on the GPU from analytic shapes
        (circles/ellipses in 2D, spheres in 3D; see geometry.to_pf_shapes)."""
        from ._lib import PfShape
        from .geometry import to_pf_shapes
        s = settings.replace(precision="mixed")
        shape = tuple(int(x) for x in shape)
        prm = make_params(s, shape)
        opt = make_options(s, use_graph=False)
        pfs = shapes if (shapes and isinstance(shapes[0], PfShape)) else to_pf_shapes(shapes, len(shape))
        arr = (PfShape * max(1, len(pfs)))(*pfs)
        slot = ctypes.c_int()
        check(self.L.pf_batch_add_shapes(self.h, ctypes.byref(prm), ctypes.byref(opt), ctypes.cast(arr, ctypes.c_void_p),
                                         len(pfs), float(edge), ctypes.byref(slot)))
        self.shapes[slot.value] = shape
        self.params[slot.value] = prm
        return slot.value

    def remove(self, slot: int):
        check(self.L.pf_batch_remove(self.h, int(slot)))
        self.shapes.pop(slot, None)
        self.params.pop(slot, None)

    def step(self, nsteps: int):
        check(self.L.pf_batch_step(self.h, int(nsteps)))

    def step_slots(self, slots: Sequence[int], nsteps: Sequence[int]):
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        ns = np.ascontiguousarray(nsteps, dtype=np.int32)
        check(self.L.pf_batch_step_slots(self.h, _ptr(sl), _ptr(ns), len(sl)))

    def synchronize(self):
        check(self.L.pf_batch_synchronize(self.h))

    def get_state(self, slot: int) -> Dict[str, np.ndarray]:
        shape = self.shapes[slot]
        dim = len(shape)
        m, n = shape[0], shape[1]
        fs = (n + 2, m + 2) if dim == 2 else (shape[2] + 2, n + 2, m + 2)
        out = {k: np.empty(fs) for k in (("u", "v", "p") + (("w",) if dim == 3 else ()))}
        check(self.L.pf_batch_get_state(self.h, int(slot), _ptr(out["u"]), _ptr(out["v"]), _ptr(out.get("w")),
                                        _ptr(out["p"]), m + 2, n + 2))
        return out

    def norms(self, slot: int) -> Tuple[float, float]:
        md, se = ctypes.c_double(), ctypes.c_double()
        rc = self.L.pf_batch_norms(self.h, int(slot), ctypes.byref(md), ctypes.byref(se))
        if rc not in (0, -4):
            check(rc)
        return md.value, se.value

    def memory(self) -> Tuple[int, int]:
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        check(self.L.pf_batch_memory(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def last_ms(self) -> float:
        """Device time of the last step call (CUDA events on the batch stream)."""
        ms = ctypes.c_double()
        check(self.L.pf_batch_last_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def graph_stats(self) -> Tuple[int, int]:
        """(graphs of the persistent launch captured, calls that replayed one)."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        check(self.L.pf_batch_graph_stats(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def kernel_launches(self) -> int:
        n = ctypes.c_int64()
        check(self.L.pf_batch_kernel_launches(self.h, ctypes.byref(n)))
        return n.value
