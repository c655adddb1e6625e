"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Wraps oracle/libpf_oracle.so (the C restatement of PixelFlow's OpenMP step in
pf_oracle.c).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm use it, always as the checker or the timed CPU
baseline -- never as a product path.  This restatement reproduces the
reference's own programs, executed from their Fortran source on small
grids, bit for bit (see pf_oracle.c and tests/test_reference_pin.py).

Arrays are numpy views in the reference's Fortran layout with ghosts:
shape (n+2, m+2) for 2D and (l+2, n+2, m+2) for 3D, so that
``a[k, j, i]`` is ``a(i, j, k)`` of the Fortran code.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import build as _build

_LIB = None


class OrParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("m", ctypes.c_int32), ("n", ctypes.c_int32), ("l", ctypes.c_int32),
        ("xnue", ctypes.c_double), ("xlambda", ctypes.c_double), ("density", ctypes.c_double),
        ("width", ctypes.c_double), ("height", ctypes.c_double), ("depth", ctypes.c_double),
        ("time", ctypes.c_double), ("inlet_velocity", ctypes.c_double),
        ("outlet_pressure", ctypes.c_double), ("aoa", ctypes.c_double),
        ("istep_max", ctypes.c_int32), ("iter_max", ctypes.c_int32),
        ("thickness", ctypes.c_double), ("threshold", ctypes.c_double),
        ("relux_factor", ctypes.c_double), ("nonslip", ctypes.c_int32), ("inflow_porosity", ctypes.c_int32),
        ("wall_mode", ctypes.c_int32), ("walls", ctypes.c_int32 * 6), ("slip_y", ctypes.c_int32),
    ]


def make_params(settings, m: int, n: int, l: int = 1, dim: int = 2) -> OrParams:
    s = settings
    return OrParams(dim, m, n, l if dim == 3 else 1, s.xnue, s.xlambda, s.density, s.width,
                    s.height, s.depth, s.time, s.inlet_velocity, s.outlet_pressure, s.aoa,
                    int(s.istep_max), int(s.iter_max), s.thickness, s.threshold, s.relux_factor,
                    1 if s.nonslip else 0, 1 if getattr(s, "inflow_porosity", False) else 0,
                    1 if getattr(s, "walls", None) is not None else 0,
                    (ctypes.c_int32 * 6)(*(getattr(s, "walls", None) or (0,) * 6)),
                    1 if getattr(s, "slip_y", False) else 0)


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        for sfx in ("_d", "_f"):
            vp = ctypes.c_void_p
            getattr(L, "or_create" + sfx).restype = vp
            getattr(L, "or_create" + sfx).argtypes = [ctypes.POINTER(OrParams)]
            getattr(L, "or_destroy" + sfx).argtypes = [vp]
            getattr(L, "or_scalars" + sfx).argtypes = [vp, vp]
            getattr(L, "or_work" + sfx).restype = vp
            getattr(L, "or_work" + sfx).argtypes = [vp, ctypes.c_int]
            getattr(L, "or_last_error" + sfx).restype = ctypes.c_double
            getattr(L, "or_last_error" + sfx).argtypes = [vp]
            getattr(L, "or_grid_conditions" + sfx).argtypes = [vp, vp, vp]
            getattr(L, "or_boundary" + sfx).argtypes = [vp, vp, vp, vp, vp]
            getattr(L, "or_initialize" + sfx).argtypes = [vp, vp, vp, vp, vp]
            getattr(L, "or_divergence" + sfx).argtypes = [vp, vp, vp, vp]
            getattr(L, "or_predictor" + sfx).argtypes = [vp] * 8
            getattr(L, "or_coefficients" + sfx).argtypes = [vp] * 5
            getattr(L, "or_boundary_matrix" + sfx).argtypes = [vp, vp]
            getattr(L, "or_sor" + sfx).restype = ctypes.c_double
            getattr(L, "or_sor" + sfx).argtypes = [vp, vp]
            getattr(L, "or_solve_p" + sfx).restype = ctypes.c_double
            getattr(L, "or_solve_p" + sfx).argtypes = [vp] * 9
            getattr(L, "or_projection" + sfx).argtypes = [vp] * 5
            getattr(L, "or_step" + sfx).restype = ctypes.c_double
            getattr(L, "or_step" + sfx).argtypes = [vp, ctypes.c_int] + [vp] * 8
            getattr(L, "or_divergence_diag" + sfx).restype = ctypes.c_double
            getattr(L, "or_divergence_diag" + sfx).argtypes = [vp] * 6
            getattr(L, "or_forces" + sfx).argtypes = [vp] * 7
        _LIB = L
    return _LIB


WORK = {"ap": 0, "ae": 1, "aw": 2, "an": 3, "as": 4, "at": 5, "ab": 6, "bb": 7, "div": 8, "p_old": 9}


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleCase:
    """One case of the restated reference step, owning its Fortran-layout arrays."""

    def __init__(self, settings, shape, porosity_values: np.ndarray, dtype=np.float64):
        self.dim = len(shape)
        if self.dim == 2:
            m, n = shape
            l = 1
            self.shape = (n + 2, m + 2)
        else:
            m, n, l = shape
            self.shape = (l + 2, n + 2, m + 2)
        self.m, self.n, self.l = m, n, l
        self.dtype = np.dtype(dtype)
        self.sfx = "_d" if self.dtype == np.float64 else "_f"
        self.settings = settings
        self.params = make_params(settings, m, n, l, self.dim)
        L = lib()
        self._f = lambda name: getattr(L, name + self.sfx)
        self.ctx = self._f("or_create")(ctypes.byref(self.params))
        if not self.ctx:
            raise MemoryError("oracle: allocation failed")
        z = lambda: np.zeros(self.shape, dtype=self.dtype)
        self.u, self.v, self.p, self.uo, self.vo, self.poro = z(), z(), z(), z(), z(), z()
        self.w = z() if self.dim == 3 else None
        self.wo = z() if self.dim == 3 else None
        vals = np.ascontiguousarray(porosity_values, dtype=np.float64)
        self._f("or_grid_conditions")(self.ctx, _ptr(vals), _ptr(self.poro))
        self.last_error = 0.0

    def __del__(self):
        try:
            if getattr(self, "ctx", None):
                self._f("or_destroy")(self.ctx)
                self.ctx = None
        except Exception:
            pass

    # scalars ------------------------------------------------------------
    def scalars(self):
        out = np.zeros(4)
        self._f("or_scalars")(self.ctx, _ptr(out))
        return dict(dx=out[0], dy=out[1], dz=out[2], dt=out[3])

    def work(self, name: str) -> np.ndarray:
        addr = self._f("or_work")(self.ctx, WORK[name])
        ct = ctypes.c_double if self.dtype == np.float64 else ctypes.c_float
        buf = (ct * int(np.prod(self.shape))).from_address(addr)
        return np.frombuffer(buf, dtype=self.dtype).reshape(self.shape)

    # reference routines --------------------------------------------------
    def initialize(self):
        self._f("or_initialize")(self.ctx, _ptr(self.p), _ptr(self.u), _ptr(self.v), _ptr(self.w))

    def boundary(self):
        self._f("or_boundary")(self.ctx, _ptr(self.p), _ptr(self.u), _ptr(self.v), _ptr(self.w))

    def copy_old(self):
        self.uo[...] = self.u
        self.vo[...] = self.v
        if self.dim == 3:
            self.wo[...] = self.w

    def divergence(self):
        self._f("or_divergence")(self.ctx, _ptr(self.uo), _ptr(self.vo), _ptr(self.wo))

    def predictor(self):
        self._f("or_predictor")(self.ctx, _ptr(self.u), _ptr(self.v), _ptr(self.w), _ptr(self.uo),
                                _ptr(self.vo), _ptr(self.wo), _ptr(self.poro))

    def coefficients(self):
        self._f("or_coefficients")(self.ctx, _ptr(self.u), _ptr(self.v), _ptr(self.w), _ptr(self.poro))

    def boundary_matrix(self):
        self._f("or_boundary_matrix")(self.ctx, _ptr(self.p))

    def sor(self) -> float:
        self.last_error = self._f("or_sor")(self.ctx, _ptr(self.p))
        return self.last_error

    def solve_p(self) -> float:
        self.last_error = self._f("or_solve_p")(self.ctx, _ptr(self.p), _ptr(self.u), _ptr(self.v),
                                                _ptr(self.w), _ptr(self.uo), _ptr(self.vo),
                                                _ptr(self.wo), _ptr(self.poro))
        return self.last_error

    def projection(self):
        self._f("or_projection")(self.ctx, _ptr(self.p), _ptr(self.u), _ptr(self.v), _ptr(self.w))

    def step(self, nsteps: int = 1) -> float:
        self.last_error = self._f("or_step")(self.ctx, int(nsteps), _ptr(self.p), _ptr(self.u),
                                             _ptr(self.v), _ptr(self.w), _ptr(self.uo), _ptr(self.vo),
                                             _ptr(self.wo), _ptr(self.poro))
        return self.last_error

    def divergence_diag(self, want_field: bool = False):
        out = np.zeros(self.shape, dtype=self.dtype) if want_field else None
        mx = self._f("or_divergence_diag")(self.ctx, _ptr(self.u), _ptr(self.v), _ptr(self.w),
                                           _ptr(self.poro), _ptr(out))
        return (mx, out) if want_field else mx

    def forces(self):
        """(pressure part (x, y, z), wall-friction part (x, y, z)) of the
        reference's force log sums."""
        out = np.zeros(6)
        self._f("or_forces")(self.ctx, _ptr(self.p), _ptr(self.u), _ptr(self.v), _ptr(self.w),
                             _ptr(self.poro), _ptr(out))
        return out[:3].copy(), out[3:].copy()

    def state(self):
        d = dict(u=self.u.copy(), v=self.v.copy(), p=self.p.copy())
        if self.dim == 3:
            d["w"] = self.w.copy()
        return d
