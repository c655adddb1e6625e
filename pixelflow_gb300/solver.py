"""Host-side mirror of PixelFlow's step routines, running on the GB300 library.

`Case` exposes the reference's own routine names with the same meaning:
`initial_conditions` (+ `boundary`), `solve_p`, `projection`, `boundary` and
the whole step loop body `step` (ibm_2d_uniform_omp_cpu.f90:80-125,
ibm_3d_uniform_omp_cpu.f90:81-132).  Fields cross the boundary in the
reference's Fortran layout: numpy arrays of shape (ld2, ld1) in 2D and
(l+2, ld2, ld1) in 3D, C-ordered, so ``a[k, j, i]`` is Fortran ``a(i, j, k)``
with the ghost layer at index 0 and m+1 (n+1, l+1).

Every call goes to libpixelflow_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .config import Settings, read_porosity_csv, read_settings
from ._lib import PfOptions, PfParams, check

PRECISIONS = {"fp64": _lib.PF_PREC_FP64, "plain": _lib.PF_PREC_FP64, "mixed": _lib.PF_PREC_MIXED}
SWEEP_FORMS = {"auto": _lib.PF_SWEEP_AUTO, "split": _lib.PF_SWEEP_SPLIT, "fused": _lib.PF_SWEEP_FUSED}
SOR_PATHS = {"auto": _lib.PF_SOR_AUTO, "cells": _lib.PF_SOR_CELLS}


def make_params(s: Settings, shape: Sequence[int]) -> PfParams:
    dim = len(shape)
    m, n = int(shape[0]), int(shape[1])
    l = int(shape[2]) if dim == 3 else 1
    return PfParams(dim, m, n, l, s.xnue, s.xlambda, s.density, s.width, s.height, s.depth, s.time,
                    s.inlet_velocity, s.outlet_pressure, s.aoa, int(s.istep_max), int(s.iter_max),
                    s.thickness, s.threshold, s.relux_factor, 1 if s.nonslip else 0,
                    1 if s.inflow_porosity else 0, 1 if s.walls is not None else 0,
                    (ctypes.c_int32 * 6)(*(s.walls or (0,) * 6)), 1 if s.slip_y else 0)


def make_options(s: Settings, use_graph: bool = True) -> PfOptions:
    L = _lib.load()
    o = PfOptions()
    L.pf_default_options(ctypes.byref(o))
    prec = str(s.precision).lower()
    if prec not in PRECISIONS:
        raise ValueError(f"unknown precision {s.precision!r}")
    o.precision = PRECISIONS[prec]
    o.outer_max = int(s.outer_max)
    o.inner_sweeps = int(s.inner_sweeps)
    o.dc_tol = float(s.dc_tol)
    o.track_sor_error = 1 if s.track_sor_error else 0
    o.use_graph = 1 if use_graph else 0
    form = str(s.sweep_form).lower()
    if form not in SWEEP_FORMS:
        raise ValueError(f"unknown sweep_form {s.sweep_form!r}")
    o.sweep_form = SWEEP_FORMS[form]
    o.fused_rows = int(s.fused_rows)
    o.fused_planes = int(s.fused_planes)
    path = str(s.sor_path).lower()
    if path not in SOR_PATHS:
        raise ValueError(f"unknown sor_path {s.sor_path!r}")
    o.sor_path = SOR_PATHS[path]
    return o


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Case:
    """One case resident on the GPU."""

    def __init__(self, settings: Settings, shape: Sequence[int], porosity_values: np.ndarray,
                 use_graph: bool = True):
        self.L = _lib.load()
        self.settings = settings
        self.shape = tuple(int(x) for x in shape)
        self.dim = len(self.shape)
        if self.dim not in (2, 3):
            raise ValueError("shape must be (m, n) or (m, n, l)")
        self.m, self.n = self.shape[0], self.shape[1]
        self.l = self.shape[2] if self.dim == 3 else 1
        vals = np.ascontiguousarray(porosity_values, dtype=np.float64)
        expect = (self.n, self.m) if self.dim == 2 else (self.l, self.n, self.m)
        if vals.shape != expect:
            raise ValueError(f"porosity values must have shape {expect}, got {vals.shape}")
        self.params = make_params(settings, self.shape)
        self.options = make_options(settings, use_graph)
        h = ctypes.c_void_p()
        check(self.L.pf_create(ctypes.byref(self.params), ctypes.byref(self.options), _ptr(vals), ctypes.byref(h)))
        self.h = h
        self.field_shape = (self.n + 2, self.m + 2) if self.dim == 2 else (self.l + 2, self.n + 2, self.m + 2)

    @classmethod
    def from_shapes(cls, settings: Settings, shape: Sequence[int], shapes, edge: float = 1.0,
                    use_graph: bool = True) -> "Case":
        """A case whose porosity is generated on the GPU from analytic shapes."""
        from ._lib import PfShape
        from .geometry import to_pf_shapes
        self = cls.__new__(cls)
        self.L = _lib.load()
        self.settings = settings
        self.shape = tuple(int(x) for x in shape)
        self.dim = len(self.shape)
        self.m, self.n = self.shape[0], self.shape[1]
        self.l = self.shape[2] if self.dim == 3 else 1
        self.params = make_params(settings, self.shape)
        self.options = make_options(settings, use_graph)
        pfs = shapes if (shapes and isinstance(shapes[0], PfShape)) else to_pf_shapes(shapes, self.dim)
        arr = (PfShape * max(1, len(pfs)))(*pfs)
        h = ctypes.c_void_p()
        check(self.L.pf_create_shapes(ctypes.byref(self.params), ctypes.byref(self.options),
                                      ctypes.cast(arr, ctypes.c_void_p), len(pfs), float(edge), ctypes.byref(h)))
        self.h = h
        self.field_shape = (self.n + 2, self.m + 2) if self.dim == 2 else (self.l + 2, self.n + 2, self.m + 2)
        return self

    @classmethod
    def from_project(cls, project_dir: str, **kw) -> "Case":
        """Open a reference project directory: config/controlDict.txt + its porosity CSV."""
        s = read_settings(os.path.join(project_dir, "config", "controlDict.txt"))
        shape, vals = read_porosity_csv(os.path.join(project_dir, s.csv_file))
        return cls(s, shape, vals, **kw)

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            check(self.L.pf_destroy(self.h))
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

    # -- reference routines ------------------------------------------------
    def initial_conditions(self):
        """initial_conditions + boundary, as the main programs call them."""
        check(self.L.pf_initial_conditions(self.h))

    def solve_p(self):
        check(self.L.pf_solve_p(self.h))

    def projection(self):
        check(self.L.pf_projection(self.h))

    def boundary(self):
        check(self.L.pf_boundary(self.h))

    def step(self, nsteps: int = 1):
        check(self.L.pf_step(self.h, int(nsteps)))
        self.steps_done = getattr(self, "steps_done", 0) + int(nsteps)

    # -- checkpoint / restart ------------------------------------------------
    def save_checkpoint(self, path: str):
        """Everything a restart needs, in one .npz: the settings, the grid,
        the porosity values, the state with its ghost layers (the next step
        reads the lagged ghosts) and the number of steps taken.  A case
        restored from it continues bit for bit as the original would."""
        import dataclasses
        import json
        st = self.get_state()
        por = self.porosity()
        inner = por[1:-1, 1:-1] if self.dim == 2 else por[1:-1, 1:-1, 1:-1]
        np.savez(path, settings=json.dumps(dataclasses.asdict(self.settings)),
                 shape=np.array(self.shape), porosity=inner, steps_done=getattr(self, "steps_done", 0), **st)

    @classmethod
    def from_checkpoint(cls, path: str, **kw) -> "Case":
        import json
        with np.load(path, allow_pickle=False) as z:
            d = json.loads(str(z["settings"]))
            if d.get("walls") is not None:
                d["walls"] = tuple(d["walls"])
            s = Settings(**d)
            shape = tuple(int(x) for x in z["shape"])
            self = cls(s, shape, z["porosity"], **kw)
            self.set_state(z["u"], z["v"], z["p"], z["w"] if "w" in z.files else None)
            self.steps_done = int(z["steps_done"])
        return self

    def synchronize(self):
        check(self.L.pf_synchronize(self.h))

    def norms(self) -> Tuple[float, float]:
        """(max|div u| of the porosity-weighted divergence, SOR error of the last solve_p)."""
        md, se = ctypes.c_double(), ctypes.c_double()
        rc = self.L.pf_norms(self.h, ctypes.byref(md), ctypes.byref(se))
        if rc not in (_lib.PF_OK, -4):
            check(rc)
        return md.value, se.value

    # -- fields ------------------------------------------------------------
    def _check_field(self, a: np.ndarray) -> Tuple[int, int]:
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("fields must be C-contiguous float64 arrays")
        if a.ndim != self.dim:
            raise ValueError(f"fields must have {self.dim} axes")
        if self.dim == 3 and a.shape[0] != self.l + 2:
            raise ValueError("3D fields need l+2 planes")
        return a.shape[-1], a.shape[-2]

    def set_state(self, u: np.ndarray, v: np.ndarray, p: np.ndarray, w: Optional[np.ndarray] = None):
        ld1, ld2 = self._check_field(u)
        for a in (v, p) + ((w,) if self.dim == 3 else ()):
            if self._check_field(a) != (ld1, ld2):
                raise ValueError("all fields must share leading dimensions")
        check(self.L.pf_set_state(self.h, _ptr(u), _ptr(v), _ptr(w), _ptr(p), ld1, ld2))

    def get_state(self, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        if out is None:
            out = {k: np.empty(self.field_shape) for k in (("u", "v", "p") + (("w",) if self.dim == 3 else ()))}
        ld1, ld2 = self._check_field(out["u"])
        check(self.L.pf_get_state(self.h, _ptr(out["u"]), _ptr(out["v"]), _ptr(out.get("w")), _ptr(out["p"]),
                                  ld1, ld2))
        return out

    def step_host(self, state: Dict[str, np.ndarray], out: Optional[Dict[str, np.ndarray]] = None
                  ) -> Dict[str, np.ndarray]:
        """One step from the host fields in `state` to the host fields in `out`:
        the same result as set_state + step(1) + get_state, with the input
        copies overlapped with the first stages of the step where the case
        allows it (3D periodic plain FP64, dense host fields)."""
        if out is None:
            out = {k: np.empty(self.field_shape) for k in (("u", "v", "p") + (("w",) if self.dim == 3 else ()))}
        ld1, ld2 = self._check_field(state["u"])
        names = ("u", "v", "p") + (("w",) if self.dim == 3 else ())
        for k in names:
            if self._check_field(state[k]) != (ld1, ld2) or self._check_field(out[k]) != (ld1, ld2):
                raise ValueError("all fields must share leading dimensions")
        check(self.L.pf_step_host(self.h, _ptr(state["u"]), _ptr(state["v"]), _ptr(state.get("w")),
                                  _ptr(state["p"]), _ptr(out["u"]), _ptr(out["v"]), _ptr(out.get("w")),
                                  _ptr(out["p"]), ld1, ld2))
        self.steps_done = getattr(self, "steps_done", 0) + 1
        return out

    def snapshot_begin(self):
        """Start copying the state as of the last enqueued step to the host
        without waiting (the copy overlaps the steps enqueued after it)."""
        check(self.L.pf_snapshot_begin(self.h))

    def snapshot_wait(self, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        """The state captured by the last snapshot_begin (waits for its copy)."""
        if out is None:
            out = {k: np.empty(self.field_shape) for k in (("u", "v", "p") + (("w",) if self.dim == 3 else ()))}
        ld1, ld2 = self._check_field(out["u"])
        check(self.L.pf_snapshot_wait(self.h, _ptr(out["u"]), _ptr(out["v"]), _ptr(out.get("w")), _ptr(out["p"]),
                                      ld1, ld2))
        return out

    def porosity(self) -> np.ndarray:
        a = np.empty(self.field_shape)
        check(self.L.pf_get_porosity(self.h, _ptr(a), a.shape[-1], a.shape[-2]))
        return a

    def forces(self, radius: Optional[float] = None) -> Dict[str, np.ndarray]:
        """The reference's force log (output_force_log_2d/_3d): pressure part
        Fp, wall-friction part Fv and F = Fp + Fv (x, y[, z]); with `radius`
        also the coefficients F/(density * inlet_velocity^2 * radius) as
        Cd, Cl (2D) or Cd_x, Cl, Cd_z (3D)."""
        fp = (ctypes.c_double * 3)()
        fv = (ctypes.c_double * 3)()
        check(self.L.pf_forces(self.h, fp, fv))
        d = self.dim
        out = {"Fp": np.array(fp[:d]), "Fv": np.array(fv[:d])}
        out["F"] = out["Fp"] + out["Fv"]
        if radius is not None:
            ref = self.settings.density * self.settings.inlet_velocity ** 2 * radius
            c = out["F"] / ref
            if d == 2:
                out["Cd"], out["Cl"] = float(c[0]), float(c[1])
            else:
                out["Cd_x"], out["Cl"], out["Cd_z"] = float(c[0]), float(c[1]), float(c[2])
        return out

    def kernel_launches(self) -> int:
        n = ctypes.c_int64()
        check(self.L.pf_kernel_launches(self.h, ctypes.byref(n)))
        return n.value

    def profile_step_times(self, max_steps: int = 1 << 20) -> np.ndarray:
        n = ctypes.c_int64()
        buf = np.zeros(max_steps)
        check(self.L.pf_profile_step_times(self.h, _ptr(buf), max_steps, ctypes.byref(n)))
        return buf[: n.value].copy()

    def sweep_info(self) -> Dict[str, object]:
        """The precision form's FP32 sweep: {"form": "fused" | "split",
        "split_ms", "fused_ms"} (per sweep, measured at creation when the form
        was chosen automatically, else 0)."""
        f, a, b = ctypes.c_int(), ctypes.c_float(), ctypes.c_float()
        check(self.L.pf_sweep_info(self.h, ctypes.byref(f), ctypes.byref(a), ctypes.byref(b)))
        return {"form": "fused" if f.value else "split", "split_ms": a.value, "fused_ms": b.value}

    def sor_info(self) -> Dict[str, object]:
        """The plain sweep's path: {"listed": bool, "fluid": [c0, c1],
        "total": [c0, c1]} -- listed when the SOR walks cell lists with the
        pure-fluid cells first (3D plain FP64, sor_path "auto")."""
        li = ctypes.c_int()
        fl = (ctypes.c_int * 2)()
        tot = (ctypes.c_int * 2)()
        check(self.L.pf_sor_info(self.h, ctypes.byref(li), fl, tot))
        return {"listed": bool(li.value), "fluid": list(fl), "total": list(tot)}

    def dc_list_info(self) -> Dict[str, object]:
        """The precision form's split FP32 sweep: {"listed": bool, "fluid":
        [c0, c1], "total": [c0, c1]} -- listed when it walks chunk lists with
        the all-fluid chunks apart (3D, sor_path "auto", grids of more than
        one wave)."""
        li = ctypes.c_int()
        fl = (ctypes.c_int * 2)()
        tot = (ctypes.c_int * 2)()
        check(self.L.pf_dc_list_info(self.h, ctypes.byref(li), fl, tot))
        return {"listed": bool(li.value), "fluid": list(fl), "total": list(tot)}

    def memory_bytes(self) -> int:
        b = ctypes.c_size_t()
        check(self.L.pf_memory_bytes(self.h, ctypes.byref(b)))
        return b.value

    # -- profiling -----------------------------------------------------------
    def profile_begin(self):
        check(self.L.pf_profile_begin(self.h))

    def profile_end(self) -> Dict[str, float]:
        sor, st = ctypes.c_double(), ctypes.c_double()
        nl, ns = ctypes.c_int64(), ctypes.c_int64()
        check(self.L.pf_profile_end(self.h, ctypes.byref(sor), ctypes.byref(nl), ctypes.byref(st), ctypes.byref(ns)))
        return dict(sor_ms=sor.value, sor_launches=nl.value, step_ms=st.value, steps=ns.value)

    def profile_stages(self) -> Dict[str, float]:
        """Device time (ms, summed over the last profiling session's steps)
        of the step's stages: divergence + predictor, RHS, SOR (all passes),
        projection + boundary."""
        ms = np.zeros(4)
        check(self.L.pf_profile_stages(self.h, _ptr(ms)))
        return dict(zip(("predictor", "rhs", "sor", "projection_boundary"), ms.tolist()))


def host_register(a: np.ndarray):
    check(_lib.load().pf_host_register(_ptr(a), a.nbytes))


def host_unregister(a: np.ndarray):
    check(_lib.load().pf_host_unregister(_ptr(a)))
