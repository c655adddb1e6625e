"""Reference-compatible inputs: controlDict namelists and porosity CSV files.

`read_settings` reads the seven namelist groups of config/controlDict.txt in
the order PixelFlow reads them (src/omp_parallel/lib/global.f90:47-62) and an
optional trailing ``&gpu_control`` group that only this library reads (the
reference stops after ``&solver_control``, so the extra group keeps the file
usable by the reference).

`read_porosity_csv` parses the porosity file format of grid.f90:36-47 (2D)
and :281-294 (3D): a header line ``m,n[,l]`` followed by one
``i,j,k,value`` record per cell with i fastest.
"""
from __future__ import annotations

import dataclasses
import re
from typing import Dict, Optional, Tuple

import numpy as np

# Namelist groups and their members, global.f90:47-54.
GROUPS = {
    "physical": ["xnue", "xlambda", "density", "width", "height", "depth", "time",
                 "inlet_velocity", "outlet_pressure", "aoa"],
    "file_control": ["istep_out"],
    "grid_control": ["istep_max"],
    "porosity_control": ["thickness", "threshold", "radius", "center_x", "center_y", "center_z"],
    "calculation_method": ["nonslip"],
    "directory_control": ["output_folder", "csv_file"],
    "solver_control": ["iter_max", "relux_factor"],
}
GPU_GROUP = "gpu_control"
GPU_KEYS = ["precision", "outer_max", "inner_sweeps", "dc_tol", "track_sor_error", "inflow_porosity", "walls",
            "sweep_form", "fused_rows", "fused_planes", "sor_path", "slip_y"]
WALL_FACES = ("top", "bottom", "east", "west", "north", "south")


@dataclasses.dataclass
class Settings:
    """Namelist values (global.f90:18-26), defaults from template/config/controlDict.txt."""
    xnue: float = 0.001
    xlambda: float = 0.0
    density: float = 1.0
    width: float = 1.0
    height: float = 1.0
    depth: float = 1.0
    time: float = 1.0
    inlet_velocity: float = 0.1
    outlet_pressure: float = 0.0
    aoa: float = 0.0
    istep_out: int = 1001
    istep_max: int = 100
    thickness: float = 1.5
    threshold: float = 1.0e-6
    radius: float = 0.1
    center_x: float = 0.5
    center_y: float = 0.5
    center_z: float = 0.5
    nonslip: bool = True
    output_folder: str = "output"
    csv_file: str = "data/porosity.csv"
    iter_max: int = 100
    relux_factor: float = 1.7
    # &gpu_control (this library only)
    precision: str = "fp64"          # "fp64" (plain) | "mixed" (FP32 sweeps + FP64 defect correction)
    outer_max: int = 4               # mixed: defect-correction passes per step
    inner_sweeps: int = 25           # mixed: FP32 SOR iterations per pass
    dc_tol: float = 0.0              # mixed: stop the passes once max|r| <= dc_tol (0: run all)
    track_sor_error: bool = True     # keep the reference's SOR max-change diagnostic
    # mixed: "split" runs one launch per colour of an FP32 sweep, "fused" both
    # colours in one launch where the case allows it (3D, even n and l),
    # "auto" times both on the case when it is created and keeps the faster;
    # the results are the same bit for bit.  fused_rows / fused_planes: the
    # fused sweep's rows per tile and cap on (tile, plane) pairs per CTA (0:
    # chosen from the grid and the device)
    sweep_form: str = "auto"
    fused_rows: int = 0
    fused_planes: int = 0
    # plain FP64, 3D: "auto" walks cell lists with the pure-fluid cells first
    # (exact neighbour sum, no coefficient loads for them); "cells" updates
    # every cell with its own stored coefficients
    sor_path: str = "auto"
    # inflow and initial velocities scaled by porosity: the boundary and initial
    # conditions of ibm_2d_backstep_omp_cpu.f90 (:533-534, :615-618)
    inflow_porosity: bool = False
    # the air-condition program (3D): its wall table, one entry per face in the
    # order top, bottom, east, west, north, south, each 0 wall, 1 inlet,
    # 2 outlet (ibm_3d_air_condition_omp_cpu.f90:4-16); None: the uniform
    # programs' x inflow/outflow with periodic y and z.  In a namelist:
    # walls = "1,0,0,0,0,2".
    walls: Optional[Tuple[int, ...]] = None
    # 2D, plain FP64: symmetry rows at j = 1 and j = n ("slip" top and bottom:
    # dp/dy = 0, v = 0, u mirrored into the ghost row) in place of the periodic
    # wrap, the option ibm_2d_uniform_omp_cpu.f90 keeps commented out
    # (:438-450, :503-518)
    slip_y: bool = False

    def replace(self, **kw) -> "Settings":
        return dataclasses.replace(self, **kw)


_TOKEN = re.compile(r"""\s*([A-Za-z_][A-Za-z0-9_]*)\s*=\s*("[^"]*"|'[^']*'|[^,\s/]+)\s*,?""")


def _convert(value: str):
    v = value.strip()
    if v[:1] in "\"'":
        return v[1:-1]
    low = v.lower()
    if low in (".true.", "t", ".t.", "true"):
        return True
    if low in (".false.", "f", ".f.", "false"):
        return False
    try:
        if re.fullmatch(r"[+-]?\d+", v):
            return int(v)
        return float(low.replace("d", "e"))
    except ValueError as exc:  # same failure the Fortran runtime raises on a bad value
        raise ValueError(f"namelist: cannot parse value {value!r}") from exc


def _outside_quotes(line: str, ch: str) -> int:
    """Index of the first `ch` outside a quoted string, or -1."""
    q = None
    for k, c in enumerate(line):
        if q:
            if c == q:
                q = None
        elif c in "\"'":
            q = c
        elif c == ch:
            return k
    return -1


def parse_namelists(text: str) -> Dict[str, Dict[str, object]]:
    """Parse Fortran namelist groups (``&name ... /``): ``!`` starts a
    comment and ``/`` ends the group, both outside quoted strings."""
    groups: Dict[str, Dict[str, object]] = {}
    current: Optional[str] = None
    for raw in text.splitlines():
        bang = _outside_quotes(raw, "!")
        line = raw if bang < 0 else raw[:bang]
        if not line.strip():
            continue
        stripped = line.strip()
        if current is None:
            if stripped.startswith("&"):
                current = stripped[1:].split()[0].lower()
                groups.setdefault(current, {})
                rest = stripped[1 + len(current):]
                line = rest
            else:
                continue
        end = False
        slash = _outside_quotes(line, "/")
        if slash >= 0:
            line, end = line[:slash], True
        for m in _TOKEN.finditer(line):
            groups[current][m.group(1).lower()] = _convert(m.group(2))
        if end:
            current = None
    return groups


def read_settings(path: str) -> Settings:
    """Read controlDict.txt like read_settings (global.f90:28-92).

    Every one of the seven reference groups must be present, as the Fortran
    ``read(11,nml=...)`` sequence requires; unknown members are an error.
    """
    with open(path, "r") as f:
        groups = parse_namelists(f.read())
    s = Settings()
    for g, keys in GROUPS.items():
        if g not in groups:
            raise ValueError(f"{path}: namelist group &{g} missing")
        for k, v in groups[g].items():
            if k not in keys:
                raise ValueError(f"{path}: &{g} has no member {k!r}")
            setattr(s, k, v)
    if GPU_GROUP in groups:
        for k, v in groups[GPU_GROUP].items():
            if k not in GPU_KEYS:
                raise ValueError(f"{path}: &{GPU_GROUP} has no member {k!r}")
            setattr(s, k, v)
    if isinstance(s.walls, str):
        s.walls = parse_walls(s.walls)
    s.nonslip = bool(s.nonslip)
    s.istep_max = int(s.istep_max)
    s.iter_max = int(s.iter_max)
    return s


def parse_walls(text: str) -> Optional[Tuple[int, ...]]:
    """"1,0,0,0,0,2" -> (1, 0, 0, 0, 0, 2); "" -> None."""
    parts = [x for x in re.split(r"[,\s]+", text.strip()) if x]
    if not parts:
        return None
    vals = tuple(int(x) for x in parts)
    if len(vals) != 6 or any(v not in (0, 1, 2) for v in vals):
        raise ValueError(f"walls: six entries of 0, 1 or 2 expected, got {text!r}")
    return vals


def write_settings(path: str, s: Settings, gpu_group: bool = False) -> None:
    """Write a controlDict.txt the reference can read."""
    def fmt(v):
        if isinstance(v, bool):
            return ".true." if v else ".false."
        if isinstance(v, str):
            return f'"{v}"'
        if v is None:
            return '""'
        if isinstance(v, tuple):
            return '"' + ",".join(str(int(x)) for x in v) + '"'
        if isinstance(v, int):
            return str(v)
        return repr(float(v))
    lines = []
    for g, keys in GROUPS.items():
        lines.append(f"&{g}")
        for k in keys:
            lines.append(f"{k} = {fmt(getattr(s, k))}")
        lines.append("/")
    if gpu_group:
        lines.append(f"&{GPU_GROUP}")
        for k in GPU_KEYS:
            lines.append(f"{k} = {fmt(getattr(s, k))}")
        lines.append("/")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_porosity_csv(path: str) -> Tuple[Tuple[int, ...], np.ndarray]:
    """Return ((m, n[, l]), values) from a porosity CSV (grid.f90:36-47, :281-294).

    ``values`` is float64 with shape (n, m) for 2D files (header ``m,n,1``) and
    (l, n, m) for 3D ones, indexed [k-1, j-1, i-1] from the records' own
    indices.  The reference stores each record at porosity(x,y[,z]); the
    same is done here, so records may come in any order.
    """
    with open(path, "r") as f:
        header = f.readline()
        dims = [int(float(t)) for t in header.replace(",", " ").split()]
        data = np.loadtxt(f, delimiter=",", dtype=np.float64, ndmin=2)
    if len(dims) == 2 or (len(dims) == 3 and dims[2] == 1):
        m, n = dims[0], dims[1]
        out = np.zeros((n, m), dtype=np.float64)
        idx = data[:, :2].astype(np.int64)
        out[idx[:, 1] - 1, idx[:, 0] - 1] = data[:, -1]
        return (m, n), out
    m, n, l = dims[:3]
    out = np.zeros((l, n, m), dtype=np.float64)
    idx = data[:, :3].astype(np.int64)
    out[idx[:, 2] - 1, idx[:, 1] - 1, idx[:, 0] - 1] = data[:, -1]
    return (m, n, l), out


def write_porosity_csv(path: str, values: np.ndarray) -> None:
    """Write values (shape (n,m) or (l,n,m)) in the reference CSV format, as
    the reference's own writer lays it out (tools/output/output_porosity.py:
    header without spaces, records "i, j, k, value" with ten decimals, i
    fastest): the same values give the same bytes."""
    if values.ndim == 2:
        n, m = values.shape
        jj, ii = np.meshgrid(np.arange(1, n + 1), np.arange(1, m + 1), indexing="ij")
        kk = np.ones_like(ii)
        header = f"{m},{n},1"
    else:
        l, n, m = values.shape
        kk, jj, ii = np.meshgrid(np.arange(1, l + 1), np.arange(1, n + 1), np.arange(1, m + 1), indexing="ij")
        header = f"{m},{n},{l}"
    rec = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1)
    with open(path, "w") as f:
        f.write(header + "\n")
        for (a, b, c), v in zip(rec, values.ravel()):
            f.write(f"{a}, {b}, {c}, {v:.10f}\n")
