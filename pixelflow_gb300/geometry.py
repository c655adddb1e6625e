"""Synthetic porosity fields for the benchmark and test geometries.

Porosity follows the reference's preprocessing tools: a tanh profile of the
signed distance to the solid, ``0.5*tanh(sdf/thickness) + 0.5`` with sdf in
cells and positive in the fluid (tools/cylinder/make_porosity_2d_cylinder.py:
119-122, tools/channel/channel.py:27).  Here sdf is computed in physical units
and divided by ``edge*dx``.  ``edge`` is the half-width of the transition in
cells: the profile rises from 0.12 to 0.88 over |sdf| <= edge, so the
benchmark's "tanh transition of width 2 cells" is edge = 1.  (With a wider
tail the solid core of a small obstacle is not clamped to the threshold and
the reference scheme itself diverges within ~100 steps of the 2D cylinder
case; edge = 1 keeps the core at the threshold as the reference's own
cylinder fixture does.)  Nodes sit at x_i = (i-1)*dx with
dx = width/(m-1) (lib/grid.f90:50,82).  Several obstacles combine by the
minimum of their signed distances.  The clamp ``max(value, threshold)`` is
applied later at ingest, as grid.f90:43 does.

All random draws use ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .config import Settings


def tanh_porosity(sdf: np.ndarray, edge: float, dx: float) -> np.ndarray:
    return 0.5 * np.tanh(sdf / (edge * dx)) + 0.5


def node_coords(count: int, length: float) -> np.ndarray:
    d = length / (count - 1)
    return np.arange(count, dtype=np.float64) * d


def cylinder_2d(m: int = 512, n: int = 256, width: float = 2.0, height: float = 1.0,
                cx: float = 0.5, cy: float = 0.5, radius: float = 0.05,
                edge: float = 1.0) -> np.ndarray:
    """Circle of `radius` at (cx, cy): porosity values, shape (n, m)."""
    x = node_coords(m, width)
    y = node_coords(n, height)
    dx = width / (m - 1)
    sdf = np.sqrt((x[None, :] - cx) ** 2 + (y[:, None] - cy) ** 2) - radius
    return tanh_porosity(sdf, edge, dx)


def _ellipse_sdf(X: np.ndarray, Y: np.ndarray, cx: float, cy: float, a: float, b: float,
                 angle: float) -> np.ndarray:
    """First-order signed distance to a rotated ellipse, (q-1)/|grad q|."""
    c, s = np.cos(angle), np.sin(angle)
    xr = (X - cx) * c + (Y - cy) * s
    yr = -(X - cx) * s + (Y - cy) * c
    q = np.sqrt((xr / a) ** 2 + (yr / b) ** 2)
    g = np.sqrt((xr / (a * a)) ** 2 + (yr / (b * b)) ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        d = np.where(g > 0, (q - 1.0) * q / np.where(g > 0, g, 1.0), -min(a, b))
    return d


def obstacles_2d(m: int, n: int, width: float, height: float,
                 shapes: Sequence[Tuple[float, float, float, float, float]],
                 edge: float = 1.0) -> np.ndarray:
    """Union of ellipses (cx, cy, a, b, angle); circles have a == b."""
    x = node_coords(m, width)
    y = node_coords(n, height)
    X, Y = np.meshgrid(x, y)
    sdf = np.full((n, m), np.inf)
    for (cx, cy, a, b, ang) in shapes:
        if a == b:
            d = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - a
        else:
            d = _ellipse_sdf(X, Y, cx, cy, a, b, ang)
        sdf = np.minimum(sdf, d)
    return tanh_porosity(sdf, edge, width / (m - 1))


def random_spheres(count: int, seed: int = 0, cmin: float = 0.15, cmax: float = 0.85,
                   rmin: float = 0.03, rmax: float = 0.08) -> np.ndarray:
    """(count, 4) array of sphere centres and radii in the unit cube."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(cmin, cmax, size=(count, 3))
    radii = rng.uniform(rmin, rmax, size=(count, 1))
    return np.concatenate([centres, radii], axis=1)


def spheres_3d(m: int = 256, n: int = 256, l: int = 256, width: float = 1.0, height: float = 1.0,
               depth: float = 1.0, spheres: np.ndarray | None = None, count: int = 32,
               seed: int = 0, edge: float = 1.0) -> np.ndarray:
    """Union of spheres: porosity values, shape (l, n, m), built plane by plane."""
    if spheres is None:
        spheres = random_spheres(count, seed)
    x = node_coords(m, width)
    y = node_coords(n, height)
    z = node_coords(l, depth)
    dx = width / (m - 1)
    out = np.empty((l, n, m), dtype=np.float64)
    dxy = [(x[None, :] - s[0]) ** 2 + (y[:, None] - s[1]) ** 2 for s in spheres]
    for k in range(l):
        sdf = np.full((n, m), np.inf)
        for s, d2 in zip(spheres, dxy):
            sdf = np.minimum(sdf, np.sqrt(d2 + (z[k] - s[2]) ** 2) - s[3])
        out[k] = tanh_porosity(sdf, edge, dx)
    return out


# --------------------------------------------------------------------------
# Benchmark configurations.
# --------------------------------------------------------------------------

def settings_cylinder_2d(**kw) -> Settings:
    """2D flow past a cylinder, 512x256, Re=100, dt=2e-4, 1000 steps."""
    s = Settings(xnue=1e-3, xlambda=0.0, density=1.0, width=2.0, height=1.0, depth=0.0,
                 time=0.2, inlet_velocity=1.0, outlet_pressure=0.0, aoa=0.0,
                 istep_max=1000, istep_out=100000, thickness=2.0, threshold=1e-6,
                 radius=0.05, center_x=0.25, center_y=0.5, nonslip=True,
                 iter_max=100, relux_factor=1.7)
    return s.replace(**kw)


def settings_spheres_3d(**kw) -> Settings:
    """3D unit cube with seeded spheres, nu=1e-3, dt=1e-4, 200 steps."""
    s = Settings(xnue=1e-3, xlambda=0.0, density=1.0, width=1.0, height=1.0, depth=1.0,
                 time=0.02, inlet_velocity=1.0, outlet_pressure=0.0, aoa=0.0,
                 istep_max=200, istep_out=100000, thickness=2.0, threshold=1e-6,
                 radius=0.05, nonslip=True, iter_max=100, relux_factor=1.7)
    return s.replace(**kw)


def cfl_dt(h: float, nu: float, u: float = 1.0, dim: int = 2, cfl: float = 0.2) -> float:
    """Time step at Courant number `cfl` of the explicit predictor's full
    stability limit.  Forward Euler on central advection plus diffusion is
    stable (von Neumann) only for dt <= h/|u| (advection), dt <= 2 nu/|u|^2
    (the central advection term needs viscous damping) and
    dt <= h^2/(2 dim nu) (diffusion); dt = cfl * the smallest of the three.
    The plain advective CFL dt = cfl*h/u alone leaves dt*u^2/nu between 1.5
    and 10 for Re 50-400 on these grids."""
    return cfl * min(h / u, 2.0 * nu / (u * u), h * h / (2.0 * dim * nu))


def grid_nu(nu: float, h: float, u: float = 1.0, cell_re: float = 2.0) -> float:
    """Viscosity raised, where needed, to cell Reynolds number u*h/nu <= cell_re.
    The reference scheme's growth there is a property of the spatial
    discretisation, not of dt: in the restated step the 2D cylinder at
    256x128 (nu = 1e-3, cell Re 7.8) diverges at the same physical time
    (t ~ 0.0075) for dt = 1e-4 and 5e-5, and stays bounded at nu = 4e-3."""
    return max(nu, u * h / cell_re)


def _fit_streamwise(a: float, b: float, cx: float, width: float) -> Tuple[float, float, float]:
    """Semi-axes scaled so the larger is at most width/4 and the centre moved
    so the obstacle (a circle of its larger semi-axis) stays width/10 clear
    of the inlet and outlet; unchanged when it already fits."""
    r = max(a, b)
    rmax = 0.25 * width
    if r > rmax:
        a, b, r = a * rmax / r, b * rmax / r, rmax
    lo, hi = r + 0.1 * width, width - r - 0.1 * width
    return a, b, min(max(cx, lo), hi)


@dataclasses.dataclass
class BatchCase2D:
    m: int
    n: int
    settings: Settings
    shapes: List[Tuple[float, float, float, float, float]]

    def porosity(self) -> np.ndarray:
        return obstacles_2d(self.m, self.n, self.settings.width, self.settings.height, self.shapes)


def batch_cases_2d(count: int = 512, seed: int = 0, steps: int = 500,
                   sizes: Sequence[int] = tuple(range(64, 513, 32)),
                   iter_max: int = 100, threshold: float = 0.1, cell_re: Optional[float] = 2.0,
                   dt_rule: str = "stable", fit_streamwise: bool = True) -> List[BatchCase2D]:
    """Independent 2D cases of uneven size: nx, ny from `sizes`, 1-4 circles or
    ellipses with semi-axes 0.02-0.1 of the height at random angles, Re uniform
    in [50, 400] (nu = U*D/Re with D twice the first obstacle's larger
    semi-axis), unit inflow, square cells.

    Stability of the reference scheme sets three choices (each checked with
    the FP64 oracle over 500 steps):
    * `threshold`, the namelist porosity floor (&porosity_control; the
      template's 1e-6): with 1e-6 a third of the cases overflow within 40
      steps, from the first step on -- the pressure solve leaves large
      gradients inside the solid cores, where the non-slip damping
      eps(1-eps)^2 vanishes, and the advection term then squares the velocity
      there every step.  0.1 keeps every case finite;
    * `cell_re`: nu is raised where needed to cell Reynolds number
      U*h/nu <= cell_re (`grid_nu`); None keeps nu = U*D/Re, under which half
      of the cases still diverge with threshold 0.1;
    * `dt_rule`: "stable" takes CFL 0.2 of the predictor's full stability
      limit (`cfl_dt`); "cfl" the plain advective 0.2*h/U, which diverges
      for most cases;
    * `fit_streamwise`: in domains much shorter than high (nx = 64 with ny
      up to 512) an obstacle of 0.1 height reaches the inlet and outlet rows,
      and those cases diverge even with the two choices above; its semi-axes
      are then scaled so its largest one is at most a quarter of the width
      and its centre kept a tenth of the width clear of both ends
      (`_fit_streamwise`).  The random draws are the same either way."""
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(count):
        m = int(rng.choice(sizes))
        n = int(rng.choice(sizes))
        height = 1.0
        h = height / (n - 1)
        width = h * (m - 1)
        nobs = int(rng.integers(1, 5))
        shapes = []
        for _o in range(nobs):
            a = float(rng.uniform(0.02, 0.1)) * height
            circle = bool(rng.integers(0, 2))
            b = a if circle else float(rng.uniform(0.02, 0.1)) * height
            ang = float(rng.uniform(0.0, np.pi))
            cx = float(rng.uniform(0.2, 0.8)) * width
            cy = float(rng.uniform(0.2, 0.8)) * height
            if fit_streamwise:
                a, b, cx = _fit_streamwise(a, b, cx, width)
            shapes.append((cx, cy, a, b, ang))
        re = float(rng.uniform(50.0, 400.0))
        d_ref = 2.0 * max(shapes[0][2], shapes[0][3])
        u_in = 1.0
        nu = u_in * d_ref / re
        if cell_re is not None:
            nu = grid_nu(nu, h, u_in, cell_re)
        dt = cfl_dt(h, nu, u_in, 2) if dt_rule == "stable" else 0.2 * h / u_in
        s = Settings(xnue=nu, xlambda=0.0, density=1.0, width=width, height=height, depth=0.0,
                     time=dt * steps, inlet_velocity=u_in, outlet_pressure=0.0, aoa=0.0,
                     istep_max=steps, istep_out=10 ** 9, thickness=2.0, threshold=threshold,
                     radius=d_ref / 2, nonslip=True, iter_max=iter_max, relux_factor=1.7,
                     precision="mixed")
        cases.append(BatchCase2D(m, n, s, shapes))
    return cases


# --------------------------------------------------------------------------
# Shape lists for the GPU geometry generator (pf_create_shapes).
# --------------------------------------------------------------------------

def to_pf_shapes(shapes, dim: int):
    """Shapes as pf_shape structs: 2D (cx, cy, a, b, angle) tuples -> circles
    or ellipses; 3D (cx, cy, cz, r) rows -> spheres."""
    from ._lib import PF_SHAPE_CIRCLE, PF_SHAPE_ELLIPSE, PF_SHAPE_SPHERE, PfShape
    out = []
    for sh in shapes:
        if dim == 2:
            cx, cy, a, b, ang = sh
            kind = PF_SHAPE_CIRCLE if a == b else PF_SHAPE_ELLIPSE
            out.append(PfShape(kind, 0, float(cx), float(cy), 0.0, float(a), float(b), float(ang)))
        else:
            cx, cy, cz, r = sh
            out.append(PfShape(PF_SHAPE_SPHERE, 0, float(cx), float(cy), float(cz), float(r), float(r), 0.0))
    return out


@dataclasses.dataclass
class Request:
    rid: int
    arrival_s: float
    dim: int
    shape: Tuple[int, ...]
    settings: Settings
    shapes: list
    steps: int

    @property
    def cells(self) -> int:
        c = 1
        for x in self.shape:
            c *= x
        return c


def serving_requests(count: int = 64, rate: float = 200.0, seed: int = 0, frac_2d: float = 0.7,
                     sizes_2d: Sequence[int] = tuple(range(128, 1025, 32)),
                     sizes_3d: Sequence[int] = (64, 96, 128, 160, 192),
                     steps_range: Tuple[int, int] = (100, 1000), threshold: float = 0.1) -> List[Request]:
    """Poisson arrivals (exponential gaps, mean 1/rate) of mixed cases.
    2D: n x n unit squares, 1-4 circles/ellipses (semi-axes 0.02-0.1),
    Re 50-400 on the first obstacle's diameter.  3D: n^3 unit cubes, 4-16
    spheres (radii 0.03-0.08, centres in [0.15, 0.85]^3), nu 2e-3..1e-2.
    Unit inflow; nu raised to cell Reynolds number <= 2 (`grid_nu`); dt at
    CFL 0.2 of the full stability limit (`cfl_dt`); porosity threshold 0.1
    (see `batch_cases_2d` for these three choices).
    Steps per request uniform in steps_range."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += float(rng.exponential(1.0 / rate))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        if rng.random() < frac_2d:
            n = int(rng.choice(sizes_2d))
            h = 1.0 / (n - 1)
            nobs = int(rng.integers(1, 5))
            shapes = []
            for _o in range(nobs):
                a = float(rng.uniform(0.02, 0.1))
                b = a if bool(rng.integers(0, 2)) else float(rng.uniform(0.02, 0.1))
                shapes.append((float(rng.uniform(0.2, 0.8)), float(rng.uniform(0.2, 0.8)), a, b,
                               float(rng.uniform(0.0, np.pi))))
            re = float(rng.uniform(50.0, 400.0))
            nu = grid_nu(2.0 * max(shapes[0][2], shapes[0][3]) / re, h)
            dt = cfl_dt(h, nu, 1.0, 2)
            s = Settings(xnue=nu, width=1.0, height=1.0, depth=0.0, time=dt * steps, inlet_velocity=1.0,
                         istep_max=steps, istep_out=10 ** 9, thickness=2.0, threshold=threshold, nonslip=True,
                         iter_max=100, relux_factor=1.7, precision="mixed")
            out.append(Request(rid, t, 2, (n, n), s, shapes, steps))
        else:
            n = int(rng.choice(sizes_3d))
            h = 1.0 / (n - 1)
            ns = int(rng.integers(4, 17))
            sph = random_spheres(ns, seed=int(rng.integers(0, 2 ** 31)))
            nu = grid_nu(float(rng.uniform(2e-3, 1e-2)), h)
            dt = cfl_dt(h, nu, 1.0, 3)
            s = Settings(xnue=nu, width=1.0, height=1.0, depth=1.0, time=dt * steps, inlet_velocity=1.0,
                         istep_max=steps, istep_out=10 ** 9, thickness=2.0, threshold=threshold, nonslip=True,
                         iter_max=100, relux_factor=1.7, precision="mixed")
            out.append(Request(rid, t, 3, (n, n, n), s, [tuple(r) for r in sph], steps))
    return out
