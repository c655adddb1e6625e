"""Independent numpy restatement of the reference step -- TEST INFRASTRUCTURE ONLY.

A second, vectorised statement of the same reference routines as
pf_oracle.c, written from the Fortran independently of the C file: whole-array
slicing instead of loops, and red-black colours chosen by the parity
predicate ((i+j) odd first in 2D, (i+j+k) even first in 3D) instead of the
reference's linear-index mapping.  numpy evaluates each binary operation
separately in IEEE arithmetic, so with the same operation order it must agree
with the C restatement bit for bit.  Used only by tests, at small sizes.

Arrays: 2D (n+2, m+2), 3D (l+2, n+2, m+2), index [k, j, i] = Fortran (i, j, k).
"""
from __future__ import annotations

import numpy as np


class NpCase:
    def __init__(self, settings, shape, porosity_values, dtype=np.float64):
        self.dim = len(shape)
        self.T = np.dtype(dtype).type
        T = self.T
        s = settings
        if self.dim == 2:
            self.m, self.n = shape
            self.l = 1
            self.shape = (self.n + 2, self.m + 2)
        else:
            self.m, self.n, self.l = shape
            self.shape = (self.l + 2, self.n + 2, self.m + 2)
        m, n, l = self.m, self.n, self.l
        self.xnue, self.xlambda, self.density = T(s.xnue), T(s.xlambda), T(s.density)
        self.thickness, self.relux = T(s.thickness), T(s.relux_factor)
        self.U, self.pout, self.aoa = T(s.inlet_velocity), T(s.outlet_pressure), T(s.aoa)
        self.nonslip, self.iter_max = bool(s.nonslip), int(s.iter_max)
        # backstep program: inflow and initial velocity times porosity
        self.inflow_porosity = bool(getattr(s, "inflow_porosity", False))
        # air-condition program: wall table (top, bottom, east, west, north, south)
        walls = getattr(s, "walls", None)
        self.wall_mode = self.dim == 3 and walls is not None
        self.walls = tuple(int(x) for x in walls) if self.wall_mode else None
        # 2D symmetry rows at j = 1 and j = n (ibm_2d_uniform_omp_cpu.f90 keeps
        # them commented out: :440-450, :512-526)
        self.slip_y = self.dim == 2 and bool(getattr(s, "slip_y", False))
        # grid.f90:50-52 / :297-300
        self.dx = T(s.width) / T(m - 1)
        self.dy = T(s.height) / T(n - 1)
        self.dz = T(s.depth) / T(l - 1) if self.dim == 3 else T(0)
        self.dt = T(s.time) / T(int(s.istep_max))
        # porosity with ghosts (grid.f90)
        po = np.zeros(self.shape, dtype=dtype)
        vals = np.maximum(np.asarray(porosity_values, dtype=dtype), T(s.threshold))
        if self.dim == 2:
            po[1:n + 1, 1:m + 1] = vals
            po[1:n + 2, 0] = po[1:n + 2, 1]
            po[1:n + 2, m + 1] = po[1:n + 2, m]
            po[0, :] = po[n, :]
            po[n + 1, :] = po[1, :]
        elif self.wall_mode:  # grid_conditions_wall (grid.f90:208-244): copies x, y, z
            po[1:l + 1, 1:n + 1, 1:m + 1] = vals
            po[:, :, 0] = po[:, :, 1]
            po[:, :, m + 1] = po[:, :, m]
            po[:, 0, :] = po[:, 1, :]
            po[:, n + 1, :] = po[:, n, :]
            po[0, :, :] = po[1, :, :]
            po[l + 1, :, :] = po[l, :, :]
        else:
            po[1:l + 1, 1:n + 1, 1:m + 1] = vals
            po[1:l + 2, 1:n + 2, 0] = po[1:l + 2, 1:n + 2, 1]
            po[1:l + 2, 1:n + 2, m + 1] = po[1:l + 2, 1:n + 2, m]
            po[:, 0, :] = po[:, n, :]
            po[:, n + 1, :] = po[:, 1, :]
            po[0, :, :] = po[l, :, :]
            po[l + 1, :, :] = po[1, :, :]
        self.poro = po
        z = lambda: np.zeros(self.shape, dtype=dtype)
        self.u, self.v, self.p = z(), z(), z()
        self.w = z() if self.dim == 3 else None
        self.last_error = 0.0

    # ---------------------------------------------------------------
    def initialize(self):
        T = self.T
        pi = T(np.arctan(T(1.0))) * T(4.0)
        if self.dim == 2:
            I = (slice(1, self.n + 1), slice(1, self.m + 1))
            self.u[I] = self.U * T(np.cos(self.aoa / T(180) * pi))
            self.v[I] = self.U * T(np.sin(self.aoa / T(180) * pi))
            if self.inflow_porosity:  # ibm_2d_backstep_omp_cpu.f90:615-618
                self.u[I] = self.u[I] * self.poro[I]
                self.v[I] = self.v[I] * self.poro[I]
            self.p[I] = self.pout
        elif self.wall_mode:  # air-condition initial_conditions: at rest, p = outlet
            I = (slice(1, self.l + 1), slice(1, self.n + 1), slice(1, self.m + 1))
            self.u[I] = T(0)
            self.v[I] = T(0)
            self.w[I] = T(0)
            self.p[I] = self.pout
        else:
            I = (slice(1, self.l + 1), slice(1, self.n + 1), slice(1, self.m + 1))
            self.u[I] = self.U * T(np.cos(self.aoa / T(360) * pi))
            self.v[I] = self.U * T(np.sin(self.aoa / T(360) * pi))
            if self.inflow_porosity:
                self.u[I] = self.u[I] * self.poro[I]
                self.v[I] = self.v[I] * self.poro[I]
            self.w[I] = T(0)
            self.p[I] = self.pout
        self.boundary()

    def _wall_boundary(self):
        """boundary() of the air-condition program, face by face (top, bottom,
        west, east, north, south), whole faces at once."""
        T = self.T
        u, v, w, p, po = self.u, self.v, self.w, self.p, self.poro
        m, n, l = self.m, self.n, self.l
        lim, U, pout = T(0.9), self.U, self.pout
        # (face index in the table, face slice, ghost slice, inner slice, inlet sign,
        #  inlet component, mirrored component, outlet copies the inner (True) or face plane)
        faces = [
            (0, (l,), (l + 1,), (l - 1,), -1, "w", "w", True),
            (1, (1,), (0,), (2,), 1, "w", "w", False),
            (3, (slice(None), slice(None), 1), (slice(None), slice(None), 0), (slice(None), slice(None), 2),
             1, "u", "u", False),
            (2, (slice(None), slice(None), m), (slice(None), slice(None), m + 1), (slice(None), slice(None), m - 1),
             -1, "u", "u", False),
            (4, (slice(None), n), (slice(None), n + 1), (slice(None), n - 1), -1, "u", "u", False),
            (5, (slice(None), 1), (slice(None), 0), (slice(None), 2), 1, "u", "v", True),
        ]
        F = {"u": u, "v": v, "w": w}
        for (idx, fs, gs, bs, sign, incomp, mirror, out_inner) in faces:
            t = self.walls[idx]
            pf = po[(l,)] if (idx == 1) else po[fs]  # the bottom inlet tests the top plane
            inlet = (t == 1) & (pf >= lim)
            outlet = (t == 2) & (po[fs] >= lim)
            wall = ~(inlet | outlet)
            for name, a in F.items():
                face_val = a[fs].copy()
                # inlet: the face takes the inflow, the ghost copies the face
                inl = T(sign) * U if name == incomp else T(0)
                a[fs] = np.where(inlet, inl, np.where(wall, T(0), face_val))
                src = a[bs] if out_inner else a[fs]
                g_old = a[gs].copy()
                g_new = np.where(inlet, a[fs], np.where(outlet, src, g_old))
                if name == mirror:
                    g_new = np.where(wall, -a[bs], g_new)
                a[gs] = g_new
            p[gs] = np.where(outlet, pout, p[bs])

    def boundary(self):
        if self.wall_mode:
            self._wall_boundary()
            return
        T = self.T
        m, n, l = self.m, self.n, self.l
        pi = T(np.arctan(T(1.0))) * T(4.0)
        u, v, w, p = self.u, self.v, self.w, self.p
        if self.dim == 2:
            J = slice(1, n + 1)
            u[J, 1] = self.U * T(np.cos(self.aoa / T(180.) * pi))
            v[J, 1] = self.U * T(np.sin(self.aoa / T(180.) * pi))
            if self.inflow_porosity:  # ibm_2d_backstep_omp_cpu.f90:533-534
                u[J, 1] = u[J, 1] * self.poro[J, 1]
                v[J, 1] = v[J, 1] * self.poro[J, 1]
            u[J, 0] = u[J, 1]
            v[J, 0] = v[J, 1]
            p[J, 0] = p[J, 2]
            u[J, m + 1] = u[J, m - 1]
            v[J, m + 1] = v[J, m - 1]
            p[J, m + 1] = self.pout
            for a in (u, v, p):
                a[0, :] = a[n, :]
                a[n + 1, :] = a[1, :]
            if self.slip_y:  # :512-526, j = 1 then j = n, columns 1..m
                I = slice(1, m + 1)
                u[0, I] = u[2, I]
                v[1, I] = 0
                v[0, I] = -v[2, I]
                p[0, I] = p[2, I]
                u[n + 1, I] = u[n - 1, I]
                v[n, I] = 0
                v[n + 1, I] = -v[n - 1, I]
                p[n + 1, I] = p[n - 1, I]
        else:
            J, K = slice(1, n + 1), slice(1, l + 1)
            u[K, J, 1] = self.U * T(np.cos(self.aoa / T(1300.) * pi))
            v[K, J, 1] = self.U * T(np.sin(self.aoa / T(1300.) * pi))
            if self.inflow_porosity:
                u[K, J, 1] = u[K, J, 1] * self.poro[K, J, 1]
                v[K, J, 1] = v[K, J, 1] * self.poro[K, J, 1]
            w[K, J, 1] = T(0)
            u[K, J, 0] = u[K, J, 1]
            v[K, J, 0] = v[K, J, 1]
            w[K, J, 0] = w[K, J, 1]
            p[K, J, 0] = p[K, J, 2]
            u[K, J, m + 1] = u[K, J, m - 1]
            v[K, J, m + 1] = v[K, J, m - 1]
            w[K, J, m + 1] = w[K, J, m - 1]
            p[K, J, m + 1] = self.pout
            for a in (u, v, w, p):
                a[:, 0, :] = a[:, n, :]
                a[:, n + 1, :] = a[:, 1, :]
            for a in (u, v, w, p):
                a[0, :, :] = a[l, :, :]
                a[l + 1, :, :] = a[1, :, :]

    # shifted interior views ----------------------------------------
    def _s(self, a, di=0, dj=0, dk=0):
        m, n, l = self.m, self.n, self.l
        if self.dim == 2:
            return a[1 + dj:n + 1 + dj, 1 + di:m + 1 + di]
        return a[1 + dk:l + 1 + dk, 1 + dj:n + 1 + dj, 1 + di:m + 1 + di]

    def _interior(self):
        if self.dim == 2:
            return (slice(1, self.n + 1), slice(1, self.m + 1))
        return (slice(1, self.l + 1), slice(1, self.n + 1), slice(1, self.m + 1))

    # ---------------------------------------------------------------
    def step(self, nsteps=1):
        for _ in range(nsteps):
            uo, vo = self.u.copy(), self.v.copy()
            wo = self.w.copy() if self.dim == 3 else None
            self.last_error = self.solve_p(uo, vo, wo)
            self.projection()
            self.boundary()
        return self.last_error

    def divergence(self, uo, vo, wo):
        T, S = self.T, self._s
        dx, dy, dz = self.dx, self.dy, self.dz
        div = np.zeros(self.shape, dtype=self.poro.dtype)
        m, n, l = self.m, self.n, self.l
        if self.dim == 2:
            div[self._interior()] = ((S(uo, 1) - S(uo, -1)) / dx * T(.5)
                                     + (S(vo, 0, 1) - S(vo, 0, -1)) / dx * T(.5))
            div[1:n + 1, 0] = 0
            div[1:n + 1, m + 1] = 0
            div[0, 1:m + 1] = div[n, 1:m + 1]
            div[n + 1, 1:m + 1] = div[1, 1:m + 1]
        else:
            div[self._interior()] = ((S(uo, 1) - S(uo, -1)) / dx * T(.5)
                                     + (S(vo, 0, 1) - S(vo, 0, -1)) / dy * T(.5)
                                     + (S(wo, 0, 0, 1) - S(wo, 0, 0, -1)) / dz * T(.5))
            div[1:l + 1, 1:n + 1, 0] = 0
            div[1:l + 1, 1:n + 1, m + 1] = 0
            if self.wall_mode:  # every face ghost stays 0
                return div
            div[1:l + 1, 0, 1:m + 1] = div[1:l + 1, n, 1:m + 1]
            div[1:l + 1, n + 1, 1:m + 1] = div[1:l + 1, 1, 1:m + 1]
            div[0, 1:n + 1, 1:m + 1] = div[l, 1:n + 1, 1:m + 1]
            div[l + 1, 1:n + 1, 1:m + 1] = div[1, 1:n + 1, 1:m + 1]
        return div

    def predictor(self, uo, vo, wo, div):
        T, S = self.T, self._s
        dx, dy, dz, dt = self.dx, self.dy, self.dz, self.dt
        nu, lam, th = self.xnue, self.xlambda, self.thickness
        po = self.poro
        pc = S(po)
        two, half, one, alpha = T(2.), T(.5), T(1.), T(32.)
        if self.dim == 2:
            def comp(f, g_conv_x, g_conv_y, d_e, d_w, d_scale, A, B, dpx, dpy, dterm):
                t = S(f) - dt * (S(uo) * (S(f, 1) - S(f, -1)) / dx / two)
                t = t - dt * (S(vo) * (S(f, 0, 1) - S(f, 0, -1)) / dy / two)
                t = t + dt * nu * (S(f, 1) - two * S(f) + S(f, -1)) / dx / dx
                t = t + dt * nu * (S(f, 0, 1) - two * S(f) + S(f, 0, -1)) / dy / dy
                t = t + dt * (nu + lam) * (d_e - d_w) / d_scale * half
                t = t + dt * (A * nu * (S(po, 1) - S(po, -1)) / dx * half
                              + B * nu * (S(po, 0, 1) - S(po, 0, -1)) / dy * half
                              + dterm) / pc
                if self.nonslip:
                    t = t - dt * nu * S(f) / ((th * dx) * (th * dx)) * alpha * pc * (one - pc) * (one - pc)
                return t
            dux = (S(uo, 1) - S(uo, -1)) / dx * half
            duy = (S(uo, 0, 1) - S(uo, 0, -1)) / dy * half
            dvx = (S(vo, 1) - S(vo, -1)) / dx * half
            dvy = (S(vo, 0, 1) - S(vo, 0, -1)) / dy * half
            un = comp(uo, None, None, S(div, 1), S(div, -1), dx, dux + dux, duy + dvx, None, None,
                      S(div) * (S(po, 1) - S(po, -1)) / dx * T(0.5) * lam)
            vn = comp(vo, None, None, S(div, 0, 1), S(div, 0, -1), dy, dvx + duy, dvy + dvy, None, None,
                      S(div) * (S(po, 0, 1) - S(po, 0, -1)) / dy * T(0.5) * lam)
            self.u[self._interior()] = un
            self.v[self._interior()] = vn
        else:
            def comp(f, d_e, d_w, d_scale, A1, A2, A3, dterm, hdamp):
                t = S(f) - dt * S(uo) * (S(f, 1) - S(f, -1)) / dx * half
                t = t - dt * S(vo) * (S(f, 0, 1) - S(f, 0, -1)) / dy * half
                t = t - dt * S(wo) * (S(f, 0, 0, 1) - S(f, 0, 0, -1)) / dz * half
                t = t + dt * nu * (S(f, 1) - two * S(f) + S(f, -1)) / dx / dx
                t = t + dt * nu * (S(f, 0, 1) - two * S(f) + S(f, 0, -1)) / dy / dy
                t = t + dt * nu * (S(f, 0, 0, 1) - two * S(f) + S(f, 0, 0, -1)) / dz / dz
                t = t + dt * (nu + lam) * (d_e - d_w) / d_scale * half
                t = t + dt * (A1 * nu * (S(po, 1) - S(po, -1)) / dx * half
                              + A2 * nu * (S(po, 0, 1) - S(po, 0, -1)) / dy * half
                              + A3 * nu * (S(po, 0, 0, 1) - S(po, 0, 0, -1)) / dz * half
                              + dterm) / pc
                if self.nonslip:
                    t = t - dt * nu * S(f) / ((th * hdamp) * (th * hdamp)) * alpha * pc * (one - pc) * (one - pc)
                return t
            g = lambda f, di, dj, dk, h: (S(f, di, dj, dk) - S(f, -di, -dj, -dk)) / h * half
            dux, duy, duz = g(uo, 1, 0, 0, dx), g(uo, 0, 1, 0, dy), g(uo, 0, 0, 1, dz)
            dvx, dvy, dvz = g(vo, 1, 0, 0, dx), g(vo, 0, 1, 0, dy), g(vo, 0, 0, 1, dz)
            dwx, dwy, dwz = g(wo, 1, 0, 0, dx), g(wo, 0, 1, 0, dy), g(wo, 0, 0, 1, dz)
            un = comp(uo, S(div, 1), S(div, -1), dx, dux + dux, duy + dvx, duz + dwx,
                      S(div) * (S(po, 1) - S(po, -1)) / dx * half * lam, dx)
            vn = comp(vo, S(div, 0, 1), S(div, 0, -1), dy, dvx + duy, dvy + dvy, dvz + dwy,
                      S(div) * (S(po, 0, 1) - S(po, 0, -1)) / dy * half * lam, dy)
            wn = comp(wo, S(div, 0, 0, 1), S(div, 0, 0, -1), dz, dwx + duz, dwy + dvz, dwz + dwz,
                      S(div) * (S(po, 0, 0, 1) - S(po, 0, 0, -1)) / dz * half * lam, dz)
            I = self._interior()
            self.u[I], self.v[I], self.w[I] = un, vn, wn

    def coefficients(self):
        """ae..ab, ap, bb after boundrary_matrix; dict of interior arrays."""
        T, S = self.T, self._s
        dx, dy, dz, dt, rho = self.dx, self.dy, self.dz, self.dt, self.density
        small, half = T(1.e-6), T(0.5)
        po, pc = self.poro, S(self.poro)
        face = lambda a, b, h: dt * np.maximum(small, (a + b) * half) / h / h
        C = {}
        C["ae"] = face(S(po, 1), pc, dx)
        C["aw"] = face(pc, S(po, -1), dx)
        C["an"] = face(S(po, 0, 1), pc, dy)
        C["as"] = face(pc, S(po, 0, -1), dy)
        u, v, w = self.u, self.v, self.w
        bb = (((S(po, 1) * S(u) + pc * S(u, 1)) * half - (S(po, -1) * S(u) + pc * S(u, -1)) * half) * rho / dx
              + ((S(po, 0, 1) * S(v) + pc * S(v, 0, 1)) * half
                 - (S(po, 0, -1) * S(v) + pc * S(v, 0, -1)) * half) * rho / dy)
        if self.dim == 3:
            C["at"] = face(S(po, 0, 0, 1), pc, dz)
            C["ab"] = face(pc, S(po, 0, 0, -1), dz)
            C["ap"] = -C["ae"] - C["aw"] - C["an"] - C["as"] - C["at"] - C["ab"]
            bb = bb + ((S(po, 0, 0, 1) * S(w) + pc * S(w, 0, 0, 1)) * half
                       - (S(po, 0, 0, -1) * S(w) + pc * S(w, 0, 0, -1)) * half) * rho / dz
        else:
            C["ap"] = -C["ae"] - C["aw"] - C["an"] - C["as"]
        C["bb"] = bb
        if self.wall_mode:
            self._wall_matrix(C)
            return C
        # boundrary_matrix
        C["ae"][..., 0] = C["ae"][..., 0] + C["aw"][..., 0]
        C["aw"][..., 0] = 0
        C["bb"][..., -1] = C["bb"][..., -1] + C["ae"][..., -1] * S(self.p, 1)[..., -1]
        for key in ("ae", "aw", "an", "as", "at", "ab"):
            if key in C:
                C[key][..., -1] = 0
        if self.slip_y:  # :440-450, rows j = 1 then j = n
            C["an"][0, :] = C["an"][0, :] + C["as"][0, :]
            C["as"][0, :] = 0
            C["as"][-1, :] = C["as"][-1, :] + C["an"][-1, :]
            C["an"][-1, :] = 0
        return C

    def _wall_matrix(self, C):
        """boundary_matrix of the air-condition program on the interior
        arrays [k, j, i]: faces top, bottom, east, west, north, south."""
        T = self.T
        lim = T(0.9)
        pc = self._s(self.poro)
        p = self.p
        m, n, l = self.m, self.n, self.l
        bb1 = C["bb"][0].copy()  # plane 1 before any edit (the top outlet starts from it)
        # (table index, face slice of the interior arrays, outward key, inward key, p ghost slice)
        faces = [(0, (-1,), "at", "ab", (l + 1, slice(1, n + 1), slice(1, m + 1))),
                 (1, (0,), "ab", "at", (0, slice(1, n + 1), slice(1, m + 1))),
                 (2, (slice(None), slice(None), -1), "ae", "aw", (slice(1, l + 1), slice(1, n + 1), m + 1)),
                 (3, (slice(None), slice(None), 0), "aw", "ae", (slice(1, l + 1), slice(1, n + 1), 0)),
                 (4, (slice(None), -1), "an", "as", (slice(1, l + 1), n + 1, slice(1, m + 1))),
                 (5, (slice(None), 0), "as", "an", (slice(1, l + 1), 0, slice(1, m + 1)))]
        keys = ("ae", "aw", "an", "as", "at", "ab")
        for (idx, fs, out, inw, gs) in faces:
            t = self.walls[idx]
            outlet = (t == 2) & (pc[fs] >= lim)
            a_out = C[out][fs].copy()
            C[inw][fs] = np.where(outlet, C[inw][fs], C[inw][fs] + a_out)
            C[out][fs] = np.where(outlet, C[out][fs], T(0))
            base = bb1 if idx == 0 else C["bb"][fs]
            C["bb"][fs] = np.where(outlet, base + a_out * p[gs], C["bb"][fs])
            for k in keys:
                C[k][fs] = np.where(outlet, T(0), C[k][fs])

    def _halo_p(self):
        if self.wall_mode:  # the air-condition program keeps its ghosts during the sweeps
            return
        p, m, n, l = self.p, self.m, self.n, self.l
        if self.dim == 2:
            p[0, 1:m + 1] = p[n, 1:m + 1]
            p[n + 1, 1:m + 1] = p[1, 1:m + 1]
        else:
            p[1:l + 1, 0, 1:m + 1] = p[1:l + 1, n, 1:m + 1]
            p[1:l + 1, n + 1, 1:m + 1] = p[1:l + 1, 1, 1:m + 1]
            p[0, 1:n + 1, 1:m + 1] = p[l, 1:n + 1, 1:m + 1]
            p[l + 1, 1:n + 1, 1:m + 1] = p[1, 1:n + 1, 1:m + 1]

    def colour_masks(self):
        """(first, second) half-sweep masks over the interior."""
        if self.dim == 2:
            j, i = np.meshgrid(np.arange(1, self.n + 1), np.arange(1, self.m + 1), indexing="ij")
            first = (i + j) % 2 == 1
        else:
            k, j, i = np.meshgrid(np.arange(1, self.l + 1), np.arange(1, self.n + 1),
                                  np.arange(1, self.m + 1), indexing="ij")
            first = (i + j + k) % 2 == 0
        return first, ~first

    def sor(self, C):
        T, S = self.T, self._s
        om = self.relux
        first, second = self.colour_masks()
        I = self._interior()
        error = T(0)
        for _ in range(self.iter_max):
            for which, mask in enumerate((first, second)):
                self._halo_p()
                po = self.p.copy()
                r = C["bb"] - C["ae"] * S(po, 1) - C["aw"] * S(po, -1) - C["an"] * S(po, 0, 1) - C["as"] * S(po, 0, -1)
                if self.dim == 3:
                    r = r - C["at"] * S(po, 0, 0, 1) - C["ab"] * S(po, 0, 0, -1)
                new = r / C["ap"] * om + S(po) * (T(1.) - om)
                interior = self.p[I]
                interior[mask] = new[mask]
                if self.dim == 2 or which == 1:
                    d = np.abs(interior - S(po))
                    error = max(error, d.max())
        self._halo_p()
        return float(error)

    def solve_p(self, uo, vo, wo):
        div = self.divergence(uo, vo, wo)
        self.predictor(uo, vo, wo, div)
        C = self.coefficients()
        return self.sor(C)

    def projection(self):
        T, S = self.T, self._s
        dt, rho, half = self.dt, self.density, T(0.5)
        I = self._interior()
        p = self.p
        self.u[I] = S(self.u) - dt / rho * (S(p, 1) - S(p, -1)) / self.dx * half
        self.v[I] = S(self.v) - dt / rho * (S(p, 0, 1) - S(p, 0, -1)) / self.dy * half
        if self.dim == 3:
            self.w[I] = S(self.w) - dt / rho * (S(p, 0, 0, 1) - S(p, 0, 0, -1)) / self.dz * half

    def divergence_diag(self):
        T, S = self.T, self._s
        po, pc, u, v = self.poro, S(self.poro), self.u, self.v
        two = T(2)
        d = (((S(po, 1) * S(u) + pc * S(u, 1)) / two - (S(po, -1) * S(u) + pc * S(u, -1)) / two) / self.dx
             + ((S(po, 0, 1) * S(v) + pc * S(v, 0, 1)) / two - (S(po, 0, -1) * S(v) + pc * S(v, 0, -1)) / two) / self.dy)
        if self.dim == 3:
            w = self.w
            d = d + ((S(po, 0, 0, 1) * S(w) + pc * S(w, 0, 0, 1)) / two
                     - (S(po, 0, 0, -1) * S(w) + pc * S(w, 0, 0, -1)) / two) / self.dz
        return float(np.abs(d).max()), d


def forces(poro, p, u, v, w, dx, dy, dz, thickness, density, xnue):
    """Force sums of output_force_log_2d/_3d (output.f90:244-305, :1090-1165),
    vectorised: returns (pressure part (3,), friction part (3,), sum of |term|
    per component (6,)) -- the last one scales the tolerance of a comparison
    whose summation order differs."""
    small, alpha = 1.e-6, 32.0
    dim = p.ndim
    if dim == 2:
        c = (slice(1, -1), slice(1, -1))
        gx = (poro[1:-1, 2:] - poro[1:-1, :-2]) * 0.5
        gy = (poro[2:, 1:-1] - poro[:-2, 1:-1]) * 0.5
        gz = np.zeros_like(gx)
        vol = dx * dy
        na = np.sqrt(gx * gx + gy * gy)
    else:
        c = (slice(1, -1), slice(1, -1), slice(1, -1))
        gx = (poro[1:-1, 1:-1, 2:] - poro[1:-1, 1:-1, :-2]) * 0.5
        gy = (poro[1:-1, 2:, 1:-1] - poro[1:-1, :-2, 1:-1]) * 0.5
        gz = (poro[2:, 1:-1, 1:-1] - poro[:-2, 1:-1, 1:-1]) * 0.5
        vol = dx * dy * dz
        na = np.sqrt(gx * gx + gy * gy + gz * gz)
    e = poro[c]
    ee = e * (1.0 - e)
    nrm = np.maximum(na, small)
    terms = []
    for g, h in ((gx, dx), (gy, dy), (gz, dz)):
        terms.append(-vol * p[c] * 2 * e * (1.0 - e) / (thickness * h) * (g / nrm) if h else np.zeros_like(e))
    for f, h in ((u, dx), (v, dy), (w, dz)):
        if f is None or not h:
            terms.append(np.zeros_like(e))
        else:
            t = ee / (thickness * h)
            terms.append(vol * alpha * density * xnue * (t * t) * f[c])
    sums = np.array([t.sum() for t in terms])
    mags = np.array([np.abs(t).sum() for t in terms])
    return sums[:3], sums[3:], mags
