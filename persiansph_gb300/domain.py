"""SPH::Domain mirror: the user-facing API of the reference on top of the GB300 path.

Same names, argument meanings and error behaviour as Source/Domain.h:44-166:
set-up (AddSingleParticle, AddBoxLength, AddBoxNo, DelParticles), the
Kernel_Set / Viscosity_Eq_Set / Gradient_Approach_Set selectors, the public
fields, the GeneralBefore / GeneralAfter hooks and Solve. Particles are held
as structure-of-arrays (`persiansph_gb300.particles`) and `Solve` runs the
per-step loop on the GPU through the C ABI (`persiansph_gb300.solver`).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from .abi import PsphConfig
from .particles import ParticleList, ParticleSet

# Source/Domain.h:38-40
Qubic_Spline, Quintic, Quintic_Spline = 0, 1, 2
Morris, Shao, Incompressible_Full, Takeda = 0, 1, 2, 3
Squared_density, Multiplied_density = 0, 1


class Fatal(RuntimeError):
    """The reference's `Fatal` exception (External/fatal.h:65)."""


class Boundary:
    """SPH::Boundary (Source/Boundary_Condition.h:26-53, defaults of
    Source/Boundary_Condition.cpp:24-41)."""

    def __init__(self):
        self.Periodic = [False, False, False]
        self.InOutFlow = 0
        self.allv = [0.0, 0.0, 0.0]
        self.allDensity = 0.0
        self.inv = [0.0, 0.0, 0.0]
        self.outv = [0.0, 0.0, 0.0]
        self.inDensity = 0.0
        self.outDensity = 0.0
        self.cellfac = 3.9
        self.MassConservation = False


def _libc_rand():
    libc = ctypes.CDLL(None)
    libc.rand.restype = ctypes.c_int
    libc.srand.argtypes = [ctypes.c_uint]
    return libc


RAND_MAX = 2147483647


class Domain:
    """Mirror of SPH::Domain (constructor defaults: Source/Domain.cpp:54-102)."""

    def __init__(self):
        self.Dimension = 2
        self.Gravity = [0.0, 0.0, 0.0]
        self.BC = Boundary()
        self.Nproc = 1
        self.Scheme = 0
        self.XSPH = 0.0
        self.InitialDist = 0.0
        self.sqrt_h_a = 0.0025
        self.DomMax = [-100000000000.0] * 3
        self.DomMin = [100000000000.0] * 3
        self.R = 0.0
        self.SWIType = 0
        self.FSI = False
        self.GeneralBefore = None
        self.GeneralAfter = None
        # UserOutput(particles) -> three per-particle arrays for the snapshot's
        # OutputName datasets; None: the reference's default OutPut (zeros)
        self.UserOutput = None
        # In/out-flow hooks (Source/Domain.h:128-130): InCon(position, BC) and
        # OutCon(position, BC) -> (velocity, density) for the in-flow and
        # out-flow particles of every step, AllCon for WholeVelocity's initial
        # state; None: the reference's InFlowCon / OutFlowCon / AllFlowCon,
        # which return BC.inv / inDensity, BC.outv / outDensity, BC.allv /
        # allDensity.
        self.InCon = None
        self.OutCon = None
        self.AllCon = None
        # Constant acceleration on free particles applied where GeneralBefore
        # runs: the device-side form of the 1-Poiseuille.cpp UserAcc hook.
        self.BodyForce = [0.0, 0.0, 0.0]
        self.Precision = 0  # PSPH_FP64
        self.WallPressureMode = 0  # PSPH_WALLP_REFERENCE
        self.ShepardStep = 40
        self.OutputName = ["Property1", "Property2", "Property3"]
        self._kernel_type = 0
        self._cellfac = 2.0
        self._vis_eq = 0
        self._gradient_type = 0
        self.particles = ParticleSet()
        self.Time = 0.0

    # -- selectors (Source/Domain.cpp:117-131) ------------------------------
    def Kernel_Set(self, kt):
        self._kernel_type = int(kt)
        self._cellfac = 3.0 if self._kernel_type == 2 else 2.0

    def Viscosity_Eq_Set(self, vq):
        self._vis_eq = int(vq)

    def Gradient_Approach_Set(self, gt):
        self._gradient_type = int(gt)

    @property
    def Particles(self):
        return ParticleList(self.particles)

    # -- particle generation ------------------------------------------------
    def AddSingleParticle(self, tag, x, Mass, Density, h, Fixed):
        """Domain::AddSingleParticle (Source/Domain.cpp:154-157)."""
        self.particles.append(1, {
            "id": [tag], "x": np.asarray(x, float).reshape(1, 3), "mass": [Mass], "density": [Density],
            "h": [h], "is_free": [0 if Fixed else 1]})

    def _check_packing(self, type_, rotation):
        if type_ not in (0, 1):
            raise Fatal("Packing Type is out of range. Please correct it and run again")
        if rotation not in (0, 90):
            raise Fatal("Packing Rotation Angle is out of range. Please correct it and run again")

    def _push(self, tag, xs, mass, density, h, fixed, random, r):
        xs = np.asarray(xs, dtype=np.float64).reshape(-1, 3)
        if random:
            # srand(100) then rand() per jittered coordinate, as the reference
            # does (Source/Domain.cpp:329-330); uses the C library's generator.
            libc = _libc_rand()
            libc.srand(100)
            qin = 0.03
            ncomp = 3 if self.Dimension == 3 else 2
            for i in range(xs.shape[0]):
                for d in range(ncomp):
                    xs[i, d] = xs[i, d] + qin * r * float(libc.rand()) / RAND_MAX
        n = xs.shape[0]
        self.particles.append(n, {
            "id": np.full(n, tag, np.int32), "x": xs, "mass": np.broadcast_to(np.asarray(mass, float), (n,)),
            "density": np.full(n, density), "h": np.full(n, h), "is_free": np.full(n, 0 if fixed else 1, np.int32)})
        return n

    @staticmethod
    def _count(start, limit, pos_of):
        """Number of iterations of `while (p <= limit)` with p = start, then pos_of(i)."""
        i = 0
        p = start
        while p <= limit:
            i += 1
            p = pos_of(i)
        return i

    def AddBoxLength(self, tag, V, Lx, Ly, Lz, r, Density, h, type_, rotation, random, Fixed):
        """Domain::AddBoxLength (Source/Domain.cpp:294-495): lattice of particles in a box."""
        self._check_packing(type_, rotation)
        V = [float(v) for v in V]
        pre = self.particles.n
        sq3 = math.sqrt(3.0)
        pts = []
        if self.Dimension == 3:
            if type_ == 0:
                k = 0
                zp = V[2]
                while zp <= (V[2] + Lz - r):
                    j = 0
                    yp = V[1]
                    while yp <= (V[1] + Ly - r):
                        odd = (k % 2 != 0) and (j % 2 != 0)
                        off = (j % 2) + (k % 2) + (-1 if odd else 1)

                        def xpos(i, off=off):
                            return V[0] + (2 * i + off) * r
                        ni = self._count(V[0], V[0] + Lx - r, xpos)
                        i = np.arange(ni)
                        x = V[0] + (2 * i + off).astype(np.float64) * r
                        y = V[1] + (sq3 * (j + (1.0 / 3.0) * (k % 2)) + 1) * r
                        z = V[2] + ((2 * math.sqrt(6.0) / 3) * k + 1) * r
                        pts.append(np.stack([x, np.full(ni, y), np.full(ni, z)], axis=1))
                        j += 1
                        yp = V[1] + (sq3 * (j + (1.0 / 3.0) * (k % 2)) + 1) * r
                    k += 1
                    zp = V[2] + ((2 * math.sqrt(6.0) / 3) * k + 1) * r
            else:
                nx = self._count(V[0], V[0] + Lx - r, lambda i: V[0] + (2 * i + 1) * r)
                ny = self._count(V[1], V[1] + Ly - r, lambda j: V[1] + (2.0 * j + 1) * r)
                nz = self._count(V[2], V[2] + Lz - r, lambda k: V[2] + (2.0 * k + 1) * r)
                xs = V[0] + (2.0 * np.arange(nx) + 1) * r
                ys = V[1] + (2.0 * np.arange(ny) + 1) * r
                zs = V[2] + (2.0 * np.arange(nz) + 1) * r
                Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
                pts.append(np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1))
            xs = np.concatenate(pts) if pts else np.zeros((0, 3))
            n = xs.shape[0]
            if random:
                n = self._push(tag, xs, 0.0, Density, h, Fixed, True, r)
            else:
                n = self._push(tag, xs, 0.0, Density, h, Fixed, False, r)
            # 3D mass from the bounding box (Source/Domain.cpp:399-415)
            x_new = self.particles.get("x")[pre:]
            mx = [V[0], V[1], V[2]]
            for d in range(3):
                m = float(x_new[:, d].max()) if n else V[d]
                if m > mx[d]:
                    mx[d] = m
            tmp = [(mx[d] + r) - V[d] for d in range(3)]
            mass = tmp[0] * tmp[1] * tmp[2] * Density / n
            self.particles.get("mass")[pre:] = mass
        else:
            if type_ == 0:
                mass = (sq3 * r * r) * Density
                if rotation == 0:
                    j = 0
                    yp = V[1]
                    while yp <= (V[1] + Ly - r):
                        off = (j % 2) + 1
                        ni = self._count(V[0], V[0] + Lx - r, lambda i, off=off: V[0] + (2 * i + off) * r)
                        x = V[0] + (2 * np.arange(ni) + off).astype(np.float64) * r
                        y = V[1] + (sq3 * j + 1) * r
                        pts.append(np.stack([x, np.full(ni, y), np.zeros(ni)], axis=1))
                        j += 1
                        yp = V[1] + (sq3 * j + 1) * r
                else:
                    i = 0
                    xp = V[0]
                    while xp <= (V[0] + Lx - r):
                        off = (i % 2) + 1
                        nj = self._count(V[1], V[1] + Ly - r, lambda j, off=off: V[1] + (2 * j + off) * r)
                        x = V[0] + (sq3 * i + 1) * r
                        y = V[1] + (2 * np.arange(nj) + off).astype(np.float64) * r
                        pts.append(np.stack([np.full(nj, x), y, np.zeros(nj)], axis=1))
                        i += 1
                        xp = V[0] + (sq3 * i + 1) * r
            else:
                mass = (sq3 * r * r) * Density if random else 2.0 * r * 2.0 * r * Density
                nx = self._count(V[0], V[0] + Lx - r, lambda i: V[0] + (2 * i + 1) * r)
                ny = self._count(V[1], V[1] + Ly - r, lambda j: V[1] + (2 * j + 1) * r)
                xs = V[0] + (2 * np.arange(nx) + 1).astype(np.float64) * r
                ys = V[1] + (2 * np.arange(ny) + 1).astype(np.float64) * r
                Y, X = np.meshgrid(ys, xs, indexing="ij")
                pts.append(np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1))
            xs = np.concatenate(pts) if pts else np.zeros((0, 3))
            self._push(tag, xs, mass, Density, h, Fixed, random, r)
        self.R = r

    def AddBoxNo(self, tag, V, nx, ny, nz, r, Density, h, type_, rotation, random, Fixed):
        """Domain::AddBoxNo (Source/Domain.cpp:159-292), cubic packing."""
        self._check_packing(type_, rotation)
        if type_ != 1:
            raise Fatal("AddBoxNo with hexagonal packing: use AddBoxLength")
        V = [float(v) for v in V]
        pre = self.particles.n
        if self.Dimension == 3:
            xs = V[0] + (2.0 * np.arange(nx) + 1) * r
            ys = V[1] + (2.0 * np.arange(ny) + 1) * r
            zs = V[2] + (2.0 * np.arange(nz) + 1) * r
            Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
            self._push(tag, np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1), 0.0, Density, h, Fixed, random, r)
            x_new = self.particles.get("x")[pre:]
            mx = [max(V[d], float(x_new[:, d].max())) for d in range(3)]
            tmp = [(mx[d] + r) - V[d] for d in range(3)]
            self.particles.get("mass")[pre:] = tmp[0] * tmp[1] * tmp[2] * Density / (self.particles.n - pre)
        else:
            xs = V[0] + (2 * np.arange(nx) + 1).astype(np.float64) * r
            ys = V[1] + (2 * np.arange(ny) + 1).astype(np.float64) * r
            Y, X = np.meshgrid(ys, xs, indexing="ij")
            mass = (math.sqrt(3.0) * r * r) * Density if random else 2.0 * r * 2.0 * r * Density
            self._push(tag, np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1), mass, Density, h, Fixed,
                       random, r)
        self.R = r

    def DelParticles(self, Tags):
        """Domain::DelParticles (Source/Domain.cpp:497-515)."""
        ids = self.particles.get("id")
        mask = ids != Tags
        if mask.all():
            raise Fatal("Domain::DelParticles: Could not find any particles to delete")
        self.particles.keep(mask)

    # -- boundary to the C ABI ----------------------------------------------
    def config(self, dt: float) -> PsphConfig:
        c = PsphConfig()
        c.dimension = int(self.Dimension)
        c.kernel_type = self._kernel_type
        c.vis_eq = self._vis_eq
        c.gradient_type = self._gradient_type
        c.scheme = int(self.Scheme)
        for d in range(3):
            c.periodic[d] = int(bool(self.BC.Periodic[d]))
            c.gravity[d] = float(self.Gravity[d])
            c.body_force[d] = float(self.BodyForce[d])
            c.dom_max[d] = float(self.DomMax[d])
            c.dom_min[d] = float(self.DomMin[d])
        c.swi_type = int(self.SWIType)
        c.fsi = int(bool(self.FSI))
        c.in_out_flow = int(self.BC.InOutFlow)
        c.mass_conservation = int(bool(self.BC.MassConservation))
        c.bc_cellfac = float(self.BC.cellfac)
        c.initial_dist = float(self.InitialDist)
        c.in_density = float(self.BC.inDensity)
        c.out_density = float(self.BC.outDensity)
        for d in range(3):
            c.in_v[d] = float(self.BC.inv[d])
            c.out_v[d] = float(self.BC.outv[d])
        c.shepard_step = int(self.ShepardStep)
        c.precision = int(self.Precision)
        c.wall_pressure_mode = int(self.WallPressureMode)
        c.xsph = float(self.XSPH)
        c.sqrt_h_a = float(self.sqrt_h_a)
        c.R = float(self.R)
        c.dt = float(dt)
        c.time = float(self.Time)
        return c

    # -- solve ---------------------------------------------------------------
    def WholeVelocity(self):
        """Domain::WholeVelocity (Source/Domain.cpp:1636-1659): with BC.allv or
        BC.allDensity set, every free particle takes the velocity and / or the
        density AllCon gives for its position (the pressure follows from the
        density at upload, InitialChecks' EOS)."""
        bc = self.BC
        set_v = math.sqrt(sum(float(a) * float(a) for a in bc.allv)) > 0.0
        set_d = bc.allDensity > 0.0
        if not (set_v or set_d):
            return
        p = self.particles
        x, v, den = p.get("x"), p.get("v"), p.get("density")
        free = p.get("is_free") != 0
        for i in range(p.n):
            if self.AllCon is not None:
                vel, d = self.AllCon(x[i].copy(), bc)
            else:
                vel, d = bc.allv, bc.allDensity
            if free[i] and set_v:
                v[i] = [float(c) for c in vel]
            if free[i] and set_d:
                den[i] = float(d)
        p.set("v", v)
        p.set("density", den)

    def Solve(self, tf, dt, dtOut, TheFileKey=None, maxidx=10**9, output=None):
        """Domain::Solve (Source/Domain.cpp:1735-1797) with the step body on the GPU.

        With TheFileKey, the reference's snapshots (WriteXDMF) are written as
        <key>_Initial and <key>_0001, ... (.bin + .xmf, the reference's
        datasets in a raw file): with the default UserOutput each is taken on
        the device after the output step's forces; a UserOutput(particle_set)
        returning three arrays runs on the host on the particles downloaded at
        the output time. `output(domain, idx)` (optional) is called at each
        output time with the particles downloaded into `self.particles`.
        GeneralBefore(domain) / GeneralAfter(domain) run on the host inside
        every step, where the reference calls them, with `self.particles` and
        `self.Time` the context's at that point; what they change is written
        back (the per-step slow path; BodyForce is the device-side constant
        acceleration).
        """
        from .solver import GpuDomain

        self.WholeVelocity()
        sim = GpuDomain(self.config(dt))
        if self.BC.InOutFlow:
            sim.use_flow_hooks(self)
        if self.GeneralBefore is not None or self.GeneralAfter is not None:
            sim.use_step_hooks(self, live=True)
        sim.upload(self.particles, initial=True)
        idx_out = 1
        tout = self.Time
        user = getattr(self, "UserOutput", None)
        names = list(self.OutputName)

        def write_now(fn):
            props = user(self.particles) if user is not None else None
            sim.write_output(fn, names, props)

        if TheFileKey is not None:
            write_now(f"{TheFileKey}_Initial")
        while sim.time < tf and idx_out <= maxidx:
            if sim.time >= tout:
                if output is not None or (TheFileKey is not None and user is not None):
                    self.particles = sim.download(self.particles)
                if output is not None:
                    output(self, idx_out)
                if TheFileKey is not None:
                    fn = f"{TheFileKey}_{idx_out:04d}"
                    if user is not None:
                        write_now(fn)
                    else:
                        sim.request_output(fn, names)
                idx_out += 1
                tout += dtOut
            sim.step(1 << 30, t_stop=min(tf, tout))
        sim.flush_output()
        self.particles = sim.download(self.particles)
        self.Time = sim.time
        return sim
