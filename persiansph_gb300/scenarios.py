"""Workload builders with the shapes of the benchmarked configurations.

Each builder fills a `Domain` through the reference's own API
(AddBoxLength + per-particle fields + DelParticles), the way the reference's
example drivers do, with sizes parameterised so tests can run them small:

  poiseuille      2D periodic channel (1-Poiseuille.cpp shape)
  dam_break_2d    2D water column in a tank (3-DamBreak.cpp shape)
  dam_break_3d    3D water column in a tank (4-DamBreak3D.cpp shape)
  granular_column 2D Drucker-Prager soil column (Old_Tests/ReposeAngle2.cpp shape)
  seepage_bed_2d  2D dam break over an erodible soil bed (Old_Tests/Dam_Scouring2.cpp shape)
  elastic_gate_2d 2D water column behind an elastic gate (Old_Tests/FSI_ElasticGate.cpp shape)

All inputs are synthetic and seeded; the reference ships no datasets.
"""
from __future__ import annotations

import math

import numpy as np

from .domain import Domain, Morris, Qubic_Spline, Quintic, Quintic_Spline, Squared_density


def poiseuille(dx=2.5e-5, H=1.0e-3, W=0.5e-3, wall_layers=3, rho=1000.0, nu=1.0e-6, gx=1.0e-4,
               scheme=1, kernel=Quintic_Spline, hfac=1.3):
    """2D Poiseuille flow between no-slip walls, periodic in x.

    Umax = gx H^2 / (8 nu); c0 = 10 Umax; dt = min(0.25 h/c0, 0.125 h^2/nu)
    (the second bound is TimestepCheck's viscous limit, Source/Domain.cpp:1724-1732).
    Returns (domain, dt, info).
    """
    dom = Domain()
    dom.Dimension = 2
    dom.BC.Periodic[0] = True
    dom.Scheme = scheme
    dom.Kernel_Set(kernel)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    h = hfac * dx
    mu = nu * rho
    umax = gx * H * H / (8.0 * nu)
    cs = 10.0 * umax
    nrow = int(round(H / dx))
    ncol = int(round(W / dx))
    half = nrow // 2
    dom.InitialDist = dx
    dom.AddBoxLength(1, (0.0, -(half + wall_layers) * dx, 0.0), ncol * dx + dx / 10.0,
                     (nrow + 2 * wall_layers) * dx + dx / 10.0, 0, dx / 2.0, rho, h, 1, 0, False, False)
    p = dom.particles
    y = p.get("x")[:, 1]
    wall = (y >= half * dx) | (y <= -half * dx)
    p.set("cs", cs)
    p.set("pres_eq", 0)
    p.set("mu", mu)
    p.set("mu_ref", mu)
    p.set("material", 1)
    p.get("id")[wall] = 2
    p.get("is_free")[wall] = 0
    p.get("no_slip")[wall] = 1
    dom.BodyForce = [gx, 0.0, 0.0]
    dt = min(0.25 * h / cs, 0.125 * h * h / nu)
    return dom, dt, {"umax": umax, "cs": cs, "H": H, "nu": nu, "gx": gx, "h": h}


def _tank(dom, dx, TL, TH, TW, wall_layers):
    """Lattice box covering the tank plus its wall layers (cubic packing)."""
    w = wall_layers
    if dom.Dimension == 2:
        dom.AddBoxLength(1, (-w * dx, -w * dx, 0.0), 2 * w * dx + TL + dx / 10.0, w * dx + TH + dx / 10.0, 0,
                         dx / 2.0, 1.0, 1.0, 1, 0, False, False)
    else:
        dom.AddBoxLength(1, (-w * dx, -w * dx, -w * dx), 2 * w * dx + TL + dx / 10.0, w * dx + TH + dx / 10.0,
                         2 * w * dx + TW + dx / 10.0, dx / 2.0, 1.0, 1.0, 1, 0, False, False)


def dam_break_2d(dx=5e-3, L=1.0, H=2.0, TL=4.0, TH=3.0, wall_layers=3, rho=1000.0, g=9.81, alpha=0.1,
                 mu=1.002e-3, scheme=0, shepard=True, kernel=Qubic_Spline, hfac=1.2, c0=None):
    """2D dam break: an L x H water column at the left of a TL x TH tank.

    Tait EOS (gamma 7) with c0 = 10 sqrt(2 g H) unless given, hydrostatic initial
    density as 3-DamBreak.cpp:95-99. Returns (domain, dt, info).
    """
    dom = Domain()
    dom.Dimension = 2
    dom.Scheme = scheme
    dom.Kernel_Set(kernel)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    h = hfac * dx
    cs = 10.0 * math.sqrt(2.0 * g * H) if c0 is None else c0
    dom.InitialDist = dx
    dom.Gravity = [0.0, -g, 0.0]
    _tank(dom, dx, TL, TH, 0.0, wall_layers)
    p = dom.particles
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = (xb < 0.0) | (yb < 0.0) | (xb > TL)
    drop = (~wall) & ((yb > H) | (xb > L))
    keep = ~drop
    p.keep(keep)
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = (xb < 0.0) | (yb < 0.0) | (xb > TL)
    _fluid_fields(p, wall, rho, cs, mu, alpha, shepard, h)
    fl = ~wall
    dens = rho * np.power((1 + 7.0 * g * (H - yb[fl]) / (cs * cs)), (1.0 / 7.0))
    p.get("density")[fl] = dens
    p.get("densityb")[fl] = dens
    p.set("mass", 2.0 * (dx / 2.0) * 2.0 * (dx / 2.0) * rho)
    dt = 0.25 * h / cs
    return dom, dt, {"cs": cs, "H": H, "L": L, "g": g, "h": h, "n_fluid": int(fl.sum()), "n_wall": int(wall.sum())}


def _fluid_fields(p, wall, rho, cs, mu, alpha, shepard, h):
    n = p.n
    p.set("h", h)
    p.set("density", rho)
    p.set("ref_density", rho)
    p.set("cs", cs)
    p.set("pres_eq", 1)
    p.set("mu", mu)
    p.set("mu_ref", mu)
    p.set("material", 1)
    p.set("alpha", alpha)
    p.set("shepard", 1 if shepard else 0)
    ids = np.ones(n, np.int32)
    ids[wall] = 2
    p.set("id", ids)
    p.set("is_free", (~wall).astype(np.int32))
    p.set("no_slip", wall.astype(np.int32))


def dam_break_3d(dx=5e-3, L=1.2, H=0.55, W=1.0, TL=3.22, TH=1.0, TW=1.0, wall_layers=3, rho=1000.0, g=9.81,
                 alpha=0.05, mu=1.002e-3, c0=40.0, scheme=0, shepard=True, kernel=Quintic, hfac=1.3):
    """3D dam break: L (x) x H (y, up) x W (z) column in a TL x TH x TW tank.

    Built directly on the cubic lattice AddBoxLength would produce for the
    whole tank (4-DamBreak3D.cpp shape) without materialising the dropped
    particles; particle mass is that box's dx^3 rho rule (Source/Domain.cpp:399-415).
    Returns (domain, dt, info).
    """
    dom = Domain()
    dom.Dimension = 3
    dom.Scheme = scheme
    dom.Kernel_Set(kernel)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    h = hfac * dx
    r = dx / 2.0
    w = wall_layers
    V = (-w * dx, -w * dx, -w * dx)
    Ls = (2 * w * dx + TL + dx / 10.0, w * dx + TH + dx / 10.0, 2 * w * dx + TW + dx / 10.0)
    axes = []
    for d in range(3):
        n = Domain._count(V[d], V[d] + Ls[d] - r, lambda i, d=d: V[d] + (2.0 * i + 1) * r)
        axes.append(V[d] + (2.0 * np.arange(n) + 1) * r)
    xs, ys, zs = axes
    xwall = (xs < 0.0) | (xs > TL)
    xfl = (~xwall) & (xs <= L)
    zwall = (zs < 0.0) | (zs > TW)
    zfl = (~zwall) & (zs <= W)
    chunks = []
    wall_flags = []
    for yk, y in enumerate(ys):
        ywall = y < 0.0
        for zk, z in enumerate(zs):
            if ywall or zwall[zk]:
                sel = np.ones(len(xs), bool)  # whole row is wall
                is_wall = np.ones(len(xs), bool)
            else:
                is_wall = xwall
                sel = xwall | (xfl if (zfl[zk] and y <= H) else np.zeros(len(xs), bool))
            nsel = int(sel.sum())
            if nsel == 0:
                continue
            pts = np.empty((nsel, 3))
            pts[:, 0] = xs[sel]
            pts[:, 1] = y
            pts[:, 2] = z
            chunks.append(pts)
            wall_flags.append(is_wall[sel])
    X = np.concatenate(chunks)
    wall = np.concatenate(wall_flags)
    # AddBoxLength orders k (z) outer, j (y) middle, i (x) inner; reorder to match
    order = np.lexsort((X[:, 0], X[:, 1], X[:, 2]))
    X = np.ascontiguousarray(X[order])
    wall = wall[order]
    n = X.shape[0]
    ext = [(axes[d][-1] + r) - V[d] for d in range(3)]
    mass = ext[0] * ext[1] * ext[2] * rho / (len(xs) * len(ys) * len(zs))
    dom.particles.append(n, {"x": X, "mass": np.full(n, mass)})
    dom.R = r
    p = dom.particles
    cs = c0
    _fluid_fields(p, wall, rho, cs, mu, alpha, shepard, h)
    fl = ~wall
    yb = X[:, 1]
    dens = rho * np.power((1 + 7.0 * g * (H - yb[fl]) / (cs * cs)), (1.0 / 7.0))
    p.get("density")[fl] = dens
    p.get("densityb")[fl] = dens
    dom.InitialDist = dx
    dom.Gravity = [0.0, -g, 0.0]
    dt = 0.25 * h / cs
    return dom, dt, {"cs": cs, "H": H, "L": L, "g": g, "h": h, "n_fluid": int(fl.sum()), "n_wall": int(wall.sum())}


def granular_column(dx=1e-3, W=0.2, aspect=1.0, TL_factor=4.0, wall_layers=3, rho=1850.0, E=0.84e6, nu=0.3,
                    phi_deg=30.0, psi_deg=0.0, cohesion=0.0, fail=2, ti=0.5, tin=2.55, alpha=0.1, beta=0.1,
                    cs=None, scheme=0, g=9.81, hfac=1.2):
    """2D granular column collapse (Drucker-Prager soil, Material 3), as
    Old_Tests/ReposeAngle2.cpp: a W x (aspect W) column against a left wall on
    a floor, geostatic initial stress, Monaghan tensile-instability correction.
    Returns (domain, dt, info).
    """
    dom = Domain()
    dom.Dimension = 2
    dom.Scheme = scheme
    dom.Kernel_Set(Qubic_Spline)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    dom.Gravity = [0.0, -g, 0.0]
    H = aspect * W
    K = E / (3.0 * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    h = hfac * dx
    if cs is None:
        cs = math.sqrt(E / rho)
    w = wall_layers
    TL = TL_factor * W + (1.0 + aspect) * W
    dom.InitialDist = dx
    dom.AddBoxLength(1, (-w * dx, 0.0, 0.0), W + w * dx + dx / 10.0, H + dx / 10.0, 0, dx / 2.0, rho, h, 1, 0,
                     False, False)
    dom.AddBoxLength(1, (-w * dx, -w * dx, 0.0), TL + w * dx, w * dx + dx / 10.0, 0, dx / 2.0, rho, h, 1, 0,
                     False, False)
    p = dom.particles
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = (yb < 0.0) | ((xb < 0.0) & (yb > 0.0))
    n = p.n
    p.set("g_mod", G)
    p.set("cs", cs)
    p.set("k_mod", K)
    p.set("material", 3)
    p.set("fail", fail)
    p.set("cohesion", cohesion)
    p.set("phi", phi_deg / 180.0 * math.pi)
    p.set("psi", psi_deg / 180.0 * math.pi)
    p.set("alpha", alpha)
    p.set("beta", beta)
    p.set("ti", ti)
    p.set("tin", tin)
    p.set("ti_init_dist", dx)
    p.set("is_free", (~wall).astype(np.int32))
    p.set("no_slip", wall.astype(np.int32))
    ids = np.ones(n, np.int32)
    ids[wall] = 3
    p.set("id", ids)
    K0 = 1 - math.sin(phi_deg / 180.0 * math.pi)
    sig = p.get("sigma")
    fl = ~wall
    sig[fl, 1, 1] = rho * -g * (H - yb[fl])
    sig[fl, 0, 0] = K0 * rho * -g * (H - yb[fl])
    sig[fl, 2, 2] = K0 * rho * -g * (H - yb[fl])
    dt = 0.2 * h / cs
    return dom, dt, {"H": H, "W": W, "K": K, "G": G, "cs": cs, "h": h, "n_soil": int(fl.sum()),
                     "n_wall": int(wall.sum())}


def granular_column_3d(dx=0.01, W=0.06, D=0.04, aspect=1.0, TL_factor=1.0, wall_layers=3, rho=1850.0, E=0.84e6,
                       nu=0.3, phi_deg=30.0, psi_deg=0.0, cohesion=0.0, fail=2, ti=0.5, tin=2.55, alpha=0.1,
                       beta=0.1, cs=None, scheme=0, g=9.81, hfac=1.2, tension=0.0, seed=0):
    """3D granular column (Drucker-Prager soil, Material 3, full 3D yield
    surface): a W (x) x aspect W (y, up) x D (z) column on a fixed floor that
    extends TL_factor W beyond it in x and wall_layers beyond it elsewhere,
    geostatic initial stress, Monaghan tensile-instability correction. With
    tension > 0 a seeded symmetric stress of that magnitude is added to the
    soil, so some particles start with a principal stress in tension and the
    tensile-instability rotation (StartAcceleration's 3D branch,
    Source/Domain.cpp:979-987) has work to do. Returns (domain, dt, info)."""
    dom = Domain()
    dom.Dimension = 3
    dom.Scheme = scheme
    dom.Kernel_Set(Qubic_Spline)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    dom.Gravity = [0.0, -g, 0.0]
    H = aspect * W
    K = E / (3.0 * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    h = hfac * dx
    if cs is None:
        cs = math.sqrt(E / rho)
    w = wall_layers
    dom.InitialDist = dx
    dom.AddBoxLength(1, (0.0, 0.0, 0.0), W + dx / 10.0, H + dx / 10.0, D + dx / 10.0, dx / 2.0, rho, h, 1, 0,
                     False, False)
    dom.AddBoxLength(3, (-w * dx, -w * dx, -w * dx), (1.0 + TL_factor) * W + 2 * w * dx + dx / 10.0,
                     w * dx + dx / 10.0, D + 2 * w * dx + dx / 10.0, dx / 2.0, rho, h, 1, 0, False, True)
    p = dom.particles
    x = p.get("x")
    yb = x[:, 1]
    wall = p.get("is_free") == 0
    n = p.n
    p.set("g_mod", G)
    p.set("cs", cs)
    p.set("k_mod", K)
    p.set("material", 3)
    p.set("fail", fail)
    p.set("cohesion", cohesion)
    p.set("phi", phi_deg / 180.0 * math.pi)
    p.set("psi", psi_deg / 180.0 * math.pi)
    p.set("alpha", alpha)
    p.set("beta", beta)
    p.set("ti", ti)
    p.set("tin", tin)
    p.set("ti_init_dist", dx)
    p.set("no_slip", wall.astype(np.int32))
    K0 = 1 - math.sin(phi_deg / 180.0 * math.pi)
    sig = p.get("sigma")
    fl = ~wall
    sig[fl, 1, 1] = rho * -g * (H - yb[fl])
    sig[fl, 0, 0] = K0 * rho * -g * (H - yb[fl])
    sig[fl, 2, 2] = K0 * rho * -g * (H - yb[fl])
    if tension > 0.0:
        rng = np.random.default_rng(seed)
        m = rng.uniform(-tension, tension, size=(int(fl.sum()), 3, 3))
        sig[fl] += 0.5 * (m + np.transpose(m, (0, 2, 1)))
    dt = 0.2 * h / cs
    return dom, dt, {"H": H, "W": W, "D": D, "K": K, "G": G, "cs": cs, "h": h, "n_soil": int(fl.sum()),
                     "n_wall": int(wall.sum())}


def seepage_bed_2d(**kw):
    """seepage_bed in 2D."""
    return seepage_bed(dim=2, **kw)


def seepage_bed(dim=2, dx=0.01, L=0.3, H=0.2, Hs=0.1, TL=0.6, TW=0.1, wall_layers=3, rho_f=1000.0, rho_grain=1580.0,
                   n0=0.42, grain=0.00392, E=5.0e6, nu=0.3, phi_deg=38.0, swi=0, seepage_type=1,
                   var_porosity=False, k=1.0e-9, k2=0.0, grains=0, scheme=0, g=9.81, hfac=1.2, mu=1.0e-3,
                   alpha=0.1, seed=0, sat_from_x=None, cohesion=0.0):
    """Dam break over an erodible soil bed, the shape of Old_Tests/Dam_Scouring2.cpp
    (in 2D, or in 3D with a tank TW deep in z):
    a TL-wide tank whose lower Hs is a saturated-density soil bed (Material 3,
    Drucker-Prager, non-associated Fail 3, density (1 - n0) rho_grain + n0 rho_f)
    and an L x H water column (Material 1) on the bed at the left. Walls are soil
    below the bed surface and fluid above it, so every pair type meets: fluid and
    soil with their own kind and walls, fluid with soil, and each with the other's
    walls. `grains` water particles (chosen with numpy default_rng(seed)) become
    soil grains suspended in the water (the surface-erosion branch of SWIType 1
    acts on soil with few soil neighbours). SWIType `swi`, SeepageType
    `seepage_type` (k and k2 are used as given for type 0, derived from n0 and
    the grain size otherwise). Bed particles right of `sat_from_x` start marked
    saturated (IsSat), as after a drained flood. Returns (domain, dt, info).
    """
    dom = Domain()
    dom.Dimension = dim
    dom.Scheme = scheme
    dom.Kernel_Set(Qubic_Spline)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    dom.Gravity = [0.0, -g, 0.0]
    dom.SWIType = swi
    dom.InitialDist = dx
    h = hfac * dx
    rho_s = rho_grain * (1.0 - n0) + n0 * rho_f
    K = E / (3.0 * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    cs_s = math.sqrt(K / (rho_s - rho_f))
    cs_f = 10.0 * math.sqrt(2.0 * g * H)
    TH = Hs + H + 2 * dx
    _tank(dom, dx, TL, TH, TW if dim == 3 else 0.0, wall_layers)
    p = dom.particles

    def walls(x):
        w = (x[:, 0] < 0.0) | (x[:, 1] < 0.0) | (x[:, 0] > TL)
        if dim == 3:
            w |= (x[:, 2] < 0.0) | (x[:, 2] > TW)
        return w

    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = walls(x)
    bed = (~wall) & (yb < Hs)
    water = (~wall) & (yb >= Hs) & (yb < Hs + H) & (xb < L)
    p.keep(wall | bed | water)
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = walls(x)
    soil = yb < Hs
    water = (~wall) & (~soil)
    if grains:
        rng = np.random.default_rng(seed)
        pick = rng.choice(np.flatnonzero(water), size=grains, replace=False)
        soil = soil.copy()
        soil[pick] = True
    fluid = ~soil
    n = p.n
    p.set("h", h)
    p.set("material", np.where(soil, 3, 1).astype(np.int32))
    p.set("is_free", (~wall).astype(np.int32))
    p.set("no_slip", wall.astype(np.int32))
    ids = np.where(wall, np.where(soil, 4, 2), np.where(soil, 3, 1)).astype(np.int32)
    p.set("id", ids)
    p.set("alpha", alpha)
    # fluid: Tait EOS, hydrostatic density above the bed
    dens = np.full(n, rho_s)
    fl_free = fluid & ~wall
    dens[fluid] = rho_f
    dens[fl_free] = rho_f * np.power(1 + 7.0 * g * (Hs + H - yb[fl_free]) / (cs_f * cs_f), 1.0 / 7.0)
    p.set("density", dens)
    p.set("densityb", dens)
    p.set("ref_density", np.where(soil, rho_s, rho_f))
    p.set("cs", np.where(soil, cs_s, cs_f))
    p.set("pres_eq", np.where(soil, 0, 1).astype(np.int32))
    p.set("mu", np.where(soil, 0.0, mu))
    p.set("mu_ref", np.where(soil, 0.0, mu))
    p.set("mass", np.where(soil, rho_s, rho_f) * dx ** dim)
    # soil: Drucker-Prager, geostatic stress of the bed
    p.set("beta", np.where(soil, 0.1, 0.0))
    p.set("g_mod", np.where(soil, G, 0.0))
    p.set("k_mod", np.where(soil, K, 0.0))
    p.set("fail", np.where(soil, 3, 0).astype(np.int32))
    p.set("phi", np.where(soil, phi_deg / 180.0 * math.pi, 0.0))
    p.set("cohesion", np.where(soil, cohesion, 0.0))
    p.set("seepage_type", np.where(soil, seepage_type, 0).astype(np.int32))
    p.set("var_porosity", (soil & bool(var_porosity)).astype(np.int32))
    p.set("n0", np.where(soil, n0, 0.0))
    p.set("d", np.where(soil, grain, 0.0))
    p.set("rho_f", np.where(soil, rho_f, 0.0))
    p.set("k", np.where(soil, k, 0.0))
    p.set("k2", np.where(soil, k2, 0.0))
    if sat_from_x is not None:
        p.set("is_sat", (soil & ~wall & (xb > sat_from_x)).astype(np.int32))
    sig = p.get("sigma")
    bed_free = soil & ~wall & (yb < Hs)
    K0 = 1 - math.sin(phi_deg / 180.0 * math.pi)
    depth = Hs - yb[bed_free]
    sig[bed_free, 1, 1] = -(rho_s - rho_f) * g * depth
    sig[bed_free, 0, 0] = K0 * sig[bed_free, 1, 1]
    sig[bed_free, 2, 2] = K0 * sig[bed_free, 1, 1]
    dt = min(0.25 * h / cs_f, 0.2 * h / cs_s)
    return dom, dt, {"h": h, "cs_f": cs_f, "cs_s": cs_s, "n_fluid": int((fluid & ~wall).sum()),
                     "n_soil": int((soil & ~wall).sum()), "n_wall": int(wall.sum())}


def elastic_gate_2d(dx=0.01, L1=0.2, H=0.15, Tr=0.03, H1=0.15, TL_extra=0.1, wall_layers=3, rho_f=1000.0,
                    rho_r=1100.0, K=2.0e7, G=4.27e6, mu=1.0e-3, fsi=False, scheme=0, g=9.81, hfac=1.2, ti=0.3):
    """2D water column held by an elastic gate, the shape of
    Old_Tests/FSI_ElasticGate.cpp: water (Material 1) fills x < L1 up to H in a
    tank; a gate of thickness Tr (Material 2, hypoelastic, PresEq 0, sound
    speed sqrt(K / rho_r), artificial viscosity alpha 1, tensile-instability
    correction `ti`) stands at x = L1 from two layers above the floor to H1,
    clamped by three fixed layers above H1. Fluid and gate meet through
    CalcForce12; `fsi` turns on the reference's FSI interpolation of the
    gate's pressure and velocity. Returns (domain, dt, info).
    """
    dom = Domain()
    dom.Dimension = 2
    dom.Scheme = scheme
    dom.Kernel_Set(Qubic_Spline)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    dom.Gravity = [0.0, -g, 0.0]
    dom.FSI = bool(fsi)
    dom.InitialDist = dx
    h = hfac * dx
    cs_w = 10.0 * math.sqrt(2.0 * g * H) * 2.0
    cs_r = math.sqrt(K / rho_r)
    TL = L1 + Tr + TL_extra
    TH = H1 + 4 * dx
    _tank(dom, dx, TL, TH, 0.0, wall_layers)
    p = dom.particles
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = (xb < 0.0) | (yb < 0.0) | (xb > TL)
    p.keep(wall | ((xb < L1) & (yb < H)))
    n_tank = p.n
    dom.AddBoxLength(3, (L1, 0.0, 0.0), Tr + dx / 10.0, H1 + 3.0 * dx + dx / 10.0, 0, dx / 2.0, rho_r, h, 1, 0,
                     False, False)
    p = dom.particles
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    gate = np.zeros(p.n, bool)
    gate[n_tank:] = True
    keep = ~gate | (yb >= 2.0 * dx)
    p.keep(keep)
    gate = gate[keep]
    x = p.get("x")
    xb, yb = x[:, 0], x[:, 1]
    wall = (~gate) & ((xb < 0.0) | (yb < 0.0) | (xb > TL))
    clamp = gate & (yb > H1)
    fixed = wall | clamp
    water = ~gate & ~wall
    p.set("h", h)
    p.set("material", np.where(gate, 2, 1).astype(np.int32))
    p.set("is_free", (~fixed).astype(np.int32))
    p.set("no_slip", fixed.astype(np.int32))
    p.set("id", np.where(gate, np.where(clamp, 4, 3), np.where(wall, 2, 1)).astype(np.int32))
    rho = np.where(gate, rho_r, rho_f).astype(float)
    dens = rho.copy()
    dens[water] = rho_f * np.power(1 + 7.0 * g * (H - yb[water]) / (cs_w * cs_w), 1.0 / 7.0)
    p.set("density", dens)
    p.set("densityb", dens)
    p.set("ref_density", rho)
    p.set("mass", rho * dx * dx)
    p.set("cs", np.where(gate, cs_r, cs_w))
    p.set("pres_eq", np.where(gate, 0, 1).astype(np.int32))
    p.set("mu", np.where(gate, 0.0, mu))
    p.set("mu_ref", np.where(gate, 0.0, mu))
    p.set("alpha", np.where(gate, 1.0, 0.1))
    p.set("g_mod", np.where(gate, G, 0.0))
    p.set("ti", np.where(gate, ti, 0.0))
    p.set("ti_init_dist", np.where(gate, dx, 0.0))
    dt = min(0.2 * h / cs_w, 0.2 * h / cs_r)
    return dom, dt, {"h": h, "cs_w": cs_w, "cs_r": cs_r, "n_water": int(water.sum()),
                     "n_gate": int((gate & ~clamp).sum()), "n_fixed": int(fixed.sum())}


def soil_damping_hook(damp, t_end, material, t_change, tag, cohesion, phi):
    """A GeneralAfter hook in the style of the reference's soil drivers
    (Old_Tests/Embankment.cpp:31-58, UserDamping): while Time < t_end the free
    particles of `material` are damped (a -= damp v); from t_change on, the
    particles with ID `tag` of that material take the given cohesion and
    friction angle (radians). Takes the Domain, as the reference's hooks do."""
    def hook(dom):
        p = dom.particles
        mat = p.get("material")
        if dom.Time < t_end:
            sel = (p.get("is_free") != 0) & (mat == material)
            a, v = p.get("a"), p.get("v")
            a[sel] -= damp * v[sel]
            p.set("a", a)
        if dom.Time >= t_change:
            sel = (p.get("id") == tag) & (mat == material)
            c, ph = p.get("cohesion"), p.get("phi")
            c[sel] = cohesion
            ph[sel] = phi
            p.set("cohesion", c)
            p.set("phi", ph)
    return hook


def spring_hook(k, xc, yc):
    """A GeneralBefore hook adding a position-dependent acceleration to the free
    particles: a += k (centre - x) in x and y."""
    def hook(dom):
        p = dom.particles
        free = p.get("is_free") != 0
        a, x = p.get("a"), p.get("x")
        a[free, 0] += k * (xc - x[free, 0])
        a[free, 1] += k * (yc - x[free, 1])
        p.set("a", a)
    return hook


def channel_profiles(H, cs, g=9.81):
    """User InCon / OutCon hooks written the way the reference's drivers write
    theirs (Old_Tests/HydraulicJump.cpp:29-53): the in-flow gets a parabolic
    velocity across a channel of height H (BC.inv[0] at its centre) and the
    hydrostatic Tait density under the level H; the out-flow gets BC.outv[0]
    scaled by 0.5 + y/H and the hydrostatic density under the level H/2
    (BC.outDensity above it). Each hook maps (position, BC) to (velocity,
    density)."""
    def in_con(x, bc):
        y = float(x[1])
        vel = (bc.inv[0] * 4.0 * y * (H - y) / (H * H), 0.0, 0.0)
        den = bc.inDensity * math.pow((1.0 + 7.0 * g * (H - y) / (cs * cs)), 1.0 / 7.0)
        return vel, den

    def out_con(x, bc):
        y = float(x[1])
        vel = (bc.outv[0] * (0.5 + y / H), 0.0, 0.0)
        den = bc.outDensity * math.pow((1.0 + 7.0 * g * (0.5 * H - y) / (cs * cs)), 1.0 / 7.0)
        if y > 0.5 * H:
            den = bc.outDensity
        return vel, den

    return in_con, out_con


def channel_flow_2d(dx=0.01, L=0.5, H=0.1, U=2.0, cs=20.0, flow=3, mass_conservation=False, out_v=None,
                    out_density=None, wall_layers=3, rho=1000.0, mu=1.0e-3, alpha=0.1, scheme=0, hfac=1.2,
                    profile=False):
    """2D channel with in/out-flow boundaries, the shape of Old_Tests/Current-flow.cpp:
    water between two no-slip walls, L long and H high, particles entering at
    -x with velocity (U, 0, 0) and density rho (BC.inv, BC.inDensity; the
    default InCon), leaving at +x (BC.InOutFlow = `flow`; BC.outv and
    BC.outDensity as given, with BC.MassConservation), no gravity. Particles
    that cross the in-flow zone are recycled upstream. Returns (domain, dt, info)."""
    dom = Domain()
    dom.Dimension = 2
    dom.Scheme = scheme
    dom.Kernel_Set(Qubic_Spline)
    dom.Viscosity_Eq_Set(Morris)
    dom.Gradient_Approach_Set(Squared_density)
    dom.Gravity = [0.0, 0.0, 0.0]
    dom.InitialDist = dx
    h = hfac * dx
    w = wall_layers
    dom.AddBoxLength(1, (0.0, -w * dx, 0.0), L + dx / 10.0, H + 2 * w * dx + dx / 10.0, 0, dx / 2.0, rho, h, 1, 0,
                     False, False)
    p = dom.particles
    x = p.get("x")
    yb = x[:, 1]
    wall = (yb < 0.0) | (yb > H)
    p.set("h", h)
    p.set("density", rho)
    p.set("ref_density", rho)
    p.set("cs", cs)
    p.set("pres_eq", 1)
    p.set("mu", mu)
    p.set("mu_ref", mu)
    p.set("material", 1)
    p.set("alpha", alpha)
    p.set("id", np.where(wall, 2, 1).astype(np.int32))
    p.set("is_free", (~wall).astype(np.int32))
    p.set("no_slip", wall.astype(np.int32))
    v = p.get("v")
    v[~wall, 0] = U
    p.set("mass", rho * dx * dx)
    dom.BC.InOutFlow = flow
    dom.BC.inv = [U, 0.0, 0.0]
    dom.BC.inDensity = rho
    dom.BC.MassConservation = bool(mass_conservation)
    if out_v is not None:
        dom.BC.outv = list(out_v)
    if out_density is not None:
        dom.BC.outDensity = out_density
    info = {"h": h, "cs": cs, "U": U, "n_fluid": int((~wall).sum()), "n_wall": int(wall.sum())}
    if profile:  # user hooks instead of the BC constants
        dom.InCon, dom.OutCon = channel_profiles(H, cs)
        info["flow_profile"] = (H, cs, 9.81)
    dt = 0.25 * h / cs
    return dom, dt, info


def granular_ensemble(n=256, seed=0, dx=1e-3, W=0.2, aspect=(0.5, 4.0), phi_deg=(20.0, 40.0), fail=2, **kw):
    """The batched granular-column workload: n independent 2D columns of width W
    at lattice spacing dx, aspect ratio H/W and friction angle drawn uniformly
    from the given ranges (numpy default_rng(seed)), cohesion 0, rho 1850,
    E 0.84 MPa, nu 0.3, Monaghan tensile-instability correction on. Particle
    counts follow from the geometry: W = 0.2 m at dx = 1 mm gives 200 x 100 to
    200 x 800 soil particles per column. Returns [(domain, dt, info)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a = float(rng.uniform(*aspect))
        phi = float(rng.uniform(*phi_deg))
        dom, dt, info = granular_column(dx=dx, W=W, aspect=a, phi_deg=phi, fail=fail, cohesion=0.0, **kw)
        info.update({"aspect": a, "phi_deg": phi})
        out.append((dom, dt, info))
    return out
