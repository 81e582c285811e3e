"""Parity cases shared by the golden generator and the tests.

Each case: builder() -> (Domain, dt, info), number of reference steps, and the
steps after which the reference state is stored. The steps are chosen to cover
the Modified Verlet restart (ct==30: steps 1 and 32), the Shepard
re-initialisation (ShepardCounter==40: step 41) and the Leapfrog first step.
"""
import math

from persiansph_gb300 import scenarios
from persiansph_gb300.domain import Multiplied_density, Takeda, Shao, Incompressible_Full


def dam2d():
    return scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.8, TL=1.6, TH=1.2)


def dam2d_leapfrog():
    return scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.8, TL=1.6, TH=1.2, scheme=1, shepard=False)


def poiseuille():
    return scenarios.poiseuille(dx=2.5e-5)


def granular():
    return scenarios.granular_column(dx=0.01, W=0.2, aspect=1.0)


def granular_lf_fail3():
    return scenarios.granular_column(dx=0.01, W=0.2, aspect=2.0, scheme=1, fail=3, psi_deg=5.0, cohesion=100.0)


def dam3d():
    return scenarios.dam_break_3d(dx=0.04, L=0.24, H=0.2, W=0.16, TL=0.48, TH=0.32, TW=0.2)


def fluid_options():
    """Takeda viscosity, multiplied-density gradient, XSPH and LES on a small dam break."""
    dom, dt, info = scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.6, TL=1.0, TH=0.8, shepard=False)
    dom.Viscosity_Eq_Set(Takeda)
    dom.Gradient_Approach_Set(Multiplied_density)
    dom.XSPH = 0.5
    p = dom.particles
    p.set("les", 1)
    p.set("beta", 0.05)
    return dom, dt, info


def fluid_shao_bingham():
    dom, dt, info = scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.6, TL=1.0, TH=0.8, kernel=2, hfac=1.3,
                                           scheme=1, shepard=False)
    dom.Viscosity_Eq_Set(Shao)
    p = dom.particles
    p.set("t0", 5.0)
    p.set("mu_ref", 0.05)
    return dom, dt, info


def fluid_incomp_quintic():
    dom, dt, info = scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.6, TL=1.0, TH=0.8, kernel=1, hfac=1.3)
    dom.Viscosity_Eq_Set(Incompressible_Full)
    p = dom.particles
    p.set("ti", 0.2)
    p.set("tin", 3.0)
    p.set("ti_init_dist", 0.02)
    p.set("pres_eq", 0)
    return dom, dt, info


def solid_block():
    """Elastic (Material 2, von Mises cap) block resting on a fixed floor, leapfrog."""
    dom, dt, info = scenarios.granular_column(dx=0.01, W=0.2, aspect=0.5, scheme=1, fail=1)
    p = dom.particles
    p.set("material", 2)
    p.set("sigmay", 2.0e3)
    p.set("pres_eq", 0)
    p.set("ti", 0.0)
    return dom, dt, info


def soil3d_ti():
    """3D Drucker-Prager soil column on a floor with the tensile-instability
    correction; a seeded stress perturbation puts principal stresses in
    tension, so StartAcceleration's 3D eigen-rotation (Source/Domain.cpp:979-987)
    produces non-zero TIR."""
    return scenarios.granular_column_3d(dx=0.01, W=0.06, D=0.04, aspect=1.0, tension=300.0, cohesion=200.0)


def fluid_preseq2():
    """PresEq 2 (p = c^2 rho, Source/Functions.cpp:188-212) on a small leapfrog dam break."""
    dom, dt, info = scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.6, TL=1.0, TH=0.8, scheme=1, shepard=False)
    dom.particles.set("pres_eq", 2)
    return dom, dt, info


# The seepage cases' soil has 1 kPa cohesion: a cohesionless bed surface sits
# on the Drucker-Prager apex, where rounding-level differences (a different
# summation order) switch the return mapping's branch within tens of steps and
# no two correct implementations agree to 1e-9 (measured on the oracle with
# 1e-14 position noise: 4e-4 after 25 steps, 4e-13 with the cohesion).


def seep_darcy():
    """Fluid over a soil bed, SWIType 0 (seepage force + buoyant weight), Kozeny-Carman permeability;
    the dry right part of the bed starts marked saturated, so it switches back at the first step."""
    return scenarios.seepage_bed_2d(swi=0, seepage_type=1, sat_from_x=0.45, cohesion=1000.0)


def seep_erosion_ergun():
    """SWIType 1 (seepage + surface erosion of suspended grains), Ergun permeability following the
    volumetric strain (VarPorosity), leapfrog."""
    return scenarios.seepage_bed_2d(swi=1, seepage_type=2, var_porosity=True, grains=6, scheme=1, cohesion=1000.0)


def seep_pore_pressure():
    """SWIType 2 (seepage + pore pressure of the fluid), Den Adel permeability."""
    return scenarios.seepage_bed_2d(swi=2, seepage_type=3, cohesion=1000.0)


def seep_buoyancy_only():
    """SWIType 3 (no drag; saturated soil still weighs its buoyant weight), Darcy with a given k."""
    return scenarios.seepage_bed_2d(swi=3, seepage_type=0, k=2.0e-9, cohesion=1000.0)


def seep3d_erosion():
    """3D fluid over a soil bed: SWIType 1, Ergun permeability with VarPorosity, suspended grains."""
    return scenarios.seepage_bed(dim=3, dx=0.02, L=0.16, H=0.1, Hs=0.06, TL=0.3, TW=0.1, swi=1, seepage_type=2,
                                 var_porosity=True, grains=4, cohesion=1000.0)


def channel_inout():
    """In/out-flow channel (InOutFlow 3), out-flow density prescribed, Modified Verlet over the
    ct==30 restart: at step 9 an in-flow column is released and its copies are appended upstream
    (beyond the grid box, as the reference places them), at step 10 they leave and the surplus
    slots are deleted."""
    return scenarios.channel_flow_2d(flow=3, out_density=1000.0)


def channel_inflow_mc():
    """InOutFlow 3 with mass conservation and an out-flow velocity, leapfrog."""
    return scenarios.channel_flow_2d(flow=3, mass_conservation=True, out_v=(2.0, 0.0, 0.0), scheme=1)


def granular_damped():
    """A cohesive granular column with a GeneralAfter hook in the style of the reference's soil
    drivers: damping of the soil's accelerations for the first 20 steps, and a new cohesion and
    friction angle for the upper half of the column (ID 6) from step 10 on."""
    dom, dt, info = scenarios.granular_column(dx=0.01, W=0.2, aspect=1.0, cohesion=1000.0)
    p = dom.particles
    ids = p.get("id")
    upper = (p.get("material") == 3) & (p.get("is_free") != 0) & (p.get("x")[:, 1] > 0.1)
    ids[upper] = 6
    p.set("id", ids)
    damping = [50.0, 20.5 * dt, 3, 10.5 * dt, 6, 500.0, 25.0 / 180.0 * math.pi]
    dom.GeneralAfter = scenarios.soil_damping_hook(*damping)
    info["damping"] = damping
    return dom, dt, info


def dam_spring():
    """A small dam break with a GeneralBefore hook that adds a position-dependent acceleration."""
    dom, dt, info = scenarios.dam_break_2d(dx=0.02, L=0.4, H=0.6, TL=1.0, TH=0.8)
    spring = [20.0, 0.5, 0.3]
    dom.GeneralBefore = scenarios.spring_hook(*spring)
    info["spring"] = spring
    return dom, dt, info


def channel_profile():
    """InOutFlow 3 with user InCon / OutCon hooks (parabolic in-flow velocity, hydrostatic densities,
    a scaled out-flow velocity) and mass conservation, Modified Verlet."""
    return scenarios.channel_flow_2d(flow=3, mass_conservation=True, out_v=(2.0, 0.0, 0.0), out_density=1000.0,
                                     profile=True)


def gate_fsi_off():
    """Water behind an elastic gate (Material 2), coupled by CalcForce12 with the FSI interpolation off."""
    return scenarios.elastic_gate_2d(fsi=False)


def gate_fsi_on():
    """The same with the FSI interpolation of the gate's pressure and velocity, leapfrog."""
    return scenarios.elastic_gate_2d(fsi=True, scheme=1)


CASES = {
    "dam2d": (dam2d, 42, (1, 2, 32, 41, 42)),
    "dam2d_leapfrog": (dam2d_leapfrog, 5, (1, 2, 5)),
    "poiseuille": (poiseuille, 20, (1, 5, 20)),
    "granular": (granular, 40, (1, 2, 32, 40)),
    "granular_lf_fail3": (granular_lf_fail3, 10, (1, 2, 10)),
    "dam3d": (dam3d, 3, (1, 3)),
    "fluid_options": (fluid_options, 5, (1, 5)),
    "fluid_shao_bingham": (fluid_shao_bingham, 5, (1, 5)),
    "fluid_incomp_quintic": (fluid_incomp_quintic, 5, (1, 5)),
    "solid_block": (solid_block, 6, (1, 6)),
    "soil3d_ti": (soil3d_ti, 5, (1, 2, 5)),
    "fluid_preseq2": (fluid_preseq2, 3, (1, 3)),
    "seep_darcy": (seep_darcy, 32, (1, 2, 32)),
    "seep_erosion_ergun": (seep_erosion_ergun, 20, (1, 2, 20)),
    "seep_pore_pressure": (seep_pore_pressure, 10, (1, 10)),
    "seep_buoyancy_only": (seep_buoyancy_only, 10, (1, 10)),
    "seep3d_erosion": (seep3d_erosion, 10, (1, 2, 10)),
    "channel_inout": (channel_inout, 40, (1, 2, 9, 10, 20, 32, 40)),
    "channel_inflow_mc": (channel_inflow_mc, 40, (1, 20, 40)),
    "channel_profile": (channel_profile, 40, (1, 9, 10, 20, 40)),
    "granular_damped": (granular_damped, 40, (1, 10, 11, 20, 21, 40)),
    "dam_spring": (dam_spring, 20, (1, 10, 20)),
    "gate_fsi_off": (gate_fsi_off, 32, (1, 2, 32)),
    "gate_fsi_on": (gate_fsi_on, 20, (1, 2, 20)),
}

# AddBoxLength argument lists: dim, tag, V, Lx, Ly, Lz, r, rho, h, type, rotation, random, fixed
BOXES = {
    "cubic2d": (2, 1, (-0.03, -0.03, 0.0), 0.5, 0.3, 0.0, 0.005, 1000.0, 0.012, 1, 0, False, False),
    "hex2d": (2, 1, (0.0, 0.0, 0.0), 0.2, 0.15, 0.0, 0.005, 1000.0, 0.012, 0, 0, False, False),
    "hex2d_rot": (2, 1, (0.0, 0.0, 0.0), 0.2, 0.15, 0.0, 0.005, 1000.0, 0.012, 0, 90, False, False),
    "cubic3d": (3, 1, (-0.06, -0.06, -0.06), 0.3, 0.2, 0.25, 0.01, 998.21, 0.024, 1, 0, False, False),
    "hex3d": (3, 1, (0.0, 0.0, 0.0), 0.2, 0.15, 0.12, 0.01, 1000.0, 0.024, 0, 0, False, True),
}


def surge2d():
    """Dam break used for the surge-front check: 0.5 x 1.0 m column in a 2.0 x 1.5 m tank, dx = 10 mm."""
    return scenarios.dam_break_2d(dx=0.01, L=0.5, H=1.0, TL=2.0, TH=1.5)


SURGE_STEPS = tuple(range(500, 5501, 500))


def surge_front(x, is_free, dx=0.01):
    """Surge-front position: largest x of a free particle within 2 dx of the floor."""
    free = is_free == 1
    low = x[:, 1] < 2.0 * dx
    sel = free & low
    return float(x[sel, 0].max())
