"""Host-side Domain API behaviour (no GPU)."""
import numpy as np
import pytest

from persiansph_gb300 import Domain, Fatal, scenarios


def test_del_particles_missing_tag_raises():
    dom = Domain()
    dom.AddSingleParticle(1, (0.0, 0.0, 0.0), 1.0, 1000.0, 0.01, False)
    with pytest.raises(Fatal):
        dom.DelParticles(7)


def test_particle_views_and_defaults():
    dom = Domain()
    dom.AddBoxLength(3, (0, 0, 0), 0.1, 0.1, 0.0, 0.005, 1000.0, 0.012, 1, 0, False, True)
    P = dom.Particles
    assert len(P) == 100
    assert P[0].IsFree is False and P[0].ID == 3 and P[0].RefDensity == 1000.0
    assert P[5].FPMassC == 1.0 and P[5].TIn == 4.0 and P[5].CSmag == 0.17
    P[5].Density = 1001.0
    assert dom.particles.get("density")[5] == 1001.0


def test_kernel_set_cellfac_and_config():
    dom = Domain()
    dom.Kernel_Set(2)
    assert dom._cellfac == 3.0
    dom.Kernel_Set(0)
    assert dom._cellfac == 2.0
    cfg = dom.config(1e-4)
    assert cfg.dt == 1e-4 and cfg.shepard_step == 40 and cfg.sqrt_h_a == 0.0025


def test_bad_packing_raises():
    dom = Domain()
    with pytest.raises(Fatal):
        dom.AddBoxLength(1, (0, 0, 0), 0.1, 0.1, 0.0, 0.005, 1000.0, 0.012, 3, 0, False, False)


def test_scenario_sizes():
    dom, dt, info = scenarios.dam_break_2d(dx=0.05, L=1.0, H=2.0, TL=4.0, TH=3.0)
    assert info["n_fluid"] == 20 * 40
    dom, dt, info = scenarios.poiseuille()
    assert dom.particles.n == 920
