"""In/out-flow boundaries on the GPU (InFlowBCFresh and InFlowBCLeave,
Source/Domain.cpp:1327-1635): the particle count, the in/out-flow flags and
the recycled particles' state against the reference's golden trajectories,
and the combinations this build rejects. x, v, density and pressure of the
same cases are checked with every other case in test_gpu_parity.py."""
import os

import numpy as np
import pytest

from persiansph_gb300 import scenarios
from persiansph_gb300.abi import PsphError
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLOW = sorted(k for k in CASES if k.startswith("channel_"))


@pytest.mark.parametrize("name", FLOW)
def test_inout_state_matches_reference(gpu, name):
    """Particle count, Particle::InOut and the class of every particle (mass,
    T0 of the recycled ones) equal the reference's at every stored step,
    including the steps that append and delete particles."""
    builder, _, dumps = CASES[name]
    dom, dt, _ = builder()
    g = dict(np.load(os.path.join(GOLD, name + ".npz")))
    gd = GpuDomain(dom.config(dt))
    gd.use_flow_hooks(dom)
    gd.upload(dom.particles, initial=True)
    prev = 0
    for k in dumps:
        gd.step(k - prev)
        prev = k
        assert gd.n == int(g[f"n_{k}"]), f"{name} step {k}: particle count"
        st = gd.download_fields()
        assert np.array_equal(st["in_out"], g[f"in_out_{k}"]), f"{name} step {k}: in/out-flow flags"
        assert np.array_equal(st["mass"], g[f"mass_{k}"]), f"{name} step {k}: masses"
        scale = np.max(np.abs(g[f"x_{k}"]))
        err = np.max(np.abs(st["x"] - g[f"x_{k}"])) / scale
        assert err <= 1e-9, f"{name} step {k}: positions {err:.3e}"


def _rejected(dom, dt, **cfg_changes):
    cfg = dom.config(dt)
    for key, val in cfg_changes.items():
        setattr(cfg, key, val)
    gd = GpuDomain(cfg)
    with pytest.raises(PsphError) as e:
        gd.upload(dom.particles, initial=True)
    return e.value


def test_inout_needs_fp64(gpu):
    dom, dt, _ = scenarios.channel_flow_2d()
    err = _rejected(dom, dt, precision=1)
    assert err.code == 2 and "FP64" in str(err)


def test_inout_rejects_shepard(gpu):
    """The reference restarts a released in-flow particle's own Shepard
    counter; this build keeps one counter per domain."""
    dom, dt, _ = scenarios.channel_flow_2d()
    dom.particles.set("shepard", 1)
    err = _rejected(dom, dt)
    assert err.code == 2 and "Shepard" in str(err)


def test_inout_rejects_periodic_x(gpu):
    dom, dt, _ = scenarios.channel_flow_2d()
    cfg = dom.config(dt)
    cfg.periodic[0] = 1
    with pytest.raises(PsphError) as e:
        GpuDomain(cfg)
    assert e.value.code == 1 and "Periodic" in str(e.value)


def test_flow_profile_errors(gpu):
    """A user InCon that raises stops the step with its exception; a profile
    on a domain without in/out-flow boundaries is refused."""
    dom, dt, _ = scenarios.channel_flow_2d()
    gd = GpuDomain(dom.config(dt))

    def bad(x):
        raise ValueError("profile failed")

    gd.set_flow_profile(1, bad)
    gd.upload(dom.particles, initial=True)
    with pytest.raises(ValueError, match="profile failed"):
        gd.step(1)
    plain, dt2, _ = scenarios.dam_break_2d(dx=0.02)
    gp = GpuDomain(plain.config(dt2))
    with pytest.raises(PsphError) as e:
        gp.set_flow_profile(1, lambda x: ((0.0, 0.0, 0.0), 1000.0))
    assert e.value.code == 10


def test_flow_profile_default_restored(gpu):
    """Setting a profile and then None gives the default constants' trajectory."""
    dom, dt, _ = scenarios.channel_flow_2d(flow=3, out_density=1000.0)
    ref = GpuDomain(dom.config(dt))
    ref.upload(dom.particles, initial=True)
    ref.step(12)
    gd = GpuDomain(dom.config(dt))
    gd.set_flow_profile(1, lambda x: ((9.0, 0.0, 0.0), 1010.0))
    gd.set_flow_profile(1, None)
    gd.upload(dom.particles, initial=True)
    gd.step(12)
    a, b = ref.download_fields(("x", "density")), gd.download_fields(("x", "density"))
    np.testing.assert_array_equal(a["x"], b["x"])
    np.testing.assert_array_equal(a["density"], b["density"])
