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
