"""Host hooks inside a step (Domain::GeneralBefore / GeneralAfter,
Source/Domain.cpp:1767-1770) on the GPU: hooks that change nothing leave
the trajectory bit for bit as without them, in both forms; psph_patch refuses
parameter changes that would change the step's kernels. The hook cases of
tests/golden/cases.py (granular_damped, dam_spring) run against the oracle
and the reference in test_gpu_parity.py with every other case."""
import numpy as np
import pytest

from persiansph_gb300 import scenarios
from persiansph_gb300.abi import PsphError
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,precision", [("dam2d", 0), ("dam2d", 1), ("granular", 0), ("granular", 1)])
def test_idle_hooks_change_nothing(gpu, name, precision):
    """Hooks that download and patch the particles unchanged: the split step
    and the round trip through the host are exact."""
    dom, dt, _ = CASES[name][0]()
    cfg = dom.config(dt)
    cfg.precision = precision
    ref = GpuDomain(cfg)
    ref.upload(dom.particles, initial=True)
    ref.step(12)
    gd = GpuDomain(cfg)
    calls = []
    gd.set_step_hooks(before=lambda t, p: calls.append(("before", t)), after=lambda t, p: calls.append(("after", t)))
    gd.upload(dom.particles, initial=True)
    gd.step(12)
    assert len(calls) == 24 and calls[0][0] == "before" and calls[1][0] == "after"
    assert calls[0][1] == calls[1][1] == 0.0
    a = ref.download_fields(("x", "v", "density", "pressure", "a"))
    b = gd.download_fields(("x", "v", "density", "pressure", "a"))
    for f in a:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    assert gd.time == ref.time


def test_before_hook_sees_start_acceleration(gpu):
    """At GeneralBefore the accelerations are Gravity and the density rates
    zero, as StartAcceleration leaves them."""
    dom, dt, _ = CASES["dam2d"][0]()
    cfg = dom.config(dt)
    gd = GpuDomain(cfg)
    seen = {}

    def before(t, p):
        seen["a"] = p.get("a").copy()
        seen["dd"] = p.get("ddensity").copy()

    gd.set_step_hooks(before=before)
    gd.upload(dom.particles, initial=True)
    gd.step(3)
    g = np.array(list(cfg.gravity))
    assert np.all(seen["a"] == g[None, :]) and np.all(seen["dd"] == 0.0)


def test_patch_refusals(gpu):
    # a new h where h is uniform: the kernels take 1/h from the launch
    dom, dt, _ = CASES["dam2d"][0]()
    gd = GpuDomain(dom.config(dt))

    def grow_h(t, p):
        h = p.get("h")
        h[0] *= 1.1
        p.set("h", h)

    gd.set_step_hooks(after=grow_h)
    gd.upload(dom.particles, initial=True)
    with pytest.raises(PsphError) as e:
        gd.step(1)
    assert e.value.code == 2 and "uniform" in str(e.value)
    # accelerations changed at GeneralBefore in the FP32C form
    cfg = dom.config(dt)
    cfg.precision = 1
    g32 = GpuDomain(cfg)
    g32.set_step_hooks(before=lambda t, p: p.set("a", p.get("a") + 1.0))
    g32.upload(dom.particles, initial=True)
    with pytest.raises(PsphError) as e:
        g32.step(1)
    assert e.value.code == 2 and "FP32C" in str(e.value)


def test_hook_exception_stops_the_step(gpu):
    dom, dt, _ = CASES["dam2d"][0]()
    gd = GpuDomain(dom.config(dt))

    def boom(t, p):
        raise RuntimeError("hook failed")

    gd.set_step_hooks(after=boom)
    gd.upload(dom.particles, initial=True)
    with pytest.raises(RuntimeError, match="hook failed"):
        gd.step(2)


def test_damping_hook_changes_parameters(gpu):
    """The granular_damped hook's new cohesion and friction angle reach the
    device (downloaded back) once its switch time has passed."""
    dom, dt, info = CASES["granular_damped"][0]()
    gd = GpuDomain(dom.config(dt))
    gd.use_step_hooks(dom)
    gd.upload(dom.particles, initial=True)
    for _ in range(100):  # past the switch time (the adaptive step may shrink)
        gd.step(1)
        if gd.time > info["damping"][3] + dt:
            break
    st = gd.download_fields(("id", "cohesion", "phi"))
    up = st["id"] == 6
    assert up.any()
    assert np.all(st["cohesion"][up] == info["damping"][5]) and np.all(st["phi"][up] == info["damping"][6])
    assert np.all(st["cohesion"][(st["id"] == 1)] == 1000.0)
