"""GPU parity against the oracle and the reference's golden outputs, through
the C ABI (persiansph_gb300.solver.GpuDomain -> libpsph_gb300.so).

Tolerances (FP64 form): per-step accelerations and density rates <= 1e-12
relative to the magnitude of the per-particle sums (the oracle's scales);
pair sets bit-exact; multi-step trajectories against the reference within
1e-9 (summation order differs, so rounding differences grow slowly).
"""
import os

import numpy as np
import pytest

from oracle.oracle import OracleDomain
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES
from tests.gpu_helpers import assert_step_parity, continue_on_gpu

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def as_set(pairs):
    return set(map(tuple, np.asarray(pairs).tolist()))


@pytest.mark.parametrize("name", sorted(CASES))
def test_candidate_pairs_bit_exact(gpu, name):
    builder, _, _ = CASES[name]
    dom, dt, _ = builder()
    g = golden(name)
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    ref = as_set(np.concatenate([g["pairs_sm"], g["pairs_fsm"], g["pairs_nsm"]]))
    got = gd.pairs(0)
    assert len(got) == len(ref)
    assert as_set(got) == ref  # same unordered pairs, in the reference's (first, second) orientation


@pytest.mark.parametrize("name", sorted(CASES))
def test_support_pairs_bit_exact(gpu, name):
    builder, _, _ = CASES[name]
    dom, dt, _ = builder()
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    o.step(2)
    gd = continue_on_gpu(dom.config(dt), o)
    assert as_set(gd.pairs(1)) == as_set(o.pairs(3))


@pytest.mark.parametrize("name", sorted(CASES))
def test_single_step_parity_1e12(gpu, name):
    builder, _, dumps = CASES[name]
    dom, dt, _ = builder()
    cfg = dom.config(dt)
    # from the initial state (Solve's set-up) and from a developed state
    for warm in (0, 3):
        o = OracleDomain(cfg, dom.particles, initial=True)
        if warm:
            o.step(warm)
        gd = continue_on_gpu(cfg, o) if warm else None
        if gd is None:
            gd = GpuDomain(cfg)
            gd.upload(dom.particles, initial=True)
        o.step(1)
        gd.step(1)
        a_scale, dr_scale = o.scales()
        assert gd.n == o.n
        assert_step_parity(gd.download_fields(), o.download(), a_scale, dr_scale, dt,
                           label=f"{name} after {warm}+1 steps")


@pytest.mark.parametrize("name", sorted(CASES))
def test_trajectory_matches_reference(gpu, name):
    builder, nsteps, dumps = CASES[name]
    dom, dt, _ = builder()
    g = golden(name)
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    prev = 0
    for k in dumps:
        gd.step(k - prev)
        prev = k
        assert gd.n == int(g[f"n_{k}"])
        st = gd.download_fields()
        it = gd.integrator()
        assert it.time == pytest.approx(float(g[f"time_{k}"]), rel=1e-9)
        t = float(g[f"time_{k}"])
        amax = np.max(np.abs(g[f"a_{k}"]))
        cs = dom.particles.get("cs").max()
        scales = {
            "x": np.max(np.abs(g[f"x_{k}"])),
            # a velocity near zero (the leapfrog start) is judged against what t*|a| could build up
            "v": np.max(np.abs(g[f"v_{k}"])) + t * amax,
            "density": np.max(np.abs(g[f"density_{k}"])),
            "pressure": np.max(np.abs(g[f"pressure_{k}"])) + 1e-6 * cs * cs * np.max(g[f"density_{k}"]),
        }
        for f, scale in scales.items():
            ref = g[f"{f}_{k}"]
            err = np.max(np.abs(st[f].reshape(ref.shape) - ref)) / scale
            assert err <= 1e-9, f"{name} step {k} {f}: {err:.3e}"


def test_deterministic_runs(gpu):
    dom, dt, _ = CASES["dam2d"][0]()
    outs = []
    for _ in range(2):
        gd = GpuDomain(dom.config(dt))
        gd.upload(dom.particles, initial=True)
        gd.step(45)
        outs.append(gd.download_fields(("x", "v", "a", "density")))
    for f in outs[0]:
        np.testing.assert_array_equal(outs[0][f], outs[1][f])


def test_step_stops_at_t_stop(gpu):
    dom, dt, _ = CASES["poiseuille"][0]()
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    done = gd.step(1000, t_stop=5.5 * dt)
    assert done == 6  # Solve's loop runs while Time < tf
    assert gd.time == pytest.approx(6 * dt)


FLUID_CASES = ["dam2d", "dam2d_leapfrog", "poiseuille", "dam3d", "fluid_options", "fluid_shao_bingham",
               "fluid_incomp_quintic"]


@pytest.mark.parametrize("name", FLUID_CASES)
def test_fp32c_single_step_parity_1e5(gpu, name):
    """FP32C form: accelerations and density rates within 1e-5 of the FP64
    oracle, relative to each particle's sum of term magnitudes."""
    builder, _, _ = CASES[name]
    dom, dt, _ = builder()
    cfg = dom.config(dt)
    cfg32 = dom.config(dt)
    cfg32.precision = 1  # PSPH_FP32C
    for warm in (0, 3):
        o = OracleDomain(cfg, dom.particles, initial=True)
        if warm:
            o.step(warm)
            gd = continue_on_gpu(cfg32, o)
        else:
            gd = GpuDomain(cfg32)
            gd.upload(dom.particles, initial=True)
        o.step(1)
        gd.step(1)
        a_scale, dr_scale = o.scales()
        g, r = gd.download_fields(), o.download()
        free = r["is_free"] == 1
        ea = np.max(np.linalg.norm(g["a"] - r["a"], axis=1)[free] / a_scale[free])
        ed = np.max(np.abs(g["ddensity"] - r["ddensity"])[free] / (dr_scale[free] + 1e-30))
        assert ea <= 1e-5, f"{name} {warm}: FP32C acceleration rel err {ea:.3e}"
        assert ed <= 1e-5, f"{name} {warm}: FP32C density-rate rel err {ed:.3e}"


def test_fp32c_rejects_solids(gpu):
    dom, dt, _ = CASES["granular"][0]()
    cfg = dom.config(dt)
    cfg.precision = 1
    gd = GpuDomain(cfg)
    with pytest.raises(Exception, match="UNSUPPORTED"):
        gd.upload(dom.particles, initial=True)
