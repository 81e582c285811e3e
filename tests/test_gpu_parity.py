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
    if dom.config(dt).in_out_flow:
        pytest.skip("an in/out-flow boundary's lists are not part of an upload (its trajectory test covers it)")
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    o.step(2)
    gd = continue_on_gpu(dom.config(dt), o)
    assert as_set(gd.pairs(1)) == as_set(o.pairs(3))


@pytest.mark.parametrize("name", sorted(CASES))
def test_single_step_parity_1e12(gpu, name):
    builder, _, dumps = CASES[name]
    dom, dt, _ = builder()
    cfg = dom.config(dt)
    # from the initial state (Solve's set-up) and from a developed state (an
    # in/out-flow boundary's lists are not part of an upload: initial state only)
    for warm in ((0,) if cfg.in_out_flow else (0, 3)):
        o = OracleDomain(cfg, dom.particles, initial=True)
        o.use_flow_hooks(dom)
        o.use_step_hooks(dom)  # GeneralBefore / GeneralAfter of the case, if any
        if warm:
            o.step(warm)
        gd = continue_on_gpu(cfg, o) if warm else None
        if gd is None:
            gd = GpuDomain(cfg)
            gd.use_flow_hooks(dom)
            gd.upload(dom.particles, initial=True)
        gd.use_step_hooks(dom)
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
    gd.use_flow_hooks(dom)
    gd.use_step_hooks(dom)
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
               "fluid_incomp_quintic", "fluid_preseq2"]


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
        # the step's pressure (the FP32C update's EOS, from the FP64 density),
        # relative to the largest pressure (absolute when every pressure is 0)
        dp = np.max(np.abs(g["pressure"] - r["pressure"])[free])
        pmax = np.max(np.abs(r["pressure"][free]))
        ep = dp / pmax if pmax > 0.0 else dp
        assert ep <= 1e-5, f"{name} {warm}: FP32C pressure rel err {ep:.3e}"


SOLID_CASES = ["granular", "granular_lf_fail3", "solid_block", "soil3d_ti"]


@pytest.mark.parametrize("name", SOLID_CASES)
def test_fp32c_solid_single_step_parity_1e5(gpu, name):
    """FP32C form of the soil / solid pair force (CalcForce2233) against the
    FP64 oracle. Accelerations: within 1e-5 of each particle's sum of term
    magnitudes. Density rates: the same per-particle bound for particles
    whose term sum is at least 1e-6 of the largest, and 1e-5 of the term sums
    norm-wise over all free particles. (Below that, a particle and its neighbours move as one
    body: their velocity differences are a few ulps of the velocities, and the
    oracle's density rate is the rounding noise of its FP64 velocities, which
    48-bit FP32 velocity pairs cannot resolve.) Strain and rotation rates
    within 1e-5 of the largest oracle rate; the FP64 stress update that
    follows keeps the step's stresses within 1e-5 of the largest stress."""
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
        assert ea <= 1e-5, f"{name} {warm}: FP32C acceleration rel err {ea:.3e}"
        resolved = free & (dr_scale > 0.0) & (dr_scale >= 1e-6 * np.max(dr_scale[free]))
        if resolved.any():
            ed = np.max(np.abs(g["ddensity"] - r["ddensity"])[resolved] / dr_scale[resolved])
            assert ed <= 1e-5, f"{name} {warm}: FP32C density-rate rel err {ed:.3e}"
        dn = np.linalg.norm((g["ddensity"] - r["ddensity"])[free]) / (np.linalg.norm(dr_scale[free]) + 1e-300)
        assert dn <= 1e-5, f"{name} {warm}: FP32C density-rate norm-wise rel err {dn:.3e}"
        for f in ("strain_rate", "rotation_rate", "sigma"):
            ref = np.max(np.abs(r[f][free]))
            if ref > 0:
                e = np.max(np.abs(g[f][free] - r[f][free])) / ref
                assert e <= 1e-5, f"{name} {warm}: FP32C {f} rel err {e:.3e}"


@pytest.mark.parametrize("precision", [0, 1])
def test_launch_tuning_does_not_change_results(gpu, precision):
    """The block size of the pair kernels and the staging depth of the
    neighbour search are launch choices only: states are bit-identical (the
    staged scan reads the same candidates in the same order from shared
    memory). The x-slab split of the cells reorders each particle's
    neighbours, so only the rounding of the sums changes: after 4 steps every
    field agrees within 1e-12 (FP64) / 1e-5 (FP32C) of its largest magnitude.
    psph_autotune returns one of the candidate settings."""
    dom, dt, _ = CASES["dam3d"][0]()
    cfg = dom.config(dt)
    cfg.precision = precision
    states = {}
    for block, split, stage in [(128, 1, 0), (64, 1, 0), (128, 1, 3072), (128, 1, 2048), (256, 2, 0),
                                (128, 4, 4096), (128, 4, 0)]:
        gd = GpuDomain(cfg)
        gd.upload(dom.particles, initial=True)
        gd.set_tuning(block, split, stage)
        gd.step(4)
        states[(block, split, stage)] = gd.download_fields(("x", "v", "density", "a", "ddensity"))
        gd.close()
    ref = states[(128, 1, 0)]
    for f in ref:
        np.testing.assert_array_equal(states[(64, 1, 0)][f], ref[f])
        np.testing.assert_array_equal(states[(128, 1, 3072)][f], ref[f])
        np.testing.assert_array_equal(states[(128, 1, 2048)][f], ref[f])
        np.testing.assert_array_equal(states[(128, 4, 4096)][f], states[(128, 4, 0)][f])
    tol = 1e-12 if precision == 0 else 1e-5
    for key in [(256, 2, 0), (128, 4, 0)]:
        for f in ref:
            scale = np.max(np.abs(ref[f])) + 1e-300
            err = np.max(np.abs(states[key][f] - ref[f])) / scale
            assert err <= tol, f"split {key}: {f} differs by {err:.2e} of its scale"
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    t = gd.autotune(2)
    assert t["pair_block"] in (64, 128, 256) and t["cell_split"] in (1, 2, 4) and t["ms_per_step"] > 0
    assert t["nlist_stage"] in (0, 2048, 3072, 4096)
    assert gd.tuning()["pair_block"] == t["pair_block"] and gd.tuning()["cell_split"] == t["cell_split"]
    gd.close()


def test_autotune_cache(gpu, tmp_path):
    """A tuning result stored for a workload signature is reused without
    trials by a context of the same workload."""
    dom, dt, _ = CASES["dam3d"][0]()
    cfg = dom.config(dt)
    cfg.precision = 1
    cache = str(tmp_path / "tuning.json")
    first = GpuDomain(cfg)
    first.upload(dom.particles, initial=True)
    t1 = first.autotune(2, cache=cache)
    first.close()
    second = GpuDomain(cfg)
    second.upload(dom.particles, initial=True)
    t2 = second.autotune(2, cache=cache)
    assert t2.get("cached") and t2["pair_block"] == t1["pair_block"] and t2["cell_split"] == t1["cell_split"]
    assert second.tuning()["pair_block"] == t1["pair_block"]
    assert second.integrator().steps == 0  # no trial steps were run
    second.close()
