"""Parity at the benchmark configurations' own sizes, through the C ABI.

The golden cases (test_gpu_parity.py) are small versions of the benchmark
configurations. Here the configurations themselves run, where cell counts,
wall layers, ghost columns and clamping differ from the small cases:

- 2D dam break at dx = 5 mm (86,018 particles, cubic spline, Tait, AV);
- 3D dam break at dx = 20 mm with LES (177,156 particles; Wendland C2), the
  learned closure's configuration, with the closure features checked;
- a sample of the 3D dam break at dx = 10 mm (1,021,104 particles; the
  headline configuration's tank and options at twice its spacing);
- the largest column of the batched granular workload: aspect 4 at
  dx = 1 mm (159,600 soil particles, Drucker-Prager Fail 2, TI on).

Each checks against the oracle (the CPU restatement pinned to the reference):
the candidate pair set (MainNeighbourSearch's SMPairs + FSMPairs + NSMPairs,
Source/Domain.cpp:808-945) and the in-support pair set bit-exact (same
unordered pairs, same orientation), then one step of the FP64 form at
1e-12 and of the FP32C form at 1e-5 of each particle's sum of term
magnitudes, from the initial state (Solve's set-up) and from a developed
state. The developed state is made by the GPU FP64 form (hundreds of steps
the oracle would take minutes for) and handed to both sides as host arrays:
from then on the oracle and the GPU start from the same numbers.
"""
import os

import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle.oracle import OracleDomain
from persiansph_gb300 import scenarios
from persiansph_gb300.closure import ClosureNet, default_network_path, les_case
from persiansph_gb300.solver import GpuDomain
from tests.gpu_helpers import assert_step_parity

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def c2_dam2d():
    return scenarios.dam_break_2d(dx=5e-3)


def c5_dam3d_les():
    return les_case(0.02, L=1.2, H=0.55, W=1.0, TL=3.22, TH=1.0, TW=1.0, c0=40.0)


def c3_dam3d_10mm():
    return scenarios.dam_break_3d(dx=0.01)


def c4_granular_tallest():
    return scenarios.granular_column(dx=1e-3, W=0.2, aspect=4.0, phi_deg=30.0)


# name: (builder, particles expected, GPU FP64 steps to the developed state,
#        candidate pair set checked (the 1M sample's ~240M candidates are not))
CONFIGS = {
    "c2_dam2d_5mm": (c2_dam2d, 86018, 2000, True),
    "c5_dam3d_20mm_les": (c5_dam3d_les, 177156, 600, True),
    "c3_dam3d_10mm": (c3_dam3d_10mm, 1021104, 300, False),
    "c4_granular_aspect4": (c4_granular_tallest, None, 1000, True),
}


def pair_keys(pairs):
    """Ordered pairs (first, second) of original indices as sorted int64 keys."""
    p = np.asarray(pairs, np.int64).reshape(-1, 2)
    return np.sort(p[:, 0] << 32 | p[:, 1])


def developed(cfg, pset, steps):
    """The state after `steps` GPU FP64 steps from the initial state, as host
    arrays with the grid and integrator, for both sides to start from."""
    gd = GpuDomain(cfg)
    gd.upload(pset, initial=True)
    assert gd.step(steps) == steps
    state = gd.download(base=pset)
    grid, integ = gd.grid(), gd.integrator()
    gd.close()
    return state, grid, integ


def gpu_from(cfg, state, grid, integ, precision):
    c = type(cfg).from_buffer_copy(cfg)
    c.precision = precision
    gd = GpuDomain(c, grid=grid, integ=integ)
    gd.upload(state, initial=False)
    return gd


def check_fp32c(g, r, a_scale, dr_scale, label, solid):
    free = r["is_free"] == 1
    ea = np.max(np.linalg.norm(g["a"] - r["a"], axis=1)[free] / a_scale[free])
    assert ea <= 1e-5, f"{label}: FP32C acceleration rel err {ea:.3e}"
    if solid:  # rates resolved above 1e-6 of the largest term sum, and norm-wise
        res = free & (dr_scale > 0.0) & (dr_scale >= 1e-6 * np.max(dr_scale[free]))
        ed = np.max(np.abs(g["ddensity"] - r["ddensity"])[res] / dr_scale[res]) if res.any() else 0.0
        dn = np.linalg.norm((g["ddensity"] - r["ddensity"])[free]) / (np.linalg.norm(dr_scale[free]) + 1e-300)
        assert dn <= 1e-5, f"{label}: FP32C density-rate norm-wise rel err {dn:.3e}"
    else:
        ed = np.max(np.abs(g["ddensity"] - r["ddensity"])[free] / (dr_scale[free] + 1e-30))
    assert ed <= 1e-5, f"{label}: FP32C density-rate rel err {ed:.3e}"
    return ea, ed


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_config_size_pairs_and_steps(gpu, name):
    builder, n_expect, warm_steps, candidates = CONFIGS[name]
    dom, dt, _ = builder()
    p = dom.particles
    if n_expect is not None:
        assert p.n == n_expect
    cfg = dom.config(dt)
    solid = bool(np.any(p.get("material") >= 2))

    # initial state: pair sets of Solve's set-up, then one step of each form
    o = OracleDomain(cfg, p, initial=True)
    g64 = GpuDomain(cfg)
    g64.upload(p, initial=True)
    if candidates:  # the oracle's lists 0-2 are SMPairs, FSMPairs, NSMPairs; 4 = all three
        np.testing.assert_array_equal(pair_keys(g64.pairs(0)), pair_keys(o.pairs(4)),
                                      err_msg=f"{name}: candidate pairs")
    np.testing.assert_array_equal(pair_keys(g64.pairs(1)), pair_keys(o.pairs(3)), err_msg=f"{name}: support pairs")
    c32 = type(cfg).from_buffer_copy(cfg)
    c32.precision = 1
    g32 = GpuDomain(c32)
    g32.upload(p, initial=True)
    o.step(1, NT)
    g64.step(1)
    g32.step(1)
    a_scale, dr_scale = o.scales()
    r = o.download()
    assert_step_parity(g64.download_fields(), r, a_scale, dr_scale, dt, label=f"{name} FP64 first step")
    check_fp32c(g32.download_fields(), r, a_scale, dr_scale, f"{name} first step", solid)
    g64.close()
    g32.close()
    o.close()

    # developed state
    state, grid, integ = developed(cfg, p, warm_steps)
    o = OracleDomain(cfg, state, initial=False, grid=grid, integ=integ)
    g64 = gpu_from(cfg, state, grid, integ, 0)
    np.testing.assert_array_equal(pair_keys(g64.pairs(1)), pair_keys(o.pairs(3)),
                                  err_msg=f"{name}: support pairs, developed state")
    g32 = gpu_from(cfg, state, grid, integ, 1)
    o.step(1, NT)
    g64.step(1)
    g32.step(1)
    a_scale, dr_scale = o.scales()
    r = o.download()
    assert np.max(np.abs(r["v"])) > 0.0
    assert_step_parity(g64.download_fields(), r, a_scale, dr_scale, dt,
                       label=f"{name} FP64 step after {warm_steps}")
    check_fp32c(g32.download_fields(), r, a_scale, dr_scale, f"{name} step after {warm_steps}", solid)


def test_c5_closure_features_at_config_size(gpu):
    """The learned closure's configuration (3D dam break, dx = 20 mm, LES):
    from a developed state, the FP32C step's closure features (shear rate,
    strain-rate invariant ratio, density ratio, h/dx, neighbour count) against
    the oracle's FP64 strain-rate sums and in-support pair list."""
    dx = 0.02
    dom, dt, _ = c5_dam3d_les()
    cfg = dom.config(dt)
    state, grid, integ = developed(cfg, dom.particles, 600)
    o = OracleDomain(cfg, state, initial=False, grid=grid, integ=integ)
    rho_before = o.download()["density"].copy()
    cnt = np.bincount(o.pairs(3).ravel(), minlength=o.n)
    g32 = gpu_from(cfg, state, grid, integ, 1)
    g32.attach_closure(ClosureNet.load(default_network_path()), dx)
    o.step(1, NT)
    g32.step(1)
    ro = o.download()
    feats = g32.closure_features()
    free = ro["is_free"] == 1
    vort = np.exp(feats[:, 2].astype(np.float64)) * ro["cs"] / ro["h"]
    f_o, shear = mo.features(ro["strain_rate"], vort, rho_before, ro["ref_density"], ro["h"], dx, cnt, ro["cs"])
    # the shear rate from the FP32C sums within 1e-5 of the largest (where the
    # log feature is resolved: rates above 1e-3 of the largest)
    sr_g = np.exp(feats[:, 0].astype(np.float64)) * ro["cs"] / ro["h"]
    smax = np.max(shear[free])
    assert smax > 0.0
    big = free & (shear > 1e-3 * smax)
    assert np.max(np.abs(sr_g[big] - shear[big])) <= 1e-5 * smax
    assert np.max(np.abs(feats[big, 1] - f_o[big, 1])) <= 1e-3
    assert np.max(np.abs(feats[free, 3] - f_o[free, 3])) <= 1e-6
    np.testing.assert_array_equal(feats[free, 4], (ro["h"][free] / dx).astype(np.float32))
    diff = np.abs(feats[free, 5] - cnt[free])
    assert diff.max() <= 1 and np.mean(diff > 0) <= 1e-4  # a pair at the support edge may differ in FP32
    ev, fb = g32.closure_stats()
    assert ev == int(free.sum())
