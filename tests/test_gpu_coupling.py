"""Domains of two materials on the GPU: fluid with soil (CalcForce13, the
saturation switch, VarPorosity) and fluid with an elastic solid (CalcForce12,
the FSI interpolation). The seepage state against the reference's golden
trajectories, and the combinations this build rejects. Per-step parity against
the oracle and the trajectories of x, v, density and pressure run with every
other case in test_gpu_parity.py (the seep_* and gate_* cases are part of its
case table)."""
import os

import numpy as np
import pytest

from persiansph_gb300 import scenarios
from persiansph_gb300.abi import PsphError
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SEEP = sorted(k for k in CASES if k.startswith("seep_"))


@pytest.mark.parametrize("name", SEEP)
def test_seepage_state_matches_reference(gpu, name):
    """Saturation flags exactly, masses and RefDensity to rounding, S and the
    strain (which VarPorosity turns into permeability) within 1e-9 of their
    largest value, at every stored step of the reference run."""
    builder, _, dumps = CASES[name]
    dom, dt, _ = builder()
    g = dict(np.load(os.path.join(GOLD, name + ".npz")))
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    prev = 0
    for k in dumps:
        gd.step(k - prev)
        prev = k
        st = gd.download_fields()
        assert np.array_equal(st["is_sat"], g[f"is_sat_{k}"]), f"{name} step {k}: saturation state"
        for f in ("mass", "ref_density"):
            err = np.max(np.abs(st[f] - g[f"{f}_{k}"]) / np.abs(g[f"{f}_{k}"]))
            assert err <= 1e-14, f"{name} step {k} {f}: {err:.3e}"
        for f in ("s", "strain"):
            ref = g[f"{f}_{k}"]
            scale = np.max(np.abs(ref))
            if scale > 0.0:
                err = np.max(np.abs(st[f].reshape(ref.shape) - ref)) / scale
                assert err <= 1e-9, f"{name} step {k} {f}: {err:.3e}"


def _rejected(dom, dt, **cfg_changes):
    cfg = dom.config(dt)
    for k, v in cfg_changes.items():
        setattr(cfg, k, v)
    gd = GpuDomain(cfg)
    with pytest.raises(PsphError) as e:
        gd.upload(dom.particles, initial=True)
    return e.value


def test_two_materials_need_fp64(gpu):
    for dom, dt, _ in (scenarios.seepage_bed_2d(), scenarios.elastic_gate_2d()):
        err = _rejected(dom, dt, precision=1)
        assert err.code == 2 and "FP64" in str(err)


def test_solid_with_soil_is_rejected(gpu):
    """The reference has no pair force between a solid (Material 2) and a soil
    (LastComputeAcceleration aborts on such a pair)."""
    dom, dt, _ = scenarios.seepage_bed_2d()
    p = dom.particles
    p.get("material")[p.get("material") == 1] = 2
    err = _rejected(dom, dt)
    assert err.code == 2 and "no pair force" in str(err)


def test_seepage_type_out_of_range(gpu):
    dom, dt, _ = scenarios.seepage_bed_2d()
    p = dom.particles
    p.get("seepage_type")[p.get("material") == 3] = 4
    err = _rejected(dom, dt)
    assert err.code == 1 and "Seepage Type" in str(err)
