"""Long-run accuracy on the GPU (both arithmetic forms):
 - 2D Poiseuille flow reaches the analytic parabola u(y) = g/(2 nu) (H^2/4 - y^2)
   within 0.5 % (L2 over fluid particles);
 - the 2D dam-break surge front follows the reference's own run (golden fixture
   tests/golden/surge2d.npz from the unmodified reference) within 1 %.
"""
import os

import numpy as np
import pytest

from persiansph_gb300 import scenarios
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import SURGE_STEPS, surge2d, surge_front

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("precision", [0, 1])
def test_poiseuille_reaches_analytic_profile(gpu, precision):
    dom, dt, info = scenarios.poiseuille()
    cfg = dom.config(dt)
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    gd.step(12000)  # t ~ 1.6 s, about 1.6 viscous times H^2/nu
    st = gd.download_fields(("x", "v", "is_free"))
    free = st["is_free"] == 1
    y, u = st["x"][free, 1], st["v"][free, 0]
    ue = info["gx"] / (2 * info["nu"]) * (info["H"] ** 2 / 4 - y ** 2)
    err = np.linalg.norm(u - ue) / np.linalg.norm(ue)
    assert err <= 0.005, f"L2 error {err:.4f} against the analytic Poiseuille profile"


@pytest.mark.parametrize("precision,skin", [(0, 0), (1, 0), (1, 100)])
def test_surge_front_follows_reference(gpu, precision, skin):
    """The surge front of a 2D dam break within 1 % of the reference's; the
    FP32C form also with neighbour lists kept under a 10 % skin."""
    g = dict(np.load(os.path.join(GOLD, "surge2d.npz")))
    dom, dt, _ = surge2d()
    cfg = dom.config(dt)
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    if skin:
        gd.set_tuning(128, 1, 0, skin)
    times, fronts, prev = [], [], 0
    for k in SURGE_STEPS:
        gd.step(k - prev)
        prev = k
        st = gd.download_fields(("x", "is_free"))
        times.append(gd.time)
        fronts.append(surge_front(st["x"], st["is_free"]))
    ours = np.interp(g["time"], times, fronts)
    rel = np.abs(ours - g["front"]) / g["front"]
    assert rel.max() <= 0.01, f"surge front differs from the reference by {rel.max():.4f}"
    if skin:  # the lists were kept on most steps
        assert gd.list_rebuilds() < SURGE_STEPS[-1] // 2
