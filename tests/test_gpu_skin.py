"""Neighbour lists with a skin (psph_tuning.skin_permille, FP32C form): the
cell sort and the lists run only when a particle has moved half the skin, on
cells at least (1 + skin) of the support wide. Every step must still evaluate
exactly the pairs inside the support, in the reference's wall-pressure
orientation: a step taken on kept lists matches the FP64 oracle continuing
from the same state within the FP32C bound (1e-5 of each particle's sum of
term magnitudes), whether or not the lists were rebuilt for it."""
import numpy as np
import pytest

from oracle.oracle import OracleDomain
from persiansph_gb300.abi import PsphError
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu


def _fp32c(name):
    dom, dt, _ = CASES[name][0]()
    cfg = dom.config(dt)
    cfg32 = dom.config(dt)
    cfg32.precision = 1
    return dom, dt, cfg, cfg32


@pytest.mark.parametrize("name,warm,skin", [("dam2d", 400, 100), ("dam3d", 150, 50), ("granular", 60, 100)])
def test_kept_lists_match_the_oracle(gpu, name, warm, skin):
    dom, dt, cfg, cfg32 = _fp32c(name)
    gd = GpuDomain(cfg32)
    gd.upload(dom.particles, initial=True)
    gd.step(warm)  # a developed flow, lists every step
    gd.set_tuning(128, 1, 0, skin)
    kept = rebuilt = 0
    for _ in range(40):
        st = gd.download()
        o = OracleDomain(cfg, st, initial=False, grid=gd.grid(), integ=gd.integrator())
        rb0 = gd.list_rebuilds()
        o.step(1)
        gd.step(1)
        if gd.list_rebuilds() == rb0:
            kept += 1
        else:
            rebuilt += 1
        a_scale, dr_scale = o.scales()
        g, r = gd.download_fields(("a", "ddensity", "is_free")), o.download()
        free = r["is_free"] == 1
        ea = np.max(np.linalg.norm(g["a"] - r["a"], axis=1)[free] / a_scale[free])
        ed = np.max(np.abs(g["ddensity"] - r["ddensity"])[free] / (dr_scale[free] + 1e-30))
        assert ea <= 1e-5 and ed <= 1e-5, f"{name}: rel err a {ea:.3e}, drho {ed:.3e} (rebuilds {gd.list_rebuilds()})"
        o.close()
    assert rebuilt >= 1 and kept >= 10, (kept, rebuilt)


def test_skin_saves_rebuilds_and_keeps_the_pair_count(gpu):
    """The same 60 steps with and without a skin from the same developed
    state: far fewer rebuilds, and the same pair-interactions per step within
    the pairs at the support's edge that FP32 rounding can flip."""
    dom, dt, cfg, cfg32 = _fp32c("dam3d")
    a = GpuDomain(cfg32)
    a.upload(dom.particles, initial=True)
    a.step(150)
    st = a.download()
    b = GpuDomain(cfg32, grid=a.grid(), integ=a.integrator())
    b.upload(st, initial=False)
    b.set_tuning(128, 1, 0, 100)
    r0a, r0b = a.list_rebuilds(), b.list_rebuilds()
    pa0, pb0 = a.pair_count(), b.pair_count()
    a.step(60)
    b.step(60)
    assert a.list_rebuilds() - r0a == 60
    assert b.list_rebuilds() - r0b < 20
    pa, pb = a.pair_count() - pa0, b.pair_count() - pb0
    assert abs(pa - pb) <= 1e-5 * pa, (pa, pb)
    xa, xb = a.download_fields(("x",))["x"], b.download_fields(("x",))["x"]
    assert np.max(np.abs(xa - xb)) <= 1e-6 * np.max(np.abs(xa))


def test_exports_keep_the_reference_cells(gpu):
    """Pair exports of a context with a skin list the reference's candidate
    and in-support pairs; the next steps still match a context without one."""
    dom, dt, cfg, cfg32 = _fp32c("dam2d")
    a = GpuDomain(cfg32)
    a.upload(dom.particles, initial=True)
    a.step(50)
    st = a.download()
    b = GpuDomain(cfg32, grid=a.grid(), integ=a.integrator())
    b.upload(st, initial=False)
    b.set_tuning(128, 1, 0, 100)
    b.step(5)
    a.step(5)
    for which in (0, 1):
        pa = set(map(tuple, a.pairs(which).tolist()))
        pb = set(map(tuple, b.pairs(which).tolist()))
        # the states differ only by FP32 summation order: compare as sets of
        # nearly all pairs
        assert len(pa ^ pb) <= 1e-4 * len(pa) + 2, (which, len(pa), len(pb), len(pa ^ pb))
    a.step(5)
    b.step(5)
    ga, gb = a.download_fields(("a",))["a"], b.download_fields(("a",))["a"]
    assert np.max(np.abs(ga - gb)) <= 1e-4 * np.max(np.abs(ga))


def test_skin_refusals(gpu):
    dom, dt, cfg, cfg32 = _fp32c("dam2d")
    g64 = GpuDomain(cfg)
    g64.upload(dom.particles, initial=True)
    with pytest.raises(PsphError) as e:
        g64.set_tuning(128, 1, 0, 100)
    assert e.value.code == 2 and "FP32C" in str(e.value)
    g32 = GpuDomain(cfg32)
    g32.upload(dom.particles, initial=True)
    with pytest.raises(PsphError) as e:
        g32.set_tuning(128, 1, 0, 400)
    assert e.value.code == 1
    pdom, pdt, _ = CASES["poiseuille"][0]()  # periodic in x
    pc = pdom.config(pdt)
    pc.precision = 1
    gp = GpuDomain(pc)
    gp.upload(pdom.particles, initial=True)
    with pytest.raises(PsphError) as e:
        gp.set_tuning(128, 1, 0, 100)
    assert e.value.code == 2 and "periodic" in str(e.value)
