"""Failure detection through the C ABI, with the failure made on the host
(bad inputs), never by faulting the GPU: each condition the reference turns
into a `Fatal` (or a removal) comes back as a status code, and the context
(or a fresh one) stays usable afterwards."""
import numpy as np
import pytest

from persiansph_gb300.abi import PsphError
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu

PSPH_ERR_NONFINITE, PSPH_ERR_DT_COLLAPSE, PSPH_ERR_CFL = 5, 6, 7


def dam2d(precision=0):
    dom, dt, _ = CASES["dam2d"][0]()
    cfg = dom.config(dt)
    cfg.precision = precision
    return dom, dt, cfg


def test_cfl_violation_is_reported_on_upload(gpu):
    """TimestepCheck (Source/Domain.cpp:1721-1733): a user dt above 0.25 h / c
    is refused before any step."""
    dom, dt, _ = dam2d()
    cfg = dom.config(100.0 * dt)
    gd = GpuDomain(cfg)
    with pytest.raises(PsphError) as e:
        gd.upload(dom.particles, initial=True)
    assert e.value.code == PSPH_ERR_CFL


@pytest.mark.parametrize("precision", [0, 1])
def test_nonfinite_state_is_reported_and_context_survives(gpu, precision):
    """A NaN density (a corrupted input) makes the step return
    PSPH_ERR_NONFINITE; the context still answers and a fresh one steps."""
    dom, dt, cfg = dam2d(precision)
    p = dom.particles.copy()
    rho = p.get("density")
    free = np.flatnonzero(p.get("is_free") == 1)
    rho[free[len(free) // 2]] = np.nan
    gd = GpuDomain(cfg)
    gd.upload(p, initial=False)
    with pytest.raises(PsphError) as e:
        gd.step(3)
    assert e.value.code == PSPH_ERR_NONFINITE
    assert gd.download_fields(("x",))["x"].shape[0] == gd.n  # the context still answers
    gd.close()
    ok = GpuDomain(cfg)
    ok.upload(dom.particles, initial=True)
    assert ok.step(3) == 3
    assert np.all(np.isfinite(ok.download_fields(("a",))["a"]))


def test_dt_collapse_is_reported(gpu):
    """AdaptiveTimeStep's 'Too small time step' (Source/Domain.cpp:150-151):
    an acceleration bound far below the user dt collapses dt."""
    dom, dt, _ = dam2d()
    dom.sqrt_h_a = 1e-12
    cfg = dom.config(dt)
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    with pytest.raises(PsphError) as e:
        gd.step(5)
    assert e.value.code == PSPH_ERR_DT_COLLAPSE


def test_particle_leaving_the_domain_is_removed(gpu):
    """CheckParticleLeave (Source/Domain.cpp:517-547): a particle pushed out
    of the domain box is removed at the next cell sort; the others keep their
    original indices."""
    dom, dt, cfg = dam2d()
    p = dom.particles.copy()
    x, v = p.get("x"), p.get("v")
    free = np.flatnonzero(p.get("is_free") == 1)
    k = int(free[np.argmax(x[free, 1] + x[free, 0])])  # the column's top corner
    v[k, 1] = 20.0  # breaks away from the column and rises above the tank walls (~0.45 m) in ~0.03 s
    gd = GpuDomain(cfg)
    gd.upload(p, initial=True)
    n0 = gd.n
    gd.step(1 << 30, t_stop=0.06)
    orig = gd.original_index()
    assert k not in set(orig.tolist())
    assert gd.n == len(orig) < n0
    # downloaded rows follow original_index after the removal: fixed wall
    # particles never move, so their rows hold exactly their uploaded positions
    got = gd.download_fields(("x", "is_free"))
    walls = got["is_free"] == 0
    assert walls.sum() > 0
    np.testing.assert_array_equal(got["x"][walls], x[orig[walls]])
