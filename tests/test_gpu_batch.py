"""Ensembles through the C ABI (psph_batch_*): every instance of a batch must
evolve exactly as the same domain alone in a single-domain context (same
pairs, same per-particle summation order, same per-instance time step), and
stop at its own stop time. The single-domain path is itself pinned against
the oracle and the reference (test_gpu_parity.py); one case here also checks
a batch instance against the oracle directly (1e-12, as the single path).
"""
import numpy as np
import pytest

from oracle.oracle import OracleDomain
from persiansph_gb300 import scenarios
from persiansph_gb300.solver import GpuDomain, GpuEnsemble
from tests.golden.cases import CASES
from tests.gpu_helpers import assert_step_parity

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "density", "pressure", "a", "ddensity")


def jittered(builder, seed, frac=0.02):
    """The case's domain with its free particles moved by up to frac*h (seeded);
    seed 0 leaves it unchanged."""
    dom, dt, _ = builder()
    if seed:
        p = dom.particles
        x = p.get("x").copy()
        free = p.get("is_free") == 1
        h = p.get("h")
        d = dom.Dimension
        rng = np.random.default_rng(seed)
        x[free, :d] += frac * h[free, None] * rng.uniform(-1.0, 1.0, (int(free.sum()), d))
        p.set("x", x)
    return dom, dt


def run_single(dom, dt, nsteps, t_stop=float("inf"), fields=FIELDS):
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    done = gd.step(nsteps, t_stop=t_stop)
    return done, gd.download_fields(fields), gd.integrator(), gd.original_index(), gd.grid()


@pytest.mark.parametrize("name", ["dam2d", "dam2d_leapfrog", "poiseuille", "granular", "granular_lf_fail3", "dam3d",
                                  "fluid_options"])
def test_batch_instances_match_single_contexts(gpu, name):
    builder = CASES[name][0]
    doms = [jittered(builder, s) for s in range(3)]
    ens = GpuEnsemble([d.config(dt) for d, dt in doms])
    ens.upload([d.particles for d, _ in doms], initial=True)
    nsteps = 33  # past the Modified Verlet restart (ct == 30)
    done = ens.step(nsteps)
    assert list(done) == [nsteps] * 3
    for q, (d, dt) in enumerate(doms):
        sdone, ref, it, keep, _ = run_single(d, dt, nsteps)
        assert sdone == nsteps
        got = ens.download_fields(q, FIELDS)
        np.testing.assert_array_equal(ens.original_index(q), keep)
        for f in FIELDS:
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{name} instance {q} field {f}")
        bit = ens.integrator(q)
        assert (bit.time, bit.deltat, bit.steps, bit.ct) == (it.time, it.deltat, it.steps, it.ct)


def test_batch_of_different_sizes(gpu):
    """Granular columns of different widths and heights: different particle
    counts and grids per instance, one launch sequence."""
    shapes = [(0.1, 1.0), (0.2, 0.5), (0.15, 2.0), (0.3, 1.0)]
    doms = [scenarios.granular_column(dx=0.01, W=W, aspect=a)[:2] for W, a in shapes]
    ens = GpuEnsemble([d.config(dt) for d, dt in doms])
    ens.upload([d.particles for d, _ in doms], initial=True)
    ens.step(12)
    for q, (d, dt) in enumerate(doms):
        _, ref, it, _, grid = run_single(d, dt, 12)
        got = ens.download_fields(q, FIELDS)
        assert ens.n(q) == d.particles.n
        for f in FIELDS:
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"instance {q} field {f}")
        assert ens.integrator(q).time == it.time
        assert list(ens.grid(q).cell_no) == list(grid.cell_no)
        assert list(ens.grid(q).blpf) == list(grid.blpf)


def test_batch_stop_times(gpu):
    """Each instance runs while its own Time < t_stop (Solve's loop test)."""
    doms = [jittered(CASES["dam2d"][0], 0) for _ in range(3)]
    # times after each step (the adaptive step makes them uneven)
    probe = GpuDomain(doms[0][0].config(doms[0][1]))
    probe.upload(doms[0][0].particles, initial=True)
    times = [probe.time]
    for _ in range(10):
        probe.step(1)
        times.append(probe.time)
    t_stop = np.array([0.5 * (times[3] + times[4]), 0.5 * (times[7] + times[8]), np.inf])
    ens = GpuEnsemble([d.config(t) for d, t in doms])
    ens.upload([d.particles for d, _ in doms], initial=True)
    done = ens.step(20, t_stop=t_stop)
    for q, (d, t) in enumerate(doms):
        sdone, ref, it, _, _ = run_single(d, t, 20, t_stop=float(t_stop[q]))
        assert done[q] == sdone
        got = ens.download_fields(q, FIELDS)
        for f in FIELDS:
            np.testing.assert_array_equal(got[f], ref[f])
        if done[q] < 20:
            assert ens.integrator(q).time >= t_stop[q]
    assert list(done) == [4, 8, 20]
    # a second call continues the instances that have time left
    more = ens.step(5, t_stop=np.array([t_stop[0], 100.0, 100.0]))
    assert more[0] == 0 and more[1] == 5 and more[2] == 5


def test_batch_instance_single_step_parity_with_oracle(gpu):
    d, dt = jittered(CASES["granular"][0], 7)
    other, dt2 = jittered(CASES["granular"][0], 3)
    ens = GpuEnsemble([other.config(dt2), d.config(dt)])
    ens.upload([other.particles, d.particles], initial=True)
    o = OracleDomain(d.config(dt), d.particles, initial=True)
    o.step(1)
    ens.step(1)
    a_scale, dr_scale = o.scales()
    assert_step_parity(ens.download_fields(1), o.download(), a_scale, dr_scale, dt, label="granular batch instance 1")


def test_batch_rejects_unshared_switches(gpu):
    d, dt = jittered(CASES["dam2d"][0], 0)
    c0, c1 = d.config(dt), d.config(dt)
    c1.kernel_type = 1
    with pytest.raises(Exception, match="INVALID_ARGUMENT"):
        GpuEnsemble([c0, c1])


def test_single_domain_calls_refused_on_batch(gpu):
    d, dt = jittered(CASES["dam2d"][0], 0)
    ens = GpuEnsemble([d.config(dt), d.config(dt)])
    ens.upload([d.particles, d.particles], initial=True)
    lib = ens._lib
    import ctypes as C
    done = C.c_int64(0)
    assert lib.psph_step(ens._ctx, 1, 1e300, C.byref(done)) != 0
    assert b"psph_batch_step" in lib.psph_last_error(ens._ctx)
