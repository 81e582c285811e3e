"""The C++ SPH::Domain (include/persiansph/Domain.h) driving the GPU: a
driver in the reference's style solves the dam2d parity case through
Domain::Solve; its final state is bit-identical to the same case solved
through the Python Domain mirror and GpuDomain (both call the same C ABI)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES
from tests.test_cxx_domain import CXX, build

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_cxx_solve_matches_python_path(gpu, tmp_path, precision):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = build(os.path.join(CXX, "dam2d_driver.cpp"), str(tmp_path / "dam2d"))
    tf = 0.05
    out = str(tmp_path / "state.bin")
    subprocess.run([exe, out, repr(tf), str(precision)], check=True, capture_output=True, text=True)
    raw = np.fromfile(out, np.uint8)
    n = int(raw[:8].view(np.int64)[0])
    a = raw[8:].view(np.float64)
    x, v = a[:3 * n].reshape(n, 3), a[3 * n:6 * n].reshape(n, 3)
    rho, p, t = a[6 * n:7 * n], a[7 * n:8 * n], a[8 * n]

    dom, dt, _ = CASES["dam2d"][0]()
    cfg = dom.config(dt)
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    gd.step(1 << 40, t_stop=tf)
    ref = gd.download_fields(("x", "v", "density", "pressure"))
    assert n == gd.n
    assert t == gd.time
    np.testing.assert_array_equal(x, ref["x"])
    np.testing.assert_array_equal(v, ref["v"])
    np.testing.assert_array_equal(rho, ref["density"])
    np.testing.assert_array_equal(p, ref["pressure"])


def test_cxx_inout_solve_matches_python_path(gpu, tmp_path):
    """An in/out-flow channel with user InCon / OutCon / AllCon hooks (the
    HydraulicJump.cpp pattern) solved through the C++ Domain::Solve and
    through the Python Domain.Solve with the same hooks: identical states,
    including the particles the boundary recycled and appended."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = build(os.path.join(CXX, "channel_driver.cpp"), str(tmp_path / "channel"))
    tf = 0.015
    out = str(tmp_path / "state.bin")
    subprocess.run([exe, out, repr(tf)], check=True, capture_output=True, text=True)
    raw = np.fromfile(out, np.uint8)
    n = int(raw[:8].view(np.int64)[0])
    a = raw[8:8 + 8 * (8 * n + 1)].view(np.float64)
    x, v = a[:3 * n].reshape(n, 3), a[3 * n:6 * n].reshape(n, 3)
    rho, p, t = a[6 * n:7 * n], a[7 * n:8 * n], a[8 * n]
    ints = raw[8 + 8 * (8 * n + 1):].view(np.int32)
    in_out, ids = ints[:n], ints[n:2 * n]

    from tests.golden.cases import channel_profile
    dom, dt, info = channel_profile()
    dom.AllCon = dom.InCon
    dom.BC.allv = [info["U"], 0.0, 0.0]
    dom.BC.allDensity = 1000.0
    dom.particles.set("v", np.zeros((dom.particles.n, 3)))
    dom.Solve(tf, dt, tf)
    ps = dom.particles
    assert n == ps.n
    assert t == dom.Time
    np.testing.assert_array_equal(x, ps.get("x"))
    np.testing.assert_array_equal(v, ps.get("v"))
    np.testing.assert_array_equal(rho, ps.get("density"))
    np.testing.assert_array_equal(p, ps.get("pressure"))
    np.testing.assert_array_equal(in_out, ps.get("in_out"))
    np.testing.assert_array_equal(ids, ps.get("id"))
    assert (in_out == 1).any() and (in_out == 2).any()


def _spring(dom):
    p = dom.particles
    free = p.get("is_free") != 0
    a, x = p.get("a"), p.get("x")
    a[free, 0] += 20.0 * (0.5 - x[free, 0])
    a[free, 1] += 20.0 * (0.3 - x[free, 1])
    p.set("a", a)


def _damping(dom):
    p = dom.particles
    free = p.get("is_free") != 0
    if dom.Time < 0.02:
        a, v = p.get("a"), p.get("v")
        a[free] -= 2.0 * v[free]
        p.set("a", a)
    if dom.Time >= 0.01:
        al, x = p.get("alpha"), p.get("x")
        al[free & (x[:, 0] < 0.2)] = 0.05
        p.set("alpha", al)


def test_cxx_hooks_solve_matches_python_path(gpu, tmp_path):
    """GeneralBefore (a spring) and GeneralAfter (damping, then a new
    artificial viscosity for part of the fluid) run every step on the host:
    the C++ Domain::Solve and the Python Domain.Solve with the same hooks give
    identical states, different from the run without hooks."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = build(os.path.join(CXX, "dam2d_driver.cpp"), str(tmp_path / "dam2d"))
    tf = 0.03
    out = str(tmp_path / "state.bin")
    subprocess.run([exe, out, repr(tf), "0", "hooks"], check=True, capture_output=True, text=True)
    raw = np.fromfile(out, np.uint8)
    n = int(raw[:8].view(np.int64)[0])
    a = raw[8:].view(np.float64)
    x, v = a[:3 * n].reshape(n, 3), a[3 * n:6 * n].reshape(n, 3)
    rho, t = a[6 * n:7 * n], a[8 * n]

    dom, dt, _ = CASES["dam2d"][0]()
    dom.GeneralBefore = _spring
    dom.GeneralAfter = _damping
    dom.Solve(tf, dt, tf)
    ps = dom.particles
    assert n == ps.n and t == dom.Time
    np.testing.assert_array_equal(x, ps.get("x"))
    np.testing.assert_array_equal(v, ps.get("v"))
    np.testing.assert_array_equal(rho, ps.get("density"))
    assert np.any(ps.get("alpha") == 0.05)

    plain, dt2, _ = CASES["dam2d"][0]()
    plain.Solve(tf, dt2, tf)
    assert not np.array_equal(plain.particles.get("x"), ps.get("x"))
