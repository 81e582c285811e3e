"""Snapshot output (the reference's WriteXDMF, Source/Domain.cpp:1869-2064)
through the C ABI: a snapshot taken at a step's output point (after its
forces, before its update) holds, in float32, that step's starting positions,
velocities, densities and pressures and the step's own accelerations, in
psph_download order; the .xmf offsets match the raw file; Solve (Python and
C++) writes the reference's series of files (<key>_Initial, <key>_0001, ...),
with the driver's UserOutput properties where it sets one."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from persiansph_gb300.snapshot import read_snapshot
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES
from tests.test_cxx_domain import CXX, build

pytestmark = pytest.mark.gpu

SYM6 = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32)


@pytest.mark.parametrize("name,precision", [("dam2d", 0), ("dam2d", 1), ("granular", 0)])
def test_snapshot_is_the_output_steps_state(gpu, tmp_path, name, precision):
    dom, dt, _ = CASES[name][0]()
    cfg = dom.config(dt)
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    gd.step(7)
    fields = ("x", "v", "density", "pressure", "sigma", "strain", "id", "mass", "h", "is_free")
    before = gd.download_fields(fields)
    key = str(tmp_path / "snap")
    gd.request_output(key, ["A", "B", "C"])
    assert gd.step(1) == 1  # the output step
    after = gd.download_fields(fields)
    assert gd.step(4) == 4
    gd.flush_output()
    snap = read_snapshot(key)
    n = len(before["x"])
    assert snap["NP"] == n
    np.testing.assert_array_equal(snap["Position"], f32(before["x"]))
    np.testing.assert_array_equal(snap["Velocity"], f32(before["v"]))
    np.testing.assert_array_equal(snap["Density"], f32(before["density"]))
    np.testing.assert_array_equal(snap["Tag"], before["id"])
    np.testing.assert_array_equal(snap["Mass"], f32(before["mass"]))
    np.testing.assert_array_equal(snap["h"], f32(before["h"]))
    # free particles: the step's starting pressure and stress; walls: the
    # values the step's wall interpolation gave them before the output point
    # (PrimaryComputeAcceleration, Source/Domain.cpp:1164-1206), which the
    # update leaves as they are
    free = before["is_free"] == 1
    pres = np.where(free, before["pressure"], after["pressure"])
    np.testing.assert_array_equal(snap["Pressure"], f32(pres))
    sig = np.where(free[:, None, None], before["sigma"], after["sigma"])
    for k, (r, c) in enumerate(SYM6):
        np.testing.assert_array_equal(snap["Sigma"][:, k], f32(sig[:, r, c]))
        np.testing.assert_array_equal(snap["Strain"][:, k], f32(before["strain"][:, r, c]))
    for nm in ("A", "B", "C"):
        assert not snap[nm].any()  # the default UserOutput writes zeros


def test_snapshot_acceleration_is_the_output_steps(gpu, tmp_path):
    """Two contexts from the same state: one takes a snapshot in its next step,
    the other steps once and downloads; the snapshot's accelerations are that
    step's."""
    dom, dt, _ = CASES["dam2d"][0]()
    cfg = dom.config(dt)
    a = GpuDomain(cfg)
    a.upload(dom.particles, initial=True)
    b = GpuDomain(cfg)
    b.upload(dom.particles, initial=True)
    a.step(4)
    b.step(4)
    key = str(tmp_path / "acc")
    a.request_output(key)
    a.step(1)
    b.step(1)
    a.flush_output()
    snap = read_snapshot(key)
    np.testing.assert_array_equal(snap["Acceleration"], f32(b.download_fields(("a",))["a"]))
    # the state after the output step is the plain step's
    np.testing.assert_array_equal(a.download_fields(("x",))["x"], b.download_fields(("x",))["x"])
    assert snap["Property1"].shape == (b.n,)


def test_write_output_with_properties(gpu, tmp_path):
    dom, dt, _ = CASES["dam2d"][0]()
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    gd.step(3)
    st = gd.download_fields(("v", "density"))
    key = str(tmp_path / "props")
    p1, p3 = st["v"][:, 0], np.arange(gd.n, dtype=np.float64)
    gd.write_output(key, ["VelocityX", "", "Index"], [p1, None, p3])
    snap = read_snapshot(key)
    np.testing.assert_array_equal(snap["VelocityX"], f32(p1))
    assert not snap["Property2"].any()
    np.testing.assert_array_equal(snap["Index"], f32(p3))
    np.testing.assert_array_equal(snap["Velocity"], f32(st["v"]))


def test_python_solve_writes_the_series(gpu, tmp_path):
    dom, dt, _ = CASES["dam2d"][0]()
    key = str(tmp_path / "run")
    dom.Solve(50 * dt, dt, 10 * dt, key)
    names = sorted(f for f in os.listdir(tmp_path) if f.endswith(".xmf"))
    assert names[0] == "run_0001.xmf" and "run_Initial.xmf" in names
    assert len([f for f in names if f != "run_Initial.xmf"]) >= 5
    first, last = read_snapshot(key + "_0001"), read_snapshot(key + "_0005")
    assert not first["Velocity"].any()  # the state at t = 0
    assert np.abs(last["Velocity"]).max() > 0.0


def test_cxx_solve_writes_snapshots(gpu, tmp_path):
    """Domain::Solve with a file key: the reference's file series; with the
    driver's UserOutput its three properties (here v_x, density, ShearRate)."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = build(os.path.join(CXX, "output_driver.cpp"), str(tmp_path / "out_driver"))
    for mode in ("default", "user"):
        key = str(tmp_path / mode)
        args = [exe, key, "0.02", "0.005"] + (["user"] if mode == "user" else [])
        subprocess.run(args, check=True, capture_output=True, text=True)
        for suffix in ("_Initial", "_0001", "_0002", "_0003", "_0004"):
            snap = read_snapshot(key + suffix)
            assert snap["NP"] == len(snap["Tag"]) > 0
            if mode == "user":
                np.testing.assert_array_equal(snap["VelocityX"], snap["Velocity"][:, 0])
                np.testing.assert_array_equal(snap["Density2"], snap["Density"])
            else:
                assert not snap["Property1"].any()
