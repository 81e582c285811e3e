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
