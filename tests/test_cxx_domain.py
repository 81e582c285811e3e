"""The C++ SPH::Domain layer (include/persiansph/Domain.h), no GPU needed:
drivers in the reference's style compile and link against it, its
AddBoxLength reproduces the reference's lattices (golden fixture from the
unmodified reference), and Solve reports a missing device as the reference
reports errors (a Fatal caught by MECHSYS_CATCH)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from persiansph_gb300 import abi
from tests.golden.cases import BOXES

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CXX = os.path.join(REPO, "tests", "cxx")
GOLD = os.path.join(REPO, "tests", "golden")


def build(src, out):
    lib = os.path.dirname(abi.library_path())
    abi.load_library()  # builds the library when it is missing or stale
    # -ffp-contract=off: no fused multiply-add in the lattice arithmetic (Arm
    # compilers contract by default), so positions match the x86 build bit for bit
    cmd = ["g++", "-std=c++14", "-O2", "-Wall", "-ffp-contract=off", "-I", os.path.join(REPO, "include", "persiansph"), "-I",
           os.path.join(REPO, "include"), src, "-L", lib, "-lpsph_gb300", f"-Wl,-rpath,{lib}", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


@pytest.fixture(scope="module")
def bindir(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    return tmp_path_factory.mktemp("cxx")


def read_lattice(path):
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    a = np.frombuffer(raw[8:], np.float64)
    return a[:3 * n].reshape(n, 3), a[3 * n:4 * n]


@pytest.mark.parametrize("name", sorted(BOXES))
def test_add_box_length_matches_reference(bindir, name):
    exe = os.path.join(bindir, "lattice_dump")
    if not os.path.exists(exe):
        build(os.path.join(CXX, "lattice_dump.cpp"), exe)
    dim, tag, V, Lx, Ly, Lz, r, rho, h, type_, rot, random, fixed = BOXES[name]
    out = os.path.join(bindir, name + ".bin")
    args = [dim, tag, *V, Lx, Ly, Lz, r, rho, h, type_, rot, int(random), int(fixed)]
    subprocess.run([exe, *[repr(float(a)) if isinstance(a, float) else str(a) for a in args], out], check=True)
    x, m = read_lattice(out)
    g = dict(np.load(os.path.join(GOLD, "boxes.npz")))
    np.testing.assert_array_equal(x, g[name + "_x"])
    np.testing.assert_array_equal(m, g[name + "_mass"])


def test_driver_builds_and_reports_missing_device(bindir):
    exe = build(os.path.join(CXX, "dam2d_driver.cpp"), os.path.join(bindir, "dam2d"))
    lib = abi.load_library()
    import ctypes
    if lib.psph_device_check(ctypes.byref(ctypes.c_int(0))) == 0:
        pytest.skip("a device is present: the GPU test runs this driver")
    res = subprocess.run([exe, os.path.join(bindir, "o.bin"), "0.01"], capture_output=True, text=True)
    assert res.returncode == 1
    assert "Fatal: no sm_103 CUDA device available" in res.stdout


def reference_dir():
    """The reference checkout: PSPH_REFERENCE_DIR, else the directory the
    oracle recipe (oracle/build_ref.sh) built the reference from."""
    env = os.environ.get("PSPH_REFERENCE_DIR")
    if env:
        return env
    rec = os.path.join(REPO, "oracle", "_ref", "REFERENCE_DIR")
    if os.path.exists(rec):
        with open(rec) as f:
            return f.read().strip()
    return None


REFERENCE_DRIVERS = ("1-Poiseuille.cpp", "2-Couette.cpp", "3-DamBreak.cpp", "4-DamBreak3D.cpp")


@pytest.mark.parametrize("name", REFERENCE_DRIVERS)
def test_reference_drivers_compile_unchanged(bindir, name):
    """The reference's own example drivers, read where the reference is
    checked out (PSPH_REFERENCE_DIR, else where oracle/build_ref.sh found it),
    compile against this Domain.h."""
    src = os.path.join(reference_dir() or "", name)
    if not os.path.exists(src):
        pytest.skip("reference sources not present")
    cmd = ["g++", "-std=c++14", "-fsyntax-only", "-I", os.path.join(REPO, "include", "persiansph"), "-I",
           os.path.join(REPO, "include"), src]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
