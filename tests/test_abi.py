"""C-ABI checks that need no GPU: the library loads, exports every function
include/psph.h declares, and the ctypes structures match the C layouts."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from persiansph_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in os.listdir(os.path.join(REPO, "include")):
        if not hdr.endswith(".h"):
            continue
        src = open(os.path.join(REPO, "include", hdr)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(psph_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = abi.load_library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert declared_functions(), "no declarations found"
    assert not missing, f"missing exports: {missing}"


def test_struct_layouts_match_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "psph.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(psph_config), sizeof(psph_grid),
         sizeof(psph_integrator), sizeof(psph_particles), offsetof(psph_config, gravity),
         offsetof(psph_particles, sigma), sizeof(psph_tuning), offsetof(psph_particles, seepage_type),
         offsetof(psph_particles, s));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe])
        out = [int(x) for x in subprocess.check_output([exe]).split()]
    assert out[0] == ctypes.sizeof(abi.PsphConfig)
    assert out[1] == ctypes.sizeof(abi.PsphGrid)
    assert out[2] == ctypes.sizeof(abi.PsphIntegrator)
    assert out[3] == ctypes.sizeof(abi.PsphParticles)
    assert out[4] == abi.PsphConfig.gravity.offset
    assert out[5] == abi.PsphParticles.sigma.offset
    assert out[6] == ctypes.sizeof(abi.PsphTuning)
    assert out[7] == abi.PsphParticles.seepage_type.offset
    assert out[8] == abi.PsphParticles.s.offset


def test_abi_version():
    assert abi.load_library().psph_abi_version() == 3


def test_create_reports_no_device_or_validates():
    """Without a GPU, psph_create fails with a status (never a crash) and the
    error text is readable; bad enums are rejected before any device call."""
    lib = abi.load_library()
    cfg = abi.PsphConfig()
    cfg.dimension = 5
    ctx = ctypes.c_void_p()
    st = lib.psph_create(ctypes.byref(cfg), ctypes.byref(ctx))
    assert st == 1
    assert b"dimension" in lib.psph_last_error(ctx)
    lib.psph_destroy(ctx)


def test_batch_create_validates_shared_switches():
    """An ensemble's instances must agree on the physics switches; the check
    runs before any device call."""
    lib = abi.load_library()
    cfgs = (abi.PsphConfig * 2)()
    for c in cfgs:
        c.dimension = 2
        c.shepard_step = 40
    cfgs[1].kernel_type = 1
    ctx = ctypes.c_void_p()
    st = lib.psph_batch_create(cfgs, 2, ctypes.byref(ctx))
    assert st == 1
    assert b"instance 1" in lib.psph_last_error(ctx)
    lib.psph_destroy(ctx)
    assert lib.psph_batch_create(cfgs, 0, ctypes.byref(ctx)) == 1
