"""psph_pairs_export_noalloc: the pair export for callers that cannot allocate
device memory when they need the pairs (their device memory is already held by
their own pool or another framework's allocator, or their loop must not take
cudaMalloc's device-wide synchronisation). It must return exactly the pairs of
the allocating psph_pairs_export, call after call, and refuse contexts larger
than its static scratch. Collected last on purpose: it runs after every other
test, and also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from persiansph_gb300 import scenarios
from persiansph_gb300.abi import PsphError
from persiansph_gb300.solver import GpuDomain
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu
MAX_PARTICLES = 1 << 20  # PSPH_NOALLOC_MAX_PARTICLES in include/psph.h


def _noalloc(gd, which, buf, cap):
    n = ctypes.c_int64(-1)
    st = gd._lib.psph_pairs_export_noalloc(gd._ctx, which, ctypes.c_void_p(buf), cap, ctypes.byref(n))
    return st, n.value


@pytest.mark.parametrize("name", ["dam2d", "poiseuille", "dam3d", "granular"])
def test_noalloc_export_matches_allocating_export(gpu, name):
    import torch
    dom, dt, _ = CASES[name][0]()
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    gd.step(3)
    for which in (0, 1):
        ref = gd.pairs(which)  # allocating export (host output)
        ref_set = set(map(tuple, ref.tolist()))
        buf = torch.empty((len(ref) + 64, 2), dtype=torch.int64, device="cuda")
        for _call in range(2):  # the static scratch keeps the last call's contents
            buf.fill_(-7)
            torch.cuda.synchronize()
            st, n = _noalloc(gd, which, buf.data_ptr(), buf.shape[0])
            assert st == 0, gd._lib.psph_last_error(gd._ctx)
            assert n == len(ref)
            got = buf[:n].cpu().numpy()
            assert set(map(tuple, got.tolist())) == ref_set
            assert (buf[n:].cpu().numpy() == -7).all()  # nothing written past the pairs
        # count only: no buffer, the full count
        st, n = _noalloc(gd, which, 0, 0)
        assert st == 0 and n == len(ref)
        # truncated output: exactly cap pairs of the set, nothing past cap, the full count
        cap = len(ref) // 2
        buf.fill_(-7)
        torch.cuda.synchronize()
        st, n = _noalloc(gd, which, buf.data_ptr(), cap)
        assert st == 0 and n == len(ref)
        got = buf[:cap].cpu().numpy()
        assert len(set(map(tuple, got.tolist()))) == cap
        assert set(map(tuple, got.tolist())) <= ref_set
        assert (buf[cap:].cpu().numpy() == -7).all()


def test_noalloc_export_rejects_contexts_above_its_limit(gpu):
    dom, dt, info = scenarios.dam_break_3d(dx=0.0085)
    assert dom.particles.n > MAX_PARTICLES
    gd = GpuDomain(dom.config(dt))
    gd.upload(dom.particles, initial=True)
    st, _ = _noalloc(gd, 0, 0, 0)
    assert st == 1  # PSPH_ERR_INVALID_ARGUMENT
    assert b"at most" in gd._lib.psph_last_error(gd._ctx)
