"""The CPU oracle against the reference's own outputs (tests/golden, made by
tests/golden/make_golden.py from the unmodified reference). These pin the
oracle: every stored field must agree to the last bits."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleDomain
from tests.golden.cases import BOXES, CASES

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference(name):
    builder, nsteps, dumps = CASES[name]
    dom, dt, _ = builder()
    g = load(name)
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    o.use_flow_hooks(dom)
    o.use_step_hooks(dom)
    grid = o.grid()
    np.testing.assert_array_equal(np.array(grid.blpf), g["grid_blpf"])
    np.testing.assert_array_equal(np.array(grid.trpr), g["grid_trpr"])
    np.testing.assert_array_equal(np.array(grid.cell_no, dtype=float), g["grid_cell_no"])
    prev = 0
    for k in dumps:
        o.step(k - prev)
        prev = k
        st = o.download()
        it = o.integrator()
        assert o.n == int(g[f"n_{k}"])
        assert it.time == pytest.approx(float(g[f"time_{k}"]), rel=1e-14)
        for key in g:
            if not key.endswith(f"_{k}") or key.startswith(("n_", "time_", "deltat_")):
                continue
            f = key[: -len(f"_{k}")]
            ref = g[key]
            got = st[f].reshape(ref.shape)
            scale = max(np.max(np.abs(ref)), 1e-300)
            err = np.max(np.abs(got - ref)) / scale if ref.size else 0.0
            assert err <= 1e-13, f"{name} step {k} field {f}: rel err {err:.3e}"


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_pair_lists_match_reference(name):
    builder, _, _ = CASES[name]
    dom, dt, _ = builder()
    g = load(name)
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    for which, key in enumerate(("sm", "fsm", "nsm")):
        got = o.pairs(which)
        np.testing.assert_array_equal(got, g["pairs_" + key])  # same pairs, same order, same orientation


@pytest.mark.parametrize("name", sorted(BOXES))
def test_add_box_length_matches_reference(name):
    from persiansph_gb300.domain import Domain
    dim, tag, V, Lx, Ly, Lz, r, rho, h, type_, rot, random, fixed = BOXES[name]
    g = load("boxes")
    dom = Domain()
    dom.Dimension = dim
    dom.AddBoxLength(tag, V, Lx, Ly, Lz, r, rho, h, type_, rot, random, fixed)
    np.testing.assert_array_equal(dom.particles.get("x"), g[name + "_x"])
    np.testing.assert_array_equal(dom.particles.get("mass"), g[name + "_mass"])
