"""Shared helpers for the GPU parity tests."""
import numpy as np

from oracle.oracle import OracleDomain
from persiansph_gb300.abi import ALL_FIELDS
from persiansph_gb300.particles import ParticleSet
from persiansph_gb300.solver import GpuDomain


def oracle_state(o: OracleDomain) -> ParticleSet:
    arrs = o.download()
    ps = ParticleSet(o.n)
    for f in ALL_FIELDS:
        ps._arr[f] = np.ascontiguousarray(arrs[f])
    return ps


def continue_on_gpu(cfg, o: OracleDomain) -> GpuDomain:
    """A GPU domain holding exactly the oracle's current state."""
    gd = GpuDomain(cfg, grid=o.grid(), integ=o.integrator())
    gd.upload(oracle_state(o), initial=False)
    return gd


def assert_step_parity(gpu: dict, ora: dict, a_scale, dr_scale, dt, tol=1e-12, label=""):
    free = ora["is_free"] == 1
    da = np.linalg.norm(gpu["a"] - ora["a"], axis=1)[free]
    ea = np.max(da / (a_scale[free] + 1e-300))
    dd = np.abs(gpu["ddensity"] - ora["ddensity"])[free]
    ed = np.max(dd / (dr_scale[free] + 1e-300 + 1e-30 * np.abs(ora["density"][free])))
    assert ea <= tol, f"{label}: acceleration rel err {ea:.3e} > {tol}"
    assert ed <= tol, f"{label}: density-rate rel err {ed:.3e} > {tol}"
    # state after the move: errors inherited from a and drho through one step
    vscale = np.abs(ora["v"]).max() + dt * a_scale.max()
    ev = np.max(np.abs(gpu["v"] - ora["v"])) / vscale
    assert ev <= tol, f"{label}: velocity rel err {ev:.3e}"
    ex = np.max(np.abs(gpu["x"] - ora["x"])) / (np.abs(ora["x"]).max() + 1e-300)
    assert ex <= tol, f"{label}: position rel err {ex:.3e}"
    er = np.max(np.abs(gpu["density"] - ora["density"]) / np.abs(ora["density"]))
    assert er <= tol, f"{label}: density rel err {er:.3e}"
    # material state the next step depends on (viscosity, stress, rates): field-norm relative
    for f in ("mu", "strain_rate", "rotation_rate", "sigma", "shear_stress", "strain", "tir", "pressure"):
        ref, got = ora[f][free], gpu[f][free]
        scale = np.max(np.abs(ref))
        if scale == 0.0:
            continue
        e = np.max(np.abs(got - ref)) / scale
        assert e <= 1e3 * tol, f"{label}: {f} rel err {e:.3e}"
    # fluid-soil coupling: saturation state and the weights it sets, the erosion derivative S
    assert np.array_equal(gpu["is_sat"], ora["is_sat"]), f"{label}: saturation state differs"
    em = np.max(np.abs(gpu["mass"] - ora["mass"]) / np.abs(ora["mass"]))
    assert em <= tol, f"{label}: mass rel err {em:.3e}"
    s_scale = np.max(np.abs(ora["s"]))
    if s_scale > 0.0:
        es = np.max(np.abs(gpu["s"] - ora["s"])[free]) / s_scale
        assert es <= 1e3 * tol, f"{label}: S rel err {es:.3e}"
    return ea, ed
