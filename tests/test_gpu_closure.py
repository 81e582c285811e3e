"""Learned closure on the GPU through the C ABI: the network's training
gradients against the CPU oracle (oracle/mlp_oracle.py), the tensor-core
inference against the CUDA-core path and the oracle, deterministic training,
and the closure inside the step (features, eddy viscosity, fallback).

Tolerances: gradients and loss are FP32 sums of FP64-checked terms, 1e-4 of
the largest gradient entry of each layer; network outputs 1e-2 relative (BF16
activations: an FP32 accumulation-order difference can move a hidden value to
the neighbouring BF16 number); features and viscosities from the FP64 form
1e-6 relative to the oracle's fields (features are FP32).
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle.oracle import OracleDomain
from persiansph_gb300 import scenarios
from persiansph_gb300.closure import ClosureNet
from persiansph_gb300.domain import Qubic_Spline
from persiansph_gb300.solver import GpuDomain
from tests.gpu_helpers import continue_on_gpu

pytestmark = pytest.mark.gpu


def synthetic_features(n, seed):
    rng = np.random.default_rng(seed)
    x = np.stack([rng.uniform(-4, 3, n), rng.uniform(-0.2, 0.2, n), rng.uniform(-4, 3, n),
                  rng.uniform(0.98, 1.05, n), np.full(n, 1.3), rng.integers(20, 90, n).astype(float)], 1)
    return x.astype(np.float32)


def synthetic_target(x):
    return (0.01 + 0.05 / (1.0 + np.exp(-(x[:, 0] - x[:, 2]))) + 0.002 * (x[:, 5] - 50) / 40).astype(np.float32)


def test_mlp_gradient_matches_oracle(gpu):
    net = ClosureNet(seed=1)
    x = synthetic_features(1000, 2)
    y = synthetic_target(x)
    net.set_data(x, y)
    net.train(20, batch=256, lr=3e-3, seed=3)  # move away from the initial weights
    p, nrm = net.get()
    loss, g = net.loss_grad(x, y)
    loss_o, g_o = mo.loss_grad(p, nrm, x, y)
    assert loss == pytest.approx(loss_o, rel=1e-5)
    blocks = [(mo.OW1, mo.OB1), (mo.OB1, mo.OW2), (mo.OW2, mo.OB2), (mo.OB2, mo.OW3), (mo.OW3, mo.OB3),
              (mo.OB3, mo.OW4), (mo.OW4, mo.OB4), (mo.OB4, mo.NPARAMS)]
    for a, b in blocks:
        scale = np.max(np.abs(g_o[a:b]))
        err = np.max(np.abs(g[a:b] - g_o[a:b])) / scale
        assert err <= 1e-4, f"gradient block [{a}, {b}): rel err {err:.2e}"


def test_mlp_inference_tensor_cores(gpu):
    net = ClosureNet(seed=4)
    x = synthetic_features(4097, 5)  # ragged last tile
    y = synthetic_target(x)
    net.set_data(x, y)
    net.train(50, batch=512, lr=3e-3, seed=6)
    p, nrm = net.get()
    c_tc = net.infer(x, tensor_cores=True)
    c_cc = net.infer(x, tensor_cores=False)
    c_o = mo.forward(p, nrm, x)["c"]
    scale = np.max(np.abs(c_o))
    assert np.max(np.abs(c_cc - c_o)) / scale <= 1e-2
    assert np.max(np.abs(c_tc - c_o)) / scale <= 1e-2
    assert np.median(np.abs(c_tc - c_o) / scale) <= 1e-4
    # one row's result does not depend on the other rows of its tile
    c_tc2 = net.infer(x[::-1].copy(), tensor_cores=True)[::-1]
    np.testing.assert_array_equal(c_tc, c_tc2)


def test_mlp_training_is_deterministic_and_learns(gpu):
    x = synthetic_features(20000, 7)
    y = synthetic_target(x)
    runs = []
    for _ in range(2):
        net = ClosureNet(seed=8)
        net.set_data(x, y)
        runs.append(net.train(600, batch=1024, lr=3e-3, seed=9))
    np.testing.assert_array_equal(runs[0], runs[1])
    l0, l1 = float(np.mean(runs[0][:10])), float(np.mean(runs[0][-20:]))
    assert l1 < 0.05 * l0, f"loss {l0:.3e} -> {l1:.3e}"


def les_dam3d(precision=0, kernel=None):
    kw = {} if kernel is None else {"kernel": kernel}
    dom, dt, info = scenarios.dam_break_3d(dx=0.04, L=0.24, H=0.2, W=0.16, TL=0.48, TH=0.32, TW=0.2, **kw)
    p = dom.particles
    p.set("les", 1)
    p.set("mu_ref", 1.002e-3)
    p.set("csmag", 0.17)
    cfg = dom.config(dt)
    cfg.precision = precision
    return dom, dt, cfg


def warm_les(warm=5):
    """The LES dam break after a few oracle steps (non-zero strain rates), on
    the oracle and continued on the GPU from the same state."""
    dom, dt, cfg = les_dam3d()
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    o.step(warm)
    rho_before = o.download()["density"].copy()
    gd = continue_on_gpu(cfg, o)
    return dom, dt, o, gd, rho_before


def test_closure_features_and_viscosity_fp64(gpu):
    dx = 0.04
    dom, dt, o, gd, rho_before = warm_les()
    net = ClosureNet(seed=10)
    gd.attach_closure(net, dx)
    o.step(1)
    gd.step(1)
    ro = o.download()
    feats = gd.closure_features()
    g = gd.download_fields(("mu",))
    free = ro["is_free"] == 1
    # neighbour counts: in-support pairs of the reference's pair list, per particle
    cnt = np.bincount(o.pairs(3).ravel(), minlength=len(free))
    vort = np.exp(feats[:, 2].astype(np.float64)) * ro["cs"] / ro["h"]  # |vorticity| from its feature
    f_o, shear = mo.features(ro["strain_rate"], vort, rho_before, ro["ref_density"], ro["h"], dx, cnt, ro["cs"])
    assert np.max(shear[free]) > 0.0
    np.testing.assert_array_equal(feats[free, 5], cnt[free].astype(np.float32))
    assert np.max(np.abs(feats[free, 0] - f_o[free, 0])) <= 1e-5
    assert np.max(np.abs(feats[free, 1] - f_o[free, 1])) <= 1e-4
    assert np.max(np.abs(feats[free, 3] - f_o[free, 3])) <= 1e-6
    np.testing.assert_array_equal(feats[free, 4], (ro["h"][free] / dx).astype(np.float32))
    # eddy viscosity from the network on these features (tensor cores), Mu = MuRef + rho0 nu_t
    c = net.infer(feats[free], tensor_cores=True).astype(np.float64)
    h = ro["h"][free]
    mu_exp = 1.002e-3 + ro["ref_density"][free] * (c * h * h * shear[free])
    err = np.max(np.abs(g["mu"][free] - mu_exp) / mu_exp)
    assert err <= 1e-9, f"closure viscosity rel err {err:.2e}"
    ev, fb = gd.closure_stats()
    assert ev == int(free.sum()) and fb == 0


def test_closure_fallback_is_smagorinsky(gpu):
    dx = 0.04
    dom, dt, o, gd, rho_before = warm_les()
    ro0 = o.download()
    free = ro0["is_free"] == 1
    net = ClosureNet(seed=11)
    _, nrm = net.get()
    # a narrow accepted range of the density ratio: particles above it fall back
    ratio = (rho_before / ro0["ref_density"]).astype(np.float32)
    cut = float(np.median(ratio[free]))
    nrm = nrm.copy()
    nrm[12 + 3], nrm[18 + 3] = -1e30, cut
    net.set(norm=nrm)
    gd.attach_closure(net, dx)
    o.step(1)
    gd.step(1)
    ro = o.download()
    feats = gd.closure_features()
    g = gd.download_fields(("mu",))
    out = free & (feats[:, 3] > np.float32(cut))
    assert out.sum() > 0
    err = np.max(np.abs(g["mu"][out] - ro["mu"][out]) / np.abs(ro["mu"][out]))
    assert err <= 1e-9, f"fallback viscosity differs from the oracle's Smagorinsky: {err:.2e}"
    ev, fb = gd.closure_stats()
    assert ev == int(free.sum()) and fb == int(out.sum())


@pytest.mark.parametrize("precision", [0, 1])
def test_closure_vorticity_rigid_rotation(gpu, precision):
    """|vorticity| of a rigid rotation is 2 Omega where the support lies inside
    the fluid (cubic spline, which integrates to one in 3D)."""
    dx = 0.02
    dom, dt, info = scenarios.dam_break_3d(dx=dx, L=0.4, H=0.4, W=0.4, TL=0.6, TH=0.5, TW=0.5, kernel=Qubic_Spline)
    p = dom.particles
    p.set("les", 1)
    p.set("mu_ref", 1.002e-3)
    x = p.get("x")
    free = p.get("is_free") == 1
    omega = 0.5
    v = np.zeros_like(x)
    v[free, 0] = -omega * (x[free, 1] - 0.2)
    v[free, 1] = omega * (x[free, 0] - 0.2)
    p.set("v", v)
    cfg = dom.config(dt)
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(p, initial=True)
    gd.attach_closure(ClosureNet(seed=12), dx)
    gd.step(1)
    feats = gd.closure_features()
    h = p.get("h")[0]
    lo, hi = np.full(3, 2 * h), np.full(3, 0.4 - 2 * h)
    inner = free & np.all((x >= lo) & (x <= hi), axis=1)
    assert inner.sum() > 100
    w = np.exp(feats[inner, 2].astype(np.float64)) * p.get("cs")[inner] / h  # feature = |vorticity| h / Cs
    assert np.max(np.abs(w / (2 * omega) - 1.0)) <= 0.03


def test_closure_gain_over_smagorinsky(gpu):
    """A-priori gain of the trained network: on a held-out fine run, filtered
    to the coarse lattice, the network's eddy viscosity is closer to the one
    that matches the filtered subgrid stress than the Smagorinsky term the
    LES option uses without it."""
    from persiansph_gb300.closure import apriori_errors, dataset
    small = dict(L=0.15, W=0.3, TL=0.8, TH=0.5, TW=0.3)
    train_cases = [dict(aspect=a, c0=c, **small) for a, c in [(1.5, 35.0), (2.5, 45.0), (1.2, 40.0)]]
    held_out = [dict(aspect=2.0, c0=40.0, **small)]
    times = [0.05, 0.1, 0.15, 0.2]
    X, Y, H, S, _ = dataset(train_cases, 0.01, 0.02, times)
    Xh, Yh, Hh, Sh, _ = dataset(held_out, 0.01, 0.02, times)
    assert len(Y) > 1000 and len(Yh) > 200
    net = ClosureNet(seed=21)
    net.set_data(X, Y)
    w = H * H * S
    net.set_weights(w * w)  # loss in eddy-viscosity units
    losses = net.train(1500, batch=min(2048, len(Y)), lr=2e-3, seed=22)
    assert np.mean(losses[-50:]) < np.mean(losses[:10])
    c_const = float(np.sum(Y * w * w) / np.sum(w * w))  # best constant coefficient (least squares in nu)
    errs = apriori_errors(net, Xh, Yh, Hh, Sh, c_const)
    assert errs["network"] < errs["smagorinsky"], errs


def test_closure_fp32c_features_match_fp64(gpu):
    """The FP32C form computes the closure's shear-rate features in FP32 from
    its own strain-rate sums: from the same state they agree with the FP64
    form's features, and so do the eddy viscosities (1e-4 relative)."""
    dx = 0.04
    dom, dt, cfg = les_dam3d()
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    o.step(5)
    net = ClosureNet(seed=13)
    out = {}
    for prec in (0, 1):
        c = dom.config(dt)
        c.precision = prec
        gd = continue_on_gpu(c, o)
        gd.attach_closure(net, dx)
        gd.step(1)
        out[prec] = (gd.closure_features(), gd.download_fields(("mu", "is_free")))
        gd.close()
    f64, f32 = out[0][0], out[1][0]
    free = out[0][1]["is_free"] == 1
    assert np.max(np.abs(f32[free, 0] - f64[free, 0])) <= 1e-3
    assert np.max(np.abs(f32[free, 1] - f64[free, 1])) <= 1e-3
    assert np.max(np.abs(f32[free, 2] - f64[free, 2])) <= 1e-3
    assert np.max(np.abs(f32[free, 3] - f64[free, 3])) <= 1e-6
    np.testing.assert_array_equal(f32[free, 4], f64[free, 4])
    assert np.max(np.abs(f32[free, 5] - f64[free, 5])) <= 1  # a pair at the support edge may differ
    mu64, mu32 = out[0][1]["mu"][free], out[1][1]["mu"][free]
    assert np.max(np.abs(mu32 - mu64) / mu64) <= 1e-4


def test_closure_aposteriori_gain(gpu):
    """A-posteriori test of the shipped network on the benchmark geometry (3D
    dam break, tank 3.22 x 1 x 1 m, column 1.2 x 0.55 x 1 m): the coarse
    dx = 20 mm run with the network, with Smagorinsky (Mat1's LES term,
    Source/Particle.cpp:157-160) and laminar (LES off), against the fine
    dx = 10 mm plain run, 0.05 - 0.4 s. What the network gains, asserted:
    - surge front: within 1 % of the fine run, and at most half the
      Smagorinsky run's error (the network 0.78 %, Smagorinsky 2.4 %);
    - box-filtered velocity at 0.35 and 0.4 s: closer to the fine run than
      laminar's (0.102 / 0.103 against 0.107 / 0.108 relative L2).
    What it does not gain (recorded, not asserted): the front matches the
    laminar run's to 1e-5, and Smagorinsky's filtered velocity is closer to
    the fine run's at every time."""
    from persiansph_gb300.closure import default_network_path, fine_snapshots
    from persiansph_gb300.closure_train import HELD_OUT, coarse_run, filtered_velocity_error, surge_front
    net = ClosureNet.load(default_network_path())
    times = [0.05 * (k + 1) for k in range(8)]
    dx_f, dx_c = 0.01, 0.02
    snaps, _ = fine_snapshots([HELD_OUT], dx_f, times)
    fine_front = np.array([surge_front(s["x"], dx_f) for s in snaps[0]])
    res = {}
    for mode in ("closure", "smagorinsky", "laminar"):
        runs, _ = coarse_run(mode, dx_c, times, net)
        front = np.array([r["front"] for r in runs])
        res[mode] = {"front_err": float(np.max(np.abs(front - fine_front) / fine_front)),
                     "vel_l2": [filtered_velocity_error(f, c, dx_c) for f, c in zip(snaps[0], runs)]}
    print(res)
    net_, smag, lam = res["closure"], res["smagorinsky"], res["laminar"]
    assert net_["front_err"] <= 0.01
    assert net_["front_err"] <= 0.5 * smag["front_err"]
    for k in (-2, -1):
        assert net_["vel_l2"][k] < lam["vel_l2"][k]
