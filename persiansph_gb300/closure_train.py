"""Trains the learned eddy-viscosity closure for the coarse 3D dam break and
evaluates it (a priori on a held-out fine run, a posteriori by coarse runs).

  python -m persiansph_gb300.closure_train [--pairs 0.01:0.02,0.005:0.01]
         [--cases 8] [--t-end 0.4] [--out persiansph_gb300/data/closure_dam3d.npz]

1. Fine runs of the plain method (LES on, FP32C pair arithmetic), generated as
   one ensemble by the batched solver for each (fine, coarse) lattice pair:
   columns L = 0.3 m wide with aspect H/L drawn from U[1, 3] and c0 from
   U[30, 50] m/s (seeded), in a 1.6 x 1.0 x 1.0 m tank (0.3 m deep, column
   and tank, for fine spacings below 7.5 mm, which bounds the particle count),
   snapshots every 0.05 s. Two lattice pairs put coarse spacings of 20 mm
   (the coarse dam break) and 10 mm into one training set; the rate features
   are in units of Cs / h, so the network also serves finer lattices.
2. Each snapshot is box-filtered onto the coarse lattice; the coarse particle
   set gets its features from one step of the runtime kernels, and the target
   eddy viscosity is the one that best matches the filtered subgrid stress.
3. The network is trained by the library's own kernels (Adam).
4. Held-out fine run: the benchmark geometry (1.2 x 0.55 x 1.0 m column in a
   3.22 x 1.0 x 1.0 m tank, c0 = 40) at the fine spacing. A priori: eddy
   viscosity error of the network, of the Smagorinsky term and of the best
   constant coefficient. A posteriori: coarse runs with the closure, with the
   Smagorinsky LES term and without LES, against the fine run's surge front and
   box-filtered velocity.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

from .closure import ClosureNet, apriori_errors, box_filter, closure_samples, coarse_from_filter, fine_snapshots, les_case

HELD_OUT = dict(L=1.2, H=0.55, W=1.0, TL=3.22, TH=1.0, TW=1.0, c0=40.0)


def surge_front(x, dx):
    low = x[:, 1] < 2.0 * dx
    return float(x[low, 0].max()) if low.any() else float("nan")


def samples_from_snapshots(cases, snaps, dx_f, dx_c):
    m3 = round(dx_c / dx_f) ** 3
    X, Y, H, S = [], [], [], []
    for q, case in enumerate(cases):
        for sn in snaps[q]:
            filt = box_filter(sn["x"], sn["v"], sn["density"], dx_c)
            cset, cfg, nw, keep = coarse_from_filter(case, dx_c, filt, 0.5 * m3)
            x, y, aux = closure_samples(cset, cfg, dx_c, nw, filt["tau"][keep])
            X.append(x); Y.append(y); H.append(aux["h"]); S.append(aux["shear"])
    return np.concatenate(X), np.concatenate(Y), np.concatenate(H), np.concatenate(S)


def coarse_run(mode, dx_c, times, net=None, precision=1):
    """The held-out geometry at the coarse spacing: 'closure', 'smagorinsky'
    (LES term of Mat1) or 'laminar' (LES off). Returns per time (front, x, v)."""
    from .solver import GpuDomain
    dom, dt, info = les_case(dx_c, **HELD_OUT)
    if mode == "laminar":
        dom.particles.set("les", 0)
    cfg = dom.config(dt)
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(dom.particles, initial=True)
    if mode == "closure":
        gd.attach_closure(net, dx_c)
    out = []
    t0 = time.perf_counter()
    for t in times:
        gd.step(1 << 30, t_stop=t)
        st = gd.download_fields(("x", "v", "is_free"))
        fl = st["is_free"] == 1
        out.append({"t": gd.time, "front": surge_front(st["x"][fl], dx_c), "x": st["x"][fl], "v": st["v"][fl]})
    wall = time.perf_counter() - t0
    stats = gd.closure_stats() if mode == "closure" else (0, 0)
    gd.close()
    return out, {"seconds": wall, "closure_evaluated": stats[0], "closure_fallbacks": stats[1]}


def filtered_velocity_error(fine, coarse, dx_c):
    """Relative L2 difference of the box-filtered velocities on the cells both
    runs occupy."""
    def cells(x, v):
        f = box_filter(x, v, np.ones(len(x)), dx_c)
        return {tuple(np.round(c / dx_c - 0.5).astype(int)): u for c, u in zip(f["centre"], f["v"])}
    a, b = cells(fine["x"], fine["v"]), cells(coarse["x"], coarse["v"])
    keys = [k for k in a if k in b]
    ua = np.array([a[k] for k in keys])
    ub = np.array([b[k] for k in keys])
    return float(np.linalg.norm(ub - ua) / np.linalg.norm(ua))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", default="0.01:0.02,0.005:0.01",
                    help="fine:coarse lattice spacings of the training runs; the first pair also serves the "
                         "held-out evaluation")
    ap.add_argument("--cases", type=int, default=8)
    ap.add_argument("--t-end", type=float, default=0.4)
    ap.add_argument("--dt-snap", type=float, default=0.05)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                                                 "closure_dam3d.npz"))
    args = ap.parse_args(argv)
    rng = np.random.default_rng(args.seed)
    times = [round(args.dt_snap * (k + 1), 10) for k in range(int(round(args.t_end / args.dt_snap)))]
    cases = [dict(aspect=float(rng.uniform(1.0, 3.0)), c0=float(rng.uniform(30.0, 50.0))) for _ in range(args.cases)]
    pairs = [tuple(float(v) for v in p.split(":")) for p in args.pairs.split(",")]
    dx_fine, dx_coarse = pairs[0]
    report = {"pairs": pairs, "cases": cases, "times": times, "fine_particles": {}, "fine_seconds": {},
              "samples": {}}

    parts = []
    for dx_f, dx_c in pairs:
        geo = {} if dx_f >= 0.0075 else dict(W=0.3, TW=0.3)
        pcases = [dict(c, **geo) for c in cases]
        t0 = time.perf_counter()
        snaps, infos = fine_snapshots(pcases, dx_f, times)
        key = f"{dx_f}:{dx_c}"
        report["fine_particles"][key] = [int(i["n_fluid"] + i["n_wall"]) for i in infos]
        report["fine_seconds"][key] = time.perf_counter() - t0
        parts.append(samples_from_snapshots(pcases, snaps, dx_f, dx_c))
        report["samples"][key] = int(len(parts[-1][1]))
        del snaps
    X, Y, H, S = (np.concatenate([p[k] for p in parts]) for k in range(4))

    hsnaps, hinfos = fine_snapshots([HELD_OUT], dx_fine, times)
    Xh, Yh, Hh, Sh = samples_from_snapshots([HELD_OUT], hsnaps, dx_fine, dx_coarse)
    report["held_out_samples"] = int(len(Yh))
    report["held_out_fine_particles"] = int(hinfos[0]["n_fluid"] + hinfos[0]["n_wall"])

    net = ClosureNet(seed=args.seed)
    net.set_data(X, Y)
    # the loss in eddy-viscosity units: nu = c h^2 ShearRate, so weight
    # (h^2 ShearRate)^2, scaled to mean 1 within each lattice pair (so that
    # the finer pair, with smaller h, counts as much as the coarser one)
    wp = [(p[2] * p[2] * p[3]) ** 2 for p in parts]
    net.set_weights(np.concatenate([a / np.mean(a) for a in wp]))
    w = H * H * S
    t1 = time.perf_counter()
    losses = net.train(args.steps, batch=min(args.batch, len(Y)), lr=args.lr, seed=args.seed + 1)
    report["train_seconds"] = time.perf_counter() - t1
    report["loss_first"] = float(np.mean(losses[:20]))
    report["loss_last"] = float(np.mean(losses[-100:]))
    c_const = float(np.sum(Y * w * w) / np.sum(w * w))
    report["c_const"] = c_const
    report["apriori_held_out"] = apriori_errors(net, Xh, Yh, Hh, Sh, c_const)

    fine_front = [surge_front(s["x"], dx_fine) for s in hsnaps[0]]
    report["fine_front"] = fine_front
    post = {}
    for mode in ("closure", "smagorinsky", "laminar"):
        runs, info = coarse_run(mode, dx_coarse, times, net)
        fr = [r["front"] for r in runs]
        post[mode] = {
            "front": fr,
            "front_rel_err_max": float(np.max(np.abs(np.array(fr) - fine_front) / np.array(fine_front))),
            "filtered_velocity_rel_l2": [filtered_velocity_error(f, c, dx_coarse) for f, c in zip(hsnaps[0], runs)],
            **info,
        }
    report["aposteriori"] = post
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    net.save(args.out, report=json.dumps(report))
    with open(os.path.splitext(args.out)[0] + "_report.json", "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps({k: report[k] for k in ("samples", "held_out_samples", "loss_first", "loss_last",
                                             "apriori_held_out")}))
    print(json.dumps({m: {k: v for k, v in post[m].items() if k != "front"} for m in post}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
