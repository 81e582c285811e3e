"""Relative error of the FP32C form against the FP64 form, field by field.

  python -m persiansph_gb300.precision_report [--dx 0.005] [--t-end 1.0]
  python -m persiansph_gb300.precision_report --case dam3d --dx 0.005 --t-end 0.25 \
         --closure persiansph_gb300/data/closure_dam3d.npz

Workload: the 2D dam break (1.0 m x 2.0 m water column in a 4.0 m x 3.0 m
tank, cubic spline h = 1.2 dx, Tait EOS c0 = 10 sqrt(2 g H), alpha = 0.1),
80,000 fluid particles at dx = 5 mm. Both forms start from the same state:

* one step: per field, max |FP32C - FP64| / max |FP64| and the RMS of the
  difference over the RMS of the FP64 field, for the accelerations, density
  rates, positions, velocities, densities and pressures (with --developed T:
  one step of each form from the same FP64 state at time T, instead of the
  long run);
* the run to t_end: surge-front position (largest x of a fluid particle within
  2 dx of the floor) of both forms over time, and the same field norms at the
  end (the flows decorrelate particle by particle as a dam break does between
  any two runs that differ in rounding, so the end-state norms measure that
  divergence, while the front measures the flow).

--case dam3d runs the 3D dam break of the benchmark instead (1.2 x 0.55 x 1.0
m column, 3.22 x 1.0 x 1.0 m tank, Wendland C2, c0 = 40); with --closure the
FP32C form also runs the learned eddy-viscosity closure (LES on, network from
the given file) while the FP64 form is the plain method.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

FIELDS = ("a", "ddensity", "x", "v", "density", "pressure")


def field_errors(a, b):
    """Per field: max |a - b| / max |b| and RMS(a - b) / RMS(b) over the
    particles both runs still hold (CheckParticleLeave may remove a particle
    in one run and not the other), matched by original index."""
    common, ia, ib = np.intersect1d(a["orig"], b["orig"], return_indices=True)
    out = {"particles_compared": int(len(common))}
    for f in FIELDS:
        x, y = np.asarray(a[f], np.float64)[ia], np.asarray(b[f], np.float64)[ib]
        ref = np.max(np.abs(y))
        rms = np.sqrt(np.mean(y * y))
        out[f] = {"max_rel": float(np.max(np.abs(x - y)) / ref) if ref > 0 else 0.0,
                  "rms_rel": float(np.sqrt(np.mean((x - y) ** 2)) / rms) if rms > 0 else 0.0}
    return out


def developed_step(dom, dt, t_dev, closure=None, dx=None):
    """Per-field errors of one FP32C step against one FP64 step, both taken
    from the same developed FP64 state at t_dev (the first step from rest has
    zero velocities and density rates, so it says little about them)."""
    from .solver import GpuDomain
    cfg = dom.config(dt)
    cfg.precision = 0
    base = GpuDomain(cfg)
    base.upload(dom.particles, initial=True)
    base.step(1 << 40, t_stop=t_dev)
    state, grid, integ = base.download(), base.grid(), base.integrator()
    base.close()
    out = {}
    for name, prec in (("fp64", 0), ("fp32c", 1)):
        c = dom.config(dt)
        c.precision = prec
        gd = GpuDomain(c, grid=grid, integ=integ)
        gd.upload(state, initial=False)
        if closure is not None:
            gd.attach_closure(closure, dx)
        gd.step(1)
        out[name] = gd.download_fields(FIELDS + ("is_free",))
        out[name]["orig"] = gd.original_index()
        gd.close()
    return {"t": t_dev, "errors": field_errors(out["fp32c"], out["fp64"])}


def front(st, dx):
    fl = st["is_free"] == 1
    low = st["x"][:, 1] < 2.0 * dx
    return float(st["x"][fl & low, 0].max())


def main(argv=None):
    from . import scenarios
    from .solver import GpuDomain
    ap = argparse.ArgumentParser()
    ap.add_argument("--dx", type=float, default=0.005)
    ap.add_argument("--t-end", type=float, default=1.0)
    ap.add_argument("--dt-out", type=float, default=0.1)
    ap.add_argument("--case", default="dam2d", choices=["dam2d", "dam3d"])
    ap.add_argument("--closure", default=None)
    ap.add_argument("--developed", type=float, default=None,
                    help="only the one-step per-field errors from the FP64 state at this time")
    args = ap.parse_args(argv)
    if args.case == "dam2d":
        dom, dt, info = scenarios.dam_break_2d(dx=args.dx)
        workload = "2D dam break, 1.0 x 2.0 m column, 4.0 x 3.0 m tank, dx=%g m" % args.dx
    else:
        dom, dt, info = scenarios.dam_break_3d(dx=args.dx)
        workload = "3D dam break, 1.2 x 0.55 x 1.0 m column, 3.22 x 1.0 x 1.0 m tank, dx=%g m" % args.dx
    if args.developed is not None:
        rep = {"workload": workload, "particles": dom.particles.n, "fluid": info["n_fluid"],
               "developed_step": developed_step(dom, dt, args.developed)}
        print(json.dumps(rep, indent=1))
        return 0
    sims = {}
    for name, prec in (("fp64", 0), ("fp32c", 1)):
        p = dom.particles
        if name == "fp32c" and args.closure:
            p = p.copy()
            p.set("les", 1)
            p.set("csmag", 0.17)
        cfg = dom.config(dt)
        cfg.precision = prec
        sims[name] = GpuDomain(cfg)
        sims[name].upload(p, initial=True)
        if name == "fp32c" and args.closure:
            from .closure import ClosureNet
            net = ClosureNet.load(args.closure)
            sims[name].attach_closure(net, args.dx)
    report = {"workload": workload, "particles": dom.particles.n, "fluid": info["n_fluid"],
              "fp32c_form": "FP32C + learned closure" if args.closure else "FP32C"}
    flds = FIELDS + ("is_free",)

    def state(sim):
        out = sim.download_fields(flds)
        out["orig"] = sim.original_index()
        return out

    for s in sims.values():
        s.step(1)
    st = {k: state(s) for k, s in sims.items()}
    report["one_step"] = field_errors(st["fp32c"], st["fp64"])
    times = [args.dt_out * (k + 1) for k in range(int(round(args.t_end / args.dt_out)))]
    fronts = {k: [] for k in sims}
    secs = {}
    for k, s in sims.items():
        t0 = time.perf_counter()
        for t in times:
            s.step(1 << 40, t_stop=t)
            fronts[k].append(front(s.download_fields(("x", "is_free")), args.dx))
        secs[k] = time.perf_counter() - t0
    st = {k: state(s) for k, s in sims.items()}
    f64, f32 = np.array(fronts["fp64"]), np.array(fronts["fp32c"])
    report["times"] = times
    report["front"] = fronts
    report["front_rel_diff_max"] = float(np.max(np.abs(f32 - f64) / f64))
    report["end_state"] = field_errors(st["fp32c"], st["fp64"])
    report["seconds"] = secs
    report["steps"] = {k: int(s.integrator().steps) for k, s in sims.items()}
    if args.closure:
        report["closure_evaluated"], report["closure_fallbacks"] = sims["fp32c"].closure_stats()
    print(json.dumps(report, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
