"""Benchmark: pair-interactions/s and steps/s of the 3D dam break on one GB300.

Workload (default): tank 3.22 x 1.0 x 1.0 m, water column 1.2 x 0.55 x 1.0 m
at dx = 5 mm -> 240 x 110 x 200 = 5,280,000 fluid particles plus 3 wall layers,
Wendland C2 (h = 1.3 dx), Tait EOS c0 = 40 m/s, artificial viscosity 0.05,
Morris viscosity, Modified Verlet + Shepard (the 4-DamBreak3D.cpp pattern).
Synthetic, seeded lattice input built by persiansph_gb300.scenarios.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
  python bench.py --workload dam2d|poiseuille2d|dam3d_coarse   (the smaller configurations)

Our arm: W untimed steps, then K steps timed with CUDA events on the solver's
stream (inputs resident in HBM; the working set, several GB, exceeds the 129 MB
L2, so no flush is needed). `e2e` repeats the measurement through the C ABI
with host buffers: upload + K steps + download inside the timed region.
The reference arm (--impl reference) times the reference algorithm on the host
cores: the CPU oracle (a restatement of the reference, OpenMP on every core)
on the same workload at the same lattice, as many timed steps as fit a fixed
budget after one warm-up step. The `cpu_baseline` of our arm is a bounded
sample of the same workload (the same tank at dx = 10 mm, 5 steps).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = ("pair-interactions/s @ 3D dam break (5.28M fluid particles), FP32C form with the learned closure; "
          "FP64 plain beside it")


def max_over_ranks(value: float, dist, device) -> float:
    """The largest of the ranks' values (the job's timed region ends with its
    slowest replica); the value itself on one rank (dist None)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def metric_name(workload: str) -> str:
    if workload == "dam3d":
        return METRIC
    return f"pair-interactions/s @ {workload}, FP32C form; FP64 plain beside it"
UNIT = "pair-interactions/s"
# Host seconds the reference arm's timed steps may take (it runs the full
# workload: one step of the 6.7M-particle 3D dam break is ~35 s on 16 cores).
REF_BUDGET_S = 90.0
# FP64 operations per pair-interaction of the fluid pair force for this
# workload's options (Wendland, Tait, artificial viscosity, Morris, squared
# density), counted from forces_fluid_kernel's arithmetic on the taken branches
# with an FMA counted as 2 and a division or square root as 1: 90 for one
# evaluation and 16 for the partner's terms (a, dDensity, ZWab, SumDen), as
# CalcForce11 does once per unordered pair (Source/Interaction.cpp:139-145).
FLOPS_PER_PAIR = 106
# Algorithmic HBM bytes per particle of one FP32C fluid pair-kernel launch:
# read each particle's inputs once (offset+h 16, v+p 16, 1/rho, p/rho^2, c, rho
# 16, class 4, cell 4) and write its outputs once (a + drho 32, zwab 8, sumden
# 8) = 104 B; with LES and the closure also the viscosity (4), the strain-rate
# sums (6 x 4) and the closure's four features (16) = 148 B.
FORCE32_BYTES_PER_PARTICLE = {False: 104, True: 148}
# DRAM bytes per particle one launch actually moved: ncu captures of the same
# kernels on the same tank at dx = 10 mm (1,021,104 particles),
# dram__bytes_read.sum + dram__bytes_write.sum per particle (LES + closure
# flavour with the 5 % list skin the autotuner picks: 276.56 + 54.12 MB; without
# LES: an earlier capture of that flavour, lists every step); the traffic grows
# with the particle count, so a full-size launch moves this x n. Most of the
# excess over the algorithmic bytes is the neighbour list (~80 entries x 4 B a
# particle).
FORCE32_TRAFFIC_BYTES_PER_PARTICLE = {False: 304.6, True: 323.9}
# Pipe activity of that launch (LES + closure flavour, list skin) and of the FP64
# pair kernel (pass A) in the same capture series (sm__pipe_*_cycles_active, % of
# peak).
FORCE32_NCU = {"issue_active": 0.573, "fma_pipe": 0.297, "fp64_pipe": 0.040, "warps_active": 0.298}
FORCE64_NCU_FP64_PIPE = 0.834


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi sampling (SM clock, throttle reasons) started before the warm-up
    steps; `summary()` keeps the samples taken inside the marked timed region."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # let the sampler come up before anything is timed
        deadline = time.time() + 10.0
        while self.proc and time.time() < deadline and os.path.getsize(self.path) == 0:
            time.sleep(0.05)
        return self

    def start(self):
        self.t0 = time.time()

    def stop(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        import datetime
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 10:
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                except ValueError:
                    ts = None
                rows.append((ts, parts[1:]))
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        inside = [r for ts, r in rows if ts is not None and self.t0 is not None and self.t1 is not None
                  and self.t0 - 0.2 <= ts <= self.t1 + 0.2]
        window = "timed region"
        if not inside:
            inside, window = [r for _, r in rows], "whole run (timed region shorter than the sampling period)"
        num = lambda x: float(x) if x.replace(".", "").isdigit() else None
        sm = [v for v in (num(r[1]) for r in inside) if v is not None]
        mx = [v for v in (num(r[2]) for r in inside) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in inside for k in range(4) if r[5 + k].lower() == "active"})
        loaded = [v for v in sm if v > 0.5 * (max(mx) if mx else 1)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside), "window": window}


# The workloads --workload selects. "dam3d" (the default) is the headline: the
# 3D dam break the metric is quoted on; the others are the smaller benchmark
# configurations, measured with the same contract.
WORKLOADS = {
    "dam3d": {"desc": "3D dam break: tank 3.22x1.0x1.0 m, column 1.2x0.55x1.0 m, dx=%g m", "dx": 0.005,
              "ref_dx": 0.01, "closure": True},
    "dam3d_coarse": {"desc": "3D dam break, LES on, learned closure: tank 3.22x1.0x1.0 m, column 1.2x0.55x1.0 m, "
                             "dx=%g m", "dx": 0.02, "ref_dx": 0.02, "closure": True},
    "dam2d": {"desc": "2D dam break: tank 4.0x3.0 m, column 1.0x2.0 m, cubic spline h=1.2dx, dx=%g m",
              "dx": 0.005, "ref_dx": 0.005, "closure": False},
    "poiseuille2d": {"desc": "2D Poiseuille flow: channel 1.0e-3 m, periodic 0.5e-3 m, quintic spline h=1.3dx, "
                             "dx=%g m", "dx": 2.5e-5, "ref_dx": 2.5e-5, "closure": False},
}


def closure_verdict():
    """What the shipped network gains a posteriori, from its training report
    (held-out benchmark geometry, coarse dx = 20 mm against the fine dx = 10 mm
    plain run, 0.05 - 0.4 s; tests/test_gpu_closure.py::test_closure_aposteriori_gain
    reruns it)."""
    from persiansph_gb300.closure import default_network_path
    path = os.path.splitext(default_network_path())[0] + "_report.json"
    try:
        post = json.load(open(path))["aposteriori"]
    except (OSError, KeyError, ValueError):
        return {}
    fr = {m: round(post[m]["front_rel_err_max"], 5) for m in ("closure", "smagorinsky", "laminar")}
    vl = {m: round(post[m]["filtered_velocity_rel_l2"][-1], 4) for m in ("closure", "smagorinsky", "laminar")}
    return {"aposteriori": {
        "surge_front_max_rel_err": fr, "filtered_velocity_rel_l2_at_0.4s": vl,
        "verdict": ("front: network 3x better than Smagorinsky, equal to laminar (no gain over laminar); "
                    "late filtered velocity: network better than laminar, slightly worse than Smagorinsky")}}


def build_workload(dx, name="dam3d"):
    from persiansph_gb300 import scenarios
    if name == "dam3d":
        return scenarios.dam_break_3d(dx=dx)
    if name == "dam3d_coarse":
        from persiansph_gb300.closure import les_case
        return les_case(dx, L=1.2, H=0.55, W=1.0, TL=3.22, TH=1.0, TW=1.0, c0=40.0)
    if name == "dam2d":
        return scenarios.dam_break_2d(dx=dx)
    if name == "poiseuille2d":
        dom, dt, info = scenarios.poiseuille(dx=dx)
        free = dom.particles.get("is_free") == 1
        info.setdefault("n_fluid", int(free.sum()))
        info.setdefault("n_wall", int((~free).sum()))
        return dom, dt, info
    raise ValueError(name)


def measure_ensemble(n_inst: int, dx: float, steps: int, warmup: int):
    """The batched granular-column workload (CalcForce2233 + Mat3): n_inst
    independent 2D columns in one context, FP32C pair sums with the FP64
    stress return mapping, each step one CUDA-graph launch sequence for all
    instances. Returns its line object."""
    from persiansph_gb300 import scenarios
    from persiansph_gb300.solver import GpuEnsemble
    cases = scenarios.granular_ensemble(n=n_inst, seed=0, dx=dx)
    cfgs = []
    for dom, dt, _ in cases:
        cfg = dom.config(dt)
        cfg.precision = 1  # PSPH_FP32C
        cfgs.append(cfg)
    ens = GpuEnsemble(cfgs)
    ens.upload([d.particles for d, _, _ in cases], initial=True)
    ens.step(warmup)
    pc0 = ens.pair_count()
    ms, done = ens.step_timed(steps)
    pairs = ens.pair_count() - pc0
    launches = ens.last_launch_count()
    ens.enable_timing(True)
    ens.step(2)
    phases = {k: x / 2.0 for k, x in ens.phase_times().items()}
    ens.close()
    counts = [d.particles.n for d, _, _ in cases]
    soil = [i["n_soil"] for _, _, i in cases]
    return {"workload": f"{n_inst} 2D granular columns (Drucker-Prager soil, Fail 2, TI on), W=0.2 m, "
                        f"H/W ~ U[0.5,4], phi ~ U[20,40] deg, dx={dx} m (seed 0)",
            "instances": n_inst, "particles": int(sum(counts)), "soil_per_instance": [int(min(soil)), int(max(soil))],
            "form": "FP32C pair sums, FP64 stress return mapping", "steps": done,
            "ms_per_step": ms / max(done, 1), "steps_per_s": done / (ms * 1e-3),
            "pair_interactions_per_s": pairs / (ms * 1e-3), "pairs_per_step": pairs / max(done, 1),
            "gpu_launches_per_step": launches / max(done, 1), "phase_ms": phases}


def cpu_reference(dx_sample: float, steps: int, warmup: int, threads: int, workload: str = "dam3d",
                  budget_s: float | None = None):
    """Times the CPU oracle (restatement of the reference's OpenMP path) on the
    workload at lattice spacing dx_sample: `warmup` untimed steps, then `steps`
    timed steps (with budget_s, fewer when the warm-up step shows that they
    would take longer than that, at least one). Returns pair-interactions/s
    (pairs counted by the oracle's own pair forces) and details."""
    from oracle.oracle import OracleDomain
    dom, dt, info = build_workload(dx_sample, workload)
    o = OracleDomain(dom.config(dt), dom.particles, initial=True)
    t_w = None
    if warmup:
        t0 = time.perf_counter()
        o.step(warmup, threads)
        t_w = (time.perf_counter() - t0) / warmup
    if budget_s is not None and t_w:
        steps = max(1, min(steps, int(budget_s / t_w)))
    p0 = o.pair_count()
    t0 = time.perf_counter()
    o.step(steps, threads)
    el = time.perf_counter() - t0
    pairs_per_step = (o.pair_count() - p0) / steps
    o.close()
    return {"value": pairs_per_step * steps / el, "steps_per_s": steps / el, "seconds": el, "steps": steps,
            "n": dom.particles.n, "n_fluid": info["n_fluid"], "pairs_per_step": pairs_per_step}


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    wl = WORKLOADS[args.workload]
    # the reference arm runs the workload itself (same lattice as our arm);
    # a step of the 6.7M-particle 3D dam break takes tens of seconds on the
    # host cores, so the timed steps are as many as fit REF_BUDGET_S after
    # one warm-up step (at most --steps)
    ref_dx = args.ref_dx if args.ref_dx else args.dx
    r = cpu_reference(ref_dx, max(1, args.steps), 1, threads, args.workload, budget_s=REF_BUDGET_S)
    steps = r["steps"]
    same = ref_dx == args.dx
    line = {
        "impl": "reference", "metric": metric_name(args.workload), "value": r["value"], "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": steps, "warmup": 1, "ms_per_step": 1e3 * r["seconds"] / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic lattice (seeded)",
        "config": {"workload": ("" if same else "sample of the ") + wl["desc"] % ref_dx,
                   "particles": r["n"], "fluid": r["n_fluid"], "pairs_per_step": r["pairs_per_step"]},
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} timed steps (after 1 warm-up step) of the {args.workload} workload "
                                   f"at dx={ref_dx} m ({r['n']} particles); steps bounded by a "
                                   f"{REF_BUDGET_S:.0f} s budget"},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "steps_per_s": r["steps_per_s"],
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam3d", choices=sorted(WORKLOADS))
    ap.add_argument("--dx", type=float, default=None, help="lattice spacing (default: the workload's)")
    ap.add_argument("--ref-dx", type=float, default=None, help="lattice spacing of the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--develop", type=float, default=0.25,
                    help="physical time (s) the workload is advanced with the headline form before any timing "
                         "(0: time from rest); the default times the dam break's surge at speed, where lists "
                         "with a skin are rebuilt most often")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched granular-column line")
    ap.add_argument("--tuning", default="auto",
                    help="'auto' (psph_autotune on the workload's own steps) or BLOCK:SPLIT[:STAGE[:SKIN]] to fix the "
                         "launch shape (STAGE: staged candidates per neighbour-scan block, 0 = none; SKIN: FP32C "
                         "neighbour-list skin in thousandths of the support, 0 = lists every step)")
    ap.add_argument("--ens-n", type=int, default=256)
    ap.add_argument("--ens-dx", type=float, default=1e-3)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.dx is None:
        args.dx = WORKLOADS[args.workload]["dx"]

    if args.impl == "reference":
        return run_reference_arm(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from persiansph_gb300.solver import GpuDomain
    from persiansph_gb300.particles import ParticleSet
    from persiansph_gb300 import abi
    import ctypes

    wl = WORKLOADS[args.workload]
    dom, dt, info = build_workload(args.dx, args.workload)
    n = dom.particles.n
    from persiansph_gb300.closure import ClosureNet, default_network_path
    net = ClosureNet.load(default_network_path())
    state = None  # (particles, grid, integrator) of the developed flow

    def upload_set(closure):
        """The particles a measured context starts from: the workload's initial
        lattice, or the developed flow (the same fields), with LES on every
        particle for the closure form (its eddy viscosity from the network)."""
        if state is None:
            ps = dom.particles.copy()
        else:
            # the workload's fields and the flow's state (the initial lattice
            # sets no velocity: v and the integrator's histories come along)
            ps = ParticleSet(state[0].n)
            for f in set(dom.particles.arrays()) | {"x", "v", "va", "vb", "density", "densitya", "densityb",
                                                    "pressure"}:
                if state[0].has(f):
                    ps.set(f, state[0].get(f).copy())
            if not closure:  # the constant viscosity, not the developed eddy viscosity
                ps.set("mu", dom.particles.get("mu").copy())
        ps.set("les", np.full(ps.n, 1 if closure else 0, np.int32))
        return ps

    def open_domain(precision, closure, pset=None):
        cfg = dom.config(dt)
        cfg.precision = precision
        gd = GpuDomain(cfg, grid=state[1] if state else None, integ=state[2] if state else None)
        gd.upload(pset if pset is not None else upload_set(closure), initial=state is None)
        if closure:
            gd.attach_closure(net, args.dx)
        return cfg, gd

    def apply_tuning(gd, precision):
        if args.tuning == "auto":
            return gd.autotune(3)  # launch shapes timed on this workload's own (untimed) steps
        parts = [int(x) for x in args.tuning.split(":")]
        gd.set_tuning(parts[0], parts[1], parts[2] if len(parts) > 2 else None,
                      parts[3] if len(parts) > 3 and precision == 1 else None)
        return gd.tuning()

    # A developed flow: the workload advanced with the headline form before any
    # timing. From rest the fluid barely moves for the first thousand steps,
    # which says little about a run and would flatter lists kept with a skin.
    develop = {"t": 0.0, "steps": 0, "s": 0.0}
    if args.develop > 0.0:
        _, gdv = open_domain(1, wl["closure"])
        apply_tuning(gdv, 1)
        t0 = time.perf_counter()
        gdv.step(1 << 40, t_stop=args.develop)
        torch.cuda.synchronize()
        integ = gdv.integrator()
        develop = {"t": integ.time, "steps": int(integ.steps), "s": time.perf_counter() - t0}
        state = (gdv.download(), gdv.grid(), integ)
        gdv.close()

    def measure(precision, closure=False):
        cfg, gd = open_domain(precision, closure)
        tuning = apply_tuning(gd, precision)
        with ClockSampler(local) as clk:
            gd.step(args.warmup)
            pc0 = gd.pair_count()
            rb0 = gd.list_rebuilds()
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            clk.start()
            ms, done = gd.step_timed(args.steps)
            torch.cuda.synchronize()
            clk.stop()
        pc1 = gd.pair_count()
        rebuilds = gd.list_rebuilds() - rb0
        ms = max_over_ranks(ms, dist, "cuda")
        launches = gd.last_launch_count()
        # per-phase device times (separate run, events between phases; long
        # enough to hold the rebuilds of a list skin)
        gd.enable_timing(True)
        gd.step(24)
        phases = {k: x / 24.0 for k, x in gd.phase_times().items()}
        gd.enable_timing(False)
        pairs = pc1 - pc0
        cstats = gd.closure_stats() if closure else (0, 0)
        gd.close()
        return {"cfg": cfg, "tuning": tuning, "closure_evaluated": cstats[0], "closure_fallbacks": cstats[1], "ms": ms, "done": done, "pairs": pairs, "launches": launches, "phases": phases,
                "clocks": clk.summary(), "value_rank": pairs / (ms * 1e-3), "steps_per_s": done / (ms * 1e-3),
                "list_rebuilds": rebuilds,
                "pairs_per_step": pairs / max(done, 1)}

    m32 = measure(1, closure=wl["closure"])  # PSPH_FP32C + learned closure: the headline form
    m32n = measure(1)                # PSPH_FP32C without the closure (LES off)
    m64 = measure(0)                 # PSPH_FP64: the plain form
    lib = abi.load_library()
    fp64 = ctypes.c_double(0.0)
    lib.psph_probe_fp64_peak(ctypes.byref(fp64))
    pk = peaks()
    force32_ms = m32["phases"]["forces"]
    force64_ms = m64["phases"]["forces"]
    cl = bool(wl["closure"])
    achieved_gbs = FORCE32_BYTES_PER_PARTICLE[cl] * n / (force32_ms * 1e-3) / 1e9
    fp64_tflops = m64["pairs_per_step"] * FLOPS_PER_PAIR / (force64_ms * 1e-3) / 1e12
    traffic = FORCE32_TRAFFIC_BYTES_PER_PARTICLE[cl] * n

    # end to end through the C ABI with host buffers: create + upload + K
    # steps + download, for the headline form and for the FP64 plain form
    fields = ("x", "v", "density", "pressure", "a", "ddensity")

    def end_to_end(precision, closure, tuning):
        host = upload_set(closure)  # the caller's host arrays, ready before the clock starts
        t0 = time.perf_counter()
        _, ge = open_domain(precision, closure, host)
        ge.set_tuning(tuning["pair_block"], tuning["cell_split"], tuning.get("nlist_stage"),
                      tuning.get("skin_permille") if precision == 1 else None)
        done_e = ge.step(args.steps)
        out = ge.download_fields(fields)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        pe = ge.pair_count()
        ge.close()
        return pe / el, done_e, sum(a.nbytes for a in out.values())

    e2e_v, done_e, d2h = end_to_end(1, wl["closure"], m32["tuning"])
    e2e64_v, done_e64, d2h64 = end_to_end(0, False, m64["tuning"])
    h2d = sum(a.nbytes for a in upload_set(False).arrays().values())

    def phase_dict(m):
        return dict(m["phases"])

    world_mult = world
    line = {
        "metric": metric_name(args.workload), "value": m32["value_rank"] * world_mult, "unit": UNIT,
        "n_gpus": world,
        "steps": m32["done"], "warmup": args.warmup, "ms_per_step": m32["ms"] / max(m32["done"], 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair arithmetic (Kahan-compensated sums), f64 integration",
        "data": ("synthetic lattice (seeded); inputs larger than L2 (no flush needed); timed from the flow "
                 f"developed to t = {develop['t']:.4f} s ({develop['steps']} steps of the headline form from rest, "
                 f"{develop['s']:.1f} s)" if develop["steps"] else
                 "synthetic lattice (seeded), timed from rest; inputs larger than L2 (no flush needed)"),
        "config": {"workload": wl["desc"] % args.dx, "particles": n, "fluid": info.get("n_fluid"),
                   "walls": info.get("n_wall"),
                   "form": ("FP32C + learned eddy-viscosity closure (LES on every fluid particle)" if wl["closure"]
                            else "FP32C"),
                   "parallelism": "replicas only" if world > 1 else "single GPU",
                   "l2": "working set > L2" if n * 300 > 129e6 else "working set fits in L2"},
        "steps_per_s": m32["steps_per_s"], "pairs_per_step": m32["pairs_per_step"], "tuning": m32["tuning"],
        "list_rebuilds": {"timed_steps": m32["done"], "rebuilds": m32["list_rebuilds"],
                          "note": "steps of the timed region that ran the cell sort and the neighbour lists "
                                  "(every step without a list skin; with one, when a particle had moved half of "
                                  "it since the last rebuild); every step evaluates exactly the in-support pairs"},
        "phase_ms": phase_dict(m32),
        "closure": {"evaluated": m32["closure_evaluated"], "fallbacks": m32["closure_fallbacks"],
                    "network": os.path.relpath(default_network_path(), REPO), **closure_verdict()},
        "fp32c_no_closure": {"value": m32n["value_rank"] * world_mult, "unit": UNIT,
                             "steps_per_s": m32n["steps_per_s"], "ms_per_step": m32n["ms"] / max(m32n["done"], 1),
                             "phase_ms": phase_dict(m32n)},
        "fp64_plain": {"value": m64["value_rank"] * world_mult, "unit": UNIT, "steps_per_s": m64["steps_per_s"],
                       "ms_per_step": m64["ms"] / max(m64["done"], 1), "phase_ms": phase_dict(m64),
                       "clocks": m64["clocks"],
                       "e2e": {"value": e2e64_v, "unit": UNIT, "h2d_bytes_per_step": h2d / max(done_e64, 1),
                               "d2h_bytes_per_step": d2h64 / max(done_e64, 1), "steps": done_e64,
                               "note": "FP64 plain form: create + upload + steps + download through the C ABI, "
                                       "host wall clock"}},
        "fp32c_closure_over_fp64_steps_per_s": m32["steps_per_s"] / m64["steps_per_s"],
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved_gbs / pk["hbm_gbs"], "traffic": traffic,
                     "kernel": "forces_fluid32_kernel", "peak_source": pk["src"],
                     "bytes_per_particle": FORCE32_BYTES_PER_PARTICLE[cl],
                     "note": "latency-bound gather kernel (neither HBM nor tensor bound); ncu pipe activity of "
                             "the same kernel at dx=10 mm in ncu_small_case "
                             "(profiles/pair_kernel_skin_dam3d_10mm.md)",
                     "ncu_small_case": FORCE32_NCU},
        "roofline_fp64": {"bound": "fp64", "kernel": "forces_fluid_kernel", "achieved": fp64_tflops,
                          "peak": fp64.value, "unit": "TFLOP/s",
                          "frac": fp64_tflops / fp64.value if fp64.value else None,
                          "peak_source": "measured here by psph_probe_fp64_peak (DFMA chains)",
                          "fp64_pipe_active_ncu_small_case": FORCE64_NCU_FP64_PIPE,
                          "note": "frac counts 106 algorithmic FP64 flops per pair-interaction (one evaluation "
                                  "and the partner's terms, each pair once) against the DFMA rate; the FP64 pipe "
                                  "itself is ~83 % busy (square roots, divisions, conversions, idle lanes)"},
        "clocks": m32["clocks"],
        "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": h2d / max(done_e, 1),
                "d2h_bytes_per_step": d2h / max(done_e, 1), "steps": done_e,
                "note": "create + upload + steps + download through the C ABI, host wall clock"},
        "gpu_launches": m32["launches"],
    }
    if not args.no_ensemble and args.workload == "dam3d":
        line["ensemble"] = measure_ensemble(args.ens_n, args.ens_dx, max(args.steps // 2, 5), args.warmup)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        ref_dx = args.ref_dx if args.ref_dx else wl["ref_dx"]
        cpu_steps = 5 if args.workload == "dam3d" else 10
        r = cpu_reference(ref_dx, cpu_steps, 1, threads, args.workload)
        line["cpu_baseline"] = {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port",
                                "steps_per_s": r["steps_per_s"],
                                "sample": f"{cpu_steps} steps of the same workload ({args.workload}) at dx={ref_dx} m "
                                          f"({r['n']} particles) after 1 warm-up step"}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
