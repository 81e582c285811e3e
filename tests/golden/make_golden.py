"""Generates the golden fixtures in tests/golden/ from the UNMODIFIED reference.

Run here, where the reference sources are present:
    sh oracle/build_ref.sh && python tests/golden/make_golden.py [case ...]
Each case builds its initial particles with persiansph_gb300.scenarios (the
same deterministic builders the tests use), runs oracle/_ref/ref_driver (the
reference compiled with the project's shims, Nproc=1) and stores, per dump
step, the fields the parity tests compare, plus the reference's pair lists of
the initial state and AddBoxLength lattices. The fixtures are small npz files.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle.oracle import read_pairs_dir, read_state_dir, reference_box, run_reference, write_state_dir  # noqa: E402
from tests.golden.cases import CASES, BOXES  # noqa: E402

FIELDS = ("x", "v", "density", "pressure", "a", "ddensity", "zwab", "sigma", "strain_rate", "rotation_rate",
          "shear_stress", "tir", "va", "vb", "densitya", "densityb", "mu", "nsv", "sumkernel", "mass",
          "ref_density", "is_sat", "s", "strain", "in_out")


def main(only=()):
    """Writes every fixture, or with case names only those cases' fixtures."""
    for name, (builder, nsteps, dumps) in CASES.items():
        if only and name not in only:
            continue
        dom, dt, info = builder()
        cfg = dom.config(dt)
        # user InCon / OutCon: the reference driver's profile hooks with the same parameters
        # user hooks: the reference driver's hooks with the same parameters
        extra = {k: list(info[k]) for k in ("flow_profile", "damping", "spring") if k in info} or None
        with tempfile.TemporaryDirectory() as d:
            write_state_dir(os.path.join(d, "in"), cfg, dom.particles, extra)
            run_reference(os.path.join(d, "in"), os.path.join(d, "out"), nsteps, 1, [0] + list(dumps))
            out = {}
            for k in dumps:
                cfgk, arrs = read_state_dir(os.path.join(d, "out", f"step_{k}"))
                out[f"n_{k}"] = np.array(int(cfgk["n"][0]))
                out[f"time_{k}"] = np.array(cfgk["time"][0])
                out[f"deltat_{k}"] = np.array(cfgk["deltat"][0])
                for f in FIELDS:
                    if f in arrs:
                        out[f"{f}_{k}"] = arrs[f]
            cfg0, _ = read_state_dir(os.path.join(d, "out", "step_0"))
            for key in ("blpf", "trpr", "cell_size", "cell_no", "dom_size", "hmax"):
                out[f"grid_{key}"] = np.array(cfg0[key])
            pairs = read_pairs_dir(os.path.join(d, "out", "pairs_0"))
            for k, v in pairs.items():
                out[f"pairs_{k}"] = v
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, "n", dom.particles.n, "pairs", sum(len(v) for v in pairs.values()))
    if only:
        return
    # surge front of a longer dam break (reference run, Nproc = all host threads)
    from tests.golden.cases import SURGE_STEPS, surge2d, surge_front
    dom, dt, _ = surge2d()
    cfg = dom.config(dt)
    with tempfile.TemporaryDirectory() as d:
        write_state_dir(os.path.join(d, "in"), cfg, dom.particles)
        run_reference(os.path.join(d, "in"), os.path.join(d, "out"), SURGE_STEPS[-1], os.cpu_count() or 1,
                      list(SURGE_STEPS))
        times, fronts = [], []
        for k in SURGE_STEPS:
            cfgk, arrs = read_state_dir(os.path.join(d, "out", f"step_{k}"))
            times.append(cfgk["time"][0])
            fronts.append(surge_front(arrs["x"], arrs["is_free"]))
    np.savez_compressed(os.path.join(HERE, "surge2d.npz"), steps=np.array(SURGE_STEPS), time=np.array(times),
                        front=np.array(fronts))
    print("surge2d", list(zip(times, fronts)))
    boxes = {}
    for name, args in BOXES.items():
        with tempfile.TemporaryDirectory() as d:
            r = reference_box(d, *args)
        boxes[f"{name}_x"] = r["x"]
        boxes[f"{name}_mass"] = r["mass"]
    np.savez_compressed(os.path.join(HERE, "boxes.npz"), **boxes)
    print("boxes", list(BOXES))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
