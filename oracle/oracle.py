"""ctypes wrapper of the CPU oracle (psph_oracle.c) and of the reference driver.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py, never by the product package.
"""
from __future__ import annotations

import copy
import ctypes as C
import json
import os
import subprocess

import numpy as np

from persiansph_gb300.abi import (ALL_FIELDS, INT_FIELDS, NO_FLOW_FN, NO_HOOK_FN, PSPH_FLOW_IN, PSPH_FLOW_OUT,
                                  PSPH_HOOK_AFTER, PSPH_HOOK_BEFORE, FlowFn, HookFn, PsphConfig, PsphGrid,
                                  PsphIntegrator, PsphParticles, field_dtype, field_shape, flow_callback,
                                  particles_struct, step_hook_callback)
from persiansph_gb300.particles import ParticleSet

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libpsph_oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")


def build_oracle(force: bool = False) -> str:
    """Compiles psph_oracle.c (plain C + OpenMP) into oracle/_build/."""
    src = os.path.join(HERE, "psph_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(REPO, "include", "psph.h"))):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-Wno-int-in-bool-context", f"-I{REPO}/include", f"-I{HERE}", src, "-o", LIB, "-lm"]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB)
        P = C.POINTER
        L.psph_oracle_create.restype = C.c_void_p
        L.psph_oracle_create.argtypes = [P(PsphConfig), P(PsphParticles), C.c_int, P(PsphGrid), P(PsphIntegrator)]
        L.psph_oracle_destroy.argtypes = [C.c_void_p]
        L.psph_oracle_error.argtypes = [C.c_void_p]
        L.psph_oracle_error.restype = C.c_char_p
        L.psph_oracle_step.argtypes = [C.c_void_p, C.c_int64, C.c_int]
        L.psph_oracle_num_particles.argtypes = [C.c_void_p]
        L.psph_oracle_num_particles.restype = C.c_int64
        L.psph_oracle_download.argtypes = [C.c_void_p, P(PsphParticles)]
        L.psph_oracle_original_index.argtypes = [C.c_void_p, P(C.c_int64)]
        L.psph_oracle_get_grid.argtypes = [C.c_void_p, P(PsphGrid)]
        L.psph_oracle_get_integrator.argtypes = [C.c_void_p, P(PsphIntegrator)]
        L.psph_oracle_pairs.argtypes = [C.c_void_p, C.c_int, P(C.c_int64), C.c_int64]
        L.psph_oracle_pairs.restype = C.c_int64
        L.psph_oracle_scales.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.psph_oracle_phase_times.argtypes = [C.c_void_p, P(C.c_double), C.c_int]
        L.psph_oracle_pair_count.argtypes = [C.c_void_p]
        L.psph_oracle_pair_count.restype = C.c_int64
        L.psph_oracle_set_flow_profile.argtypes = [C.c_void_p, C.c_int, FlowFn, C.c_void_p]
        L.psph_oracle_set_step_hooks.argtypes = [C.c_void_p, HookFn, C.c_void_p, C.c_int]
        L.psph_oracle_patch.argtypes = [C.c_void_p, P(PsphParticles)]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


class OracleDomain:
    """CPU oracle with the same call surface as persiansph_gb300.solver.GpuDomain."""

    def __init__(self, cfg: PsphConfig, pset: ParticleSet, initial: bool = True, grid: PsphGrid | None = None,
                 integ: PsphIntegrator | None = None):
        L = lib()
        arrs = {f: np.ascontiguousarray(pset.get(f)) for f in ALL_FIELDS if pset.has(f)}
        s = particles_struct(arrs, pset.n)
        self._cfg = cfg
        self._flow_cbs, self._flow_errors = {}, []
        self._h = L.psph_oracle_create(C.byref(cfg), C.byref(s), int(initial),
                                       C.byref(grid) if grid is not None else None,
                                       C.byref(integ) if integ is not None else None)
        err = L.psph_oracle_error(self._h).decode()
        if err:
            L.psph_oracle_destroy(self._h)
            self._h = None
            raise OracleError(err)

    def close(self):
        if self._h:
            lib().psph_oracle_destroy(self._h)
            self._h = None

    def set_flow_profile(self, which: int, fn=None):
        """A user InCon (PSPH_FLOW_IN) or OutCon (PSPH_FLOW_OUT): fn(position)
        -> (velocity, density); None restores the BC constants."""
        cb = flow_callback(fn, self._flow_errors) if fn is not None else NO_FLOW_FN
        lib().psph_oracle_set_flow_profile(self._h, int(which), cb, None)
        self._flow_cbs[which] = cb

    def set_step_hooks(self, before=None, after=None):
        """Domain::GeneralBefore / GeneralAfter: hook(time, particles) with the
        particles as a ParticleSet, changed in place (or returned), written back."""
        hooks = {}
        if before is not None:
            hooks[PSPH_HOOK_BEFORE] = before
        if after is not None:
            hooks[PSPH_HOOK_AFTER] = after
        if not hooks:
            lib().psph_oracle_set_step_hooks(self._h, NO_HOOK_FN, None, 0)
            self._hook_cb = None
            return

        def run(fn):
            pset = ParticleSet(self.n)
            pset._arr.update(self.download())
            out = fn(self.integrator().time, pset)
            self.patch(out if out is not None else pset)

        cb = step_hook_callback(hooks, run, self._flow_errors)
        lib().psph_oracle_set_step_hooks(self._h, cb, None, sum(hooks))
        self._hook_cb = cb

    def use_step_hooks(self, dom):
        """A Domain's GeneralBefore / GeneralAfter (hook(domain)), each called on a
        shallow copy of dom holding the oracle's particles and Time."""
        def adapt(h):
            if h is None:
                return None

            def run(t, pset):
                view = copy.copy(dom)
                view.Time = t
                view.particles = pset
                h(view)
                return view.particles
            return run
        self.set_step_hooks(adapt(getattr(dom, "GeneralBefore", None)), adapt(getattr(dom, "GeneralAfter", None)))

    def patch(self, pset):
        arrs = {f: np.ascontiguousarray(pset.get(f)) for f in ALL_FIELDS if pset.has(f)}
        s = particles_struct(arrs, pset.n)
        st = lib().psph_oracle_patch(self._h, C.byref(s))
        if st:
            raise OracleError(f"patch: status {st}")

    def use_flow_hooks(self, dom):
        """Registers a Domain's user InCon / OutCon (None: the defaults)."""
        for which, hook in ((PSPH_FLOW_IN, getattr(dom, "InCon", None)), (PSPH_FLOW_OUT, getattr(dom, "OutCon", None))):
            if hook is not None:
                self.set_flow_profile(which, lambda x, h=hook, bc=dom.BC: h(x, bc))

    def __del__(self):
        self.close()

    def step(self, nsteps: int, nthreads: int = 1):
        st = lib().psph_oracle_step(self._h, nsteps, nthreads)
        if self._flow_errors:
            err = self._flow_errors[0]
            self._flow_errors.clear()
            raise err
        if st:
            raise OracleError(f"status {st}: {lib().psph_oracle_error(self._h).decode()}")

    @property
    def n(self) -> int:
        return lib().psph_oracle_num_particles(self._h)

    def download(self, fields=ALL_FIELDS) -> dict:
        n = self.n
        out = {f: np.zeros(field_shape(f, n), field_dtype(f)) for f in fields}
        s = particles_struct(out, n)
        lib().psph_oracle_download(self._h, C.byref(s))
        return out

    def original_index(self) -> np.ndarray:
        out = np.zeros(self.n, np.int64)
        lib().psph_oracle_original_index(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)))
        return out

    def grid(self) -> PsphGrid:
        g = PsphGrid()
        lib().psph_oracle_get_grid(self._h, C.byref(g))
        return g

    def integrator(self) -> PsphIntegrator:
        it = PsphIntegrator()
        lib().psph_oracle_get_integrator(self._h, C.byref(it))
        return it

    def pairs(self, which: int) -> np.ndarray:
        L = lib()
        cnt = L.psph_oracle_pairs(self._h, which, None, 0)
        buf = np.zeros((max(cnt, 1), 2), np.int64)
        L.psph_oracle_pairs(self._h, which, buf.ctypes.data_as(C.POINTER(C.c_int64)), cnt)
        return buf[:cnt]

    def scales(self):
        n = self.n
        a = np.zeros(n)
        d = np.zeros(n)
        lib().psph_oracle_scales(self._h, a.ctypes.data_as(C.POINTER(C.c_double)),
                                 d.ctypes.data_as(C.POINTER(C.c_double)))
        return a, d

    def pair_count(self) -> int:
        """In-support pairs evaluated by the pair forces since create."""
        return int(lib().psph_oracle_pair_count(self._h))

    def phase_times(self):
        buf = (C.c_double * 5)()
        lib().psph_oracle_phase_times(self._h, buf, 5)
        return list(buf)


# ---------------------------------------------------------------------------
# state directories (oracle/state_io.h layout) and the reference driver
# ---------------------------------------------------------------------------

def write_state_dir(path: str, cfg: PsphConfig, pset: ParticleSet, extra: dict | None = None) -> None:
    os.makedirs(path, exist_ok=True)
    for f in ALL_FIELDS:
        if pset.has(f):
            np.ascontiguousarray(pset.get(f)).tofile(os.path.join(path, f + ".bin"))
    lines = {
        "n": [pset.n], "dimension": [cfg.dimension], "kernel_type": [cfg.kernel_type], "vis_eq": [cfg.vis_eq],
        "gradient_type": [cfg.gradient_type], "scheme": [cfg.scheme], "periodic": list(cfg.periodic),
        "gravity": list(cfg.gravity), "body_force": list(cfg.body_force), "xsph": [cfg.xsph],
        "sqrt_h_a": [cfg.sqrt_h_a], "R": [cfg.R], "dom_max": list(cfg.dom_max), "dom_min": list(cfg.dom_min),
        "dt": [cfg.dt], "time": [cfg.time], "shepard_step": [cfg.shepard_step], "swi_type": [cfg.swi_type],
        "fsi": [cfg.fsi], "in_out_flow": [cfg.in_out_flow], "mass_conservation": [cfg.mass_conservation],
        "bc_cellfac": [cfg.bc_cellfac], "in_v": list(cfg.in_v), "in_density": [cfg.in_density],
        "out_v": list(cfg.out_v), "out_density": [cfg.out_density], "initial_dist": [cfg.initial_dist],
    }
    if extra:
        lines.update(extra)
    with open(os.path.join(path, "config.txt"), "w") as fh:
        for k, v in lines.items():
            fh.write(k + " " + " ".join(repr(float(x)) for x in v) + "\n")


def read_state_dir(path: str) -> tuple[dict, dict]:
    cfg = {}
    with open(os.path.join(path, "config.txt")) as fh:
        for line in fh:
            parts = line.split()
            cfg[parts[0]] = [float(x) for x in parts[1:]]
    n = int(cfg["n"][0])
    arrs = {}
    for f in ALL_FIELDS + ("cc",):
        p = os.path.join(path, f + ".bin")
        if os.path.exists(p):
            dt = np.float64 if f == "cc" else field_dtype(f)
            shape = (n, 3) if f == "cc" else field_shape(f, n)
            arrs[f] = np.fromfile(p, dtype=dt).reshape(shape)
    return cfg, arrs


def read_pairs_dir(path: str) -> dict:
    out = {}
    for k in ("sm", "fsm", "nsm"):
        p = os.path.join(path, k + ".bin")
        out[k] = np.fromfile(p, dtype=np.int64).reshape(-1, 2) if os.path.exists(p) else np.zeros((0, 2), np.int64)
    return out


def have_reference() -> bool:
    return os.path.exists(REF_DRIVER)


def run_reference(state_in: str, out_dir: str, nsteps: int, nproc: int, dumps) -> dict:
    """Runs the unmodified reference (oracle/_ref/ref_driver) on a state directory."""
    if not have_reference():
        raise OracleError("oracle/_ref/ref_driver is not built (needs the reference sources)")
    cmd = [REF_DRIVER, "run", state_in, out_dir, str(nsteps), str(nproc)] + [str(d) for d in dumps]
    env = dict(os.environ, OMP_NUM_THREADS=str(nproc))
    res = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env)
    last = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    return json.loads(last[-1]) if last else {}


def reference_box(out_dir: str, dim, tag, V, Lx, Ly, Lz, r, rho, h, type_, rot, random, fixed) -> dict:
    if not have_reference():
        raise OracleError("oracle/_ref/ref_driver is not built")
    args = [REF_DRIVER, "box", out_dir, str(dim), str(tag)] + [repr(float(v)) for v in V] + \
        [repr(float(v)) for v in (Lx, Ly, Lz, r, rho, h)] + [str(type_), str(rot), str(int(random)), str(int(fixed))]
    subprocess.run(args, check=True, capture_output=True)
    n = int(open(os.path.join(out_dir, "config.txt")).read().split()[1])
    return {
        "x": np.fromfile(os.path.join(out_dir, "x.bin"), np.float64).reshape(n, 3),
        "mass": np.fromfile(os.path.join(out_dir, "mass.bin"), np.float64),
    }
