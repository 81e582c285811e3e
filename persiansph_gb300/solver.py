"""Host side of one GPU domain: a thin owner of a psph_ctx (include/psph.h).

`GpuDomain` is what `Domain.Solve` drives and what the parity tests and the
benchmark call. Every call goes through the C ABI of the CUDA library; a
non-zero status raises `PsphError` (the reference throws `Fatal` there).
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np

from .abi import (ALL_FIELDS, NO_FLOW_FN, NO_HOOK_FN, PSPH_FLOW_IN, PSPH_FLOW_OUT, PSPH_HOOK_AFTER, PSPH_HOOK_BEFORE,
                  PsphConfig, PsphError, PsphGrid, PsphIntegrator, PsphTuning, field_dtype, field_shape, flow_callback,
                  load_library, particles_struct, step_hook_callback)
from .particles import ParticleSet


# the step phases psph_phase_times reports, in order
PHASES = ("sort", "nlist", "prepare", "forces", "closure", "dt", "update")

class GpuDomain:
    def __init__(self, cfg: PsphConfig, grid: PsphGrid | None = None, integ: PsphIntegrator | None = None):
        self._lib = load_library()
        self._ctx = C.c_void_p()
        self.cfg = cfg
        self._flow_cbs = {}
        self._flow_errors = []
        st = self._lib.psph_create(C.byref(cfg), C.byref(self._ctx))
        self._check(st)
        if grid is not None:
            self._check(self._lib.psph_set_grid(self._ctx, C.byref(grid)))
        if integ is not None:
            self._check(self._lib.psph_set_integrator(self._ctx, C.byref(integ)))
        self._uploaded = None

    def _check(self, st: int):
        if self._flow_errors:
            err = self._flow_errors[0]
            self._flow_errors.clear()
            raise err
        if st != 0:
            msg = self._lib.psph_last_error(self._ctx).decode() if self._ctx else ""
            raise PsphError(st, msg)

    def set_flow_profile(self, which: int, fn=None):
        """psph_set_flow_profile: fn(position) -> (velocity, density) replaces
        the in-flow (PSPH_FLOW_IN) or out-flow (PSPH_FLOW_OUT) constants of an
        in/out-flow domain, like a user InCon / OutCon; None restores them."""
        cb = flow_callback(fn, self._flow_errors) if fn is not None else NO_FLOW_FN
        self._check(self._lib.psph_set_flow_profile(self._ctx, int(which), cb, None))
        self._flow_cbs[which] = cb  # kept alive while the context may call it

    def set_step_hooks(self, before=None, after=None):
        """psph_set_step_hooks: host hooks inside every step, where the reference
        calls GeneralBefore (after the neighbour search) and GeneralAfter (after
        the forces). Each is hook(time, particles) with the particles downloaded
        into a ParticleSet; it changes them in place (or returns a replacement)
        and the result is written back with psph_patch. None removes a hook."""
        hooks = {}
        if before is not None:
            hooks[PSPH_HOOK_BEFORE] = before
        if after is not None:
            hooks[PSPH_HOOK_AFTER] = after
        if not hooks:
            self._check(self._lib.psph_set_step_hooks(self._ctx, NO_HOOK_FN, None, 0))
            self._hook_cb = None
            return

        def run(fn):
            pset = self.download()
            out = fn(self.time, pset)
            self.patch(out if out is not None else pset)

        cb = step_hook_callback(hooks, run, self._flow_errors)
        self._check(self._lib.psph_set_step_hooks(self._ctx, cb, None, sum(hooks)))
        self._hook_cb = cb  # kept alive while the context may call it

    def use_step_hooks(self, dom, live: bool = False):
        """Registers a Domain's GeneralBefore / GeneralAfter (hook(domain), the
        reference's form). The hook sees a Domain whose `particles` and `Time`
        are the context's at that point: `dom` itself when live (Solve), else a
        shallow copy, so the caller's Domain keeps its particles."""
        def adapt(h):
            if h is None:
                return None

            def run(t, pset):
                view = dom if live else copy.copy(dom)
                view.Time = t
                view.particles = pset
                h(view)
                return view.particles
            return run
        self.set_step_hooks(adapt(getattr(dom, "GeneralBefore", None)), adapt(getattr(dom, "GeneralAfter", None)))

    def patch(self, pset: ParticleSet):
        """psph_patch: writes the particles (psph_download's order) back."""
        arrs = {f: np.ascontiguousarray(pset.get(f)) for f in ALL_FIELDS if pset.has(f)}
        s = particles_struct(arrs, pset.n)
        self._check(self._lib.psph_patch(self._ctx, C.byref(s)))

    def use_flow_hooks(self, dom):
        """Registers a Domain's user InCon / OutCon (None: the defaults)."""
        for which, hook in ((PSPH_FLOW_IN, getattr(dom, "InCon", None)), (PSPH_FLOW_OUT, getattr(dom, "OutCon", None))):
            if hook is not None:
                self.set_flow_profile(which, lambda x, h=hook, bc=dom.BC: h(x, bc))

    def close(self):
        if self._ctx:
            self._lib.psph_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- data movement --------------------------------------------------------
    def upload(self, pset: ParticleSet, initial: bool = True):
        arrs = {f: np.ascontiguousarray(pset.get(f)) for f in ALL_FIELDS if pset.has(f)}
        for req in ("x", "h", "density", "mass"):
            if req not in arrs:
                arrs[req] = np.ascontiguousarray(pset.get(req))
        s = particles_struct(arrs, pset.n)
        self._check(self._lib.psph_upload(self._ctx, C.byref(s), int(initial)))
        self._uploaded = pset

    def step(self, nsteps: int, t_stop: float = float("inf")) -> int:
        done = C.c_int64(0)
        self._check(self._lib.psph_step(self._ctx, int(nsteps), float(t_stop), C.byref(done)))
        return done.value

    @property
    def n(self) -> int:
        return int(self._lib.psph_num_particles(self._ctx))

    def download_fields(self, fields=ALL_FIELDS) -> dict:
        n = self.n
        out = {f: np.zeros(field_shape(f, n), field_dtype(f)) for f in fields}
        s = particles_struct(out, n)
        self._check(self._lib.psph_download(self._ctx, C.byref(s)))
        return out

    def original_index(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.int64)
        self._check(self._lib.psph_original_index(self._ctx, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out[: self.n]

    def download(self, base: ParticleSet | None = None) -> ParticleSet:
        """Current state as a ParticleSet. Fields the device does not track for
        the chosen scheme keep their values from `base` (the uploaded set)."""
        base = base if base is not None else self._uploaded
        fields = self.download_fields()
        keep = self.original_index()
        out = ParticleSet(len(keep))
        for f in ALL_FIELDS:
            arr = fields[f]
            if base is not None and base.has(f) and self._untracked(f):
                # fields the device does not keep come from the uploaded set
                # (particles an in/out-flow boundary appended have none: zero)
                src = base.get(f)
                arr = np.zeros_like(arr)
                old = keep < src.shape[0]
                arr[old] = src[keep[old]]
            out._arr[f] = np.ascontiguousarray(arr)
        return out

    def _untracked(self, f: str) -> bool:
        if f in ("k", "k2"):  # permeabilities are read on upload only
            return True
        lf = self.cfg.scheme == 1
        if lf:
            return False
        return f in ("va", "densitya", "sigmaa", "straina", "shear_stressa")

    def pairs(self, which: int) -> np.ndarray:
        total = C.c_int64(0)
        self._check(self._lib.psph_pairs_export(self._ctx, which, None, 0, C.byref(total)))
        buf = np.zeros((max(total.value, 1), 2), np.int64)
        self._check(self._lib.psph_pairs_export(self._ctx, which, buf.ctypes.data_as(C.POINTER(C.c_int64)),
                                                total.value, C.byref(total)))
        return buf[: total.value]

    def grid(self) -> PsphGrid:
        g = PsphGrid()
        self._check(self._lib.psph_get_grid(self._ctx, C.byref(g)))
        return g

    def integrator(self) -> PsphIntegrator:
        it = PsphIntegrator()
        self._check(self._lib.psph_get_integrator(self._ctx, C.byref(it)))
        return it

    @property
    def time(self) -> float:
        return self.integrator().time

    def enable_timing(self, on: bool = True):
        self._check(self._lib.psph_enable_timing(self._ctx, int(on)))

    def phase_times(self):
        """Device ms of the last step call's phases (timing enabled), keyed by
        PHASES."""
        buf = (C.c_double * len(PHASES))()
        n = C.c_int(0)
        self._check(self._lib.psph_phase_times(self._ctx, buf, len(buf), C.byref(n)))
        return dict(zip(PHASES, list(buf)[: n.value]))

    def step_timed(self, nsteps: int):
        ms = C.c_double(0.0)
        done = C.c_int64(0)
        self._check(self._lib.psph_step_timed(self._ctx, int(nsteps), C.byref(ms), C.byref(done)))
        return ms.value, done.value

    # -- snapshot output (WriteXDMF, Source/Domain.cpp:1869-2064) ------------
    @staticmethod
    def _names(names):
        names = list(names) if names else []
        return (C.c_char_p * 3)(*[(names[k].encode() if k < len(names) and names[k] else None) for k in range(3)])

    def request_output(self, file_key: str, names=None):
        """The next step writes <file_key>.bin / .xmf after its forces (Solve's
        output point); the copy and the write overlap the following steps."""
        self._check(self._lib.psph_output_request(self._ctx, file_key.encode(), self._names(names)))

    def write_output(self, file_key: str, names=None, props=None):
        """Writes a snapshot of the current state now; props: up to three arrays
        (psph_download order) of UserOutput properties, zeros by default."""
        arrs = [None, None, None]
        keep = []
        for k, p in enumerate(props or []):
            if p is None:
                continue
            a = np.ascontiguousarray(p, dtype=np.float64)
            keep.append(a)
            arrs[k] = a.ctypes.data_as(C.POINTER(C.c_double))
        self._check(self._lib.psph_output_write(self._ctx, file_key.encode(), self._names(names), *arrs))

    def flush_output(self):
        """Waits until every requested snapshot is on disk."""
        self._check(self._lib.psph_output_flush(self._ctx))

    def pair_count(self) -> int:
        v = C.c_uint64(0)
        self._check(self._lib.psph_pair_count(self._ctx, C.byref(v)))
        return int(v.value)

    def last_launch_count(self) -> int:
        return int(self._lib.psph_last_launch_count(self._ctx))


class GpuEnsemble:
    """Many independent domains in one context (psph_batch_*): one launch
    sequence per step serves all instances; each keeps its own grid, time step
    and stop time. Instance q's particles are indexed as uploaded."""

    def __init__(self, cfgs):
        self._lib = load_library()
        self._ctx = C.c_void_p()
        self.cfgs = list(cfgs)
        arr = (PsphConfig * len(self.cfgs))(*self.cfgs)
        self._keep = arr
        self._check(self._lib.psph_batch_create(arr, len(self.cfgs), C.byref(self._ctx)))
        self._uploaded = None

    def _check(self, st: int):
        if st != 0:
            msg = self._lib.psph_last_error(self._ctx).decode() if self._ctx else ""
            raise PsphError(st, msg)

    def close(self):
        if self._ctx:
            self._lib.psph_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def size(self) -> int:
        return int(self._lib.psph_batch_size(self._ctx))

    def upload(self, psets, initial: bool = True):
        structs, hold = [], []
        for pset in psets:
            arrs = {f: np.ascontiguousarray(pset.get(f)) for f in ALL_FIELDS if pset.has(f)}
            for req in ("x", "h", "density", "mass"):
                if req not in arrs:
                    arrs[req] = np.ascontiguousarray(pset.get(req))
            hold.append(arrs)
            structs.append(particles_struct(arrs, pset.n))
        arr = (type(structs[0]) * len(structs))(*structs)
        self._check(self._lib.psph_batch_upload(self._ctx, arr, int(initial)))
        self._uploaded = list(psets)

    def step(self, nsteps: int, t_stop=None) -> np.ndarray:
        k = len(self.cfgs)
        done = np.zeros(k, np.int64)
        ts = None
        if t_stop is not None:
            ts = np.ascontiguousarray(np.broadcast_to(np.asarray(t_stop, np.float64), (k,)))
        self._check(self._lib.psph_batch_step(
            self._ctx, int(nsteps), ts.ctypes.data_as(C.POINTER(C.c_double)) if ts is not None else None,
            done.ctypes.data_as(C.POINTER(C.c_int64))))
        return done

    def n(self, q: int) -> int:
        return int(self._lib.psph_batch_num_particles(self._ctx, q))

    def download_fields(self, q: int, fields=ALL_FIELDS) -> dict:
        n = self.n(q)
        out = {f: np.zeros(field_shape(f, n), field_dtype(f)) for f in fields}
        s = particles_struct(out, n)
        self._check(self._lib.psph_batch_download(self._ctx, q, C.byref(s)))
        return out

    def original_index(self, q: int) -> np.ndarray:
        n = self.n(q)
        out = np.zeros(max(n, 1), np.int64)
        self._check(self._lib.psph_batch_original_index(self._ctx, q, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out[:n]

    def grid(self, q: int) -> PsphGrid:
        g = PsphGrid()
        self._check(self._lib.psph_batch_get_grid(self._ctx, q, C.byref(g)))
        return g

    def integrator(self, q: int) -> PsphIntegrator:
        it = PsphIntegrator()
        self._check(self._lib.psph_batch_get_integrator(self._ctx, q, C.byref(it)))
        return it

    def enable_timing(self, on: bool = True):
        self._check(self._lib.psph_enable_timing(self._ctx, int(on)))

    def phase_times(self):
        """Device ms of the last step call's phases (timing enabled), keyed by
        PHASES."""
        buf = (C.c_double * len(PHASES))()
        n = C.c_int(0)
        self._check(self._lib.psph_phase_times(self._ctx, buf, len(buf), C.byref(n)))
        return dict(zip(PHASES, list(buf)[: n.value]))

    def step_timed(self, nsteps: int):
        ms = C.c_double(0.0)
        done = C.c_int64(0)
        self._check(self._lib.psph_step_timed(self._ctx, int(nsteps), C.byref(ms), C.byref(done)))
        return ms.value, done.value

    def pair_count(self) -> int:
        v = C.c_uint64(0)
        self._check(self._lib.psph_pair_count(self._ctx, C.byref(v)))
        return int(v.value)

    def last_launch_count(self) -> int:
        return int(self._lib.psph_last_launch_count(self._ctx))


def _attach_closure(self, net, dx: float):
    """Learned eddy viscosity for the LES particles of this context (see
    persiansph_gb300.closure)."""
    self._check(self._lib.psph_closure_attach(self._ctx, net.handle, float(dx)))
    self._closure = net


def _closure_stats(self):
    ev, fb = C.c_uint64(0), C.c_uint64(0)
    self._check(self._lib.psph_closure_stats(self._ctx, C.byref(ev), C.byref(fb)))
    return int(ev.value), int(fb.value)


def _closure_features(self):
    n = self.n if isinstance(self.n, int) else self.n(0)
    out = np.zeros((max(n, 1), 6), np.float32)
    self._check(self._lib.psph_closure_features(self._ctx, out.ctypes.data_as(C.POINTER(C.c_float))))
    return out[:n]


def _workload_key(self) -> str:
    """Signature of the workload a tuning result belongs to: the switches that
    select kernels and the particle count (to the nearest 2^k)."""
    cfg = self.cfg if hasattr(self, "cfg") else self.cfgs[0]
    n = self.n if isinstance(self.n, int) else sum(self.n(q) for q in range(len(self.cfgs)))
    return (f"dim{cfg.dimension}-kt{cfg.kernel_type}-vis{cfg.vis_eq}-grad{cfg.gradient_type}-"
            f"prec{cfg.precision}-per{int(any(cfg.periodic))}-inst{1 if hasattr(self, 'cfg') else len(self.cfgs)}-"
            f"n2^{max(int(n), 1).bit_length()}-closure{int(getattr(self, '_closure', None) is not None)}")


def _autotune(self, steps_per_trial: int = 5, cache: str | None = None) -> dict:
    """psph_autotune: times every candidate launch setting on this context's
    own steps (which advance the simulation) and keeps the fastest. With
    `cache` (a JSON file), a setting stored for the same workload signature is
    applied without trials, and a new result is stored there."""
    import json
    import os
    key = _workload_key(self)
    if cache and os.path.exists(cache):
        try:
            known = json.load(open(cache))
        except (OSError, ValueError):
            known = {}
        if key in known:
            t = known[key]
            self.set_tuning(t["pair_block"], t["cell_split"], t.get("nlist_stage", 0), t.get("skin_permille", 0))
            return dict(t, cached=True)
    t = PsphTuning()
    self._check(self._lib.psph_autotune(self._ctx, int(steps_per_trial), C.byref(t)))
    out = {"pair_block": t.pair_block, "cell_split": t.cell_split, "nlist_stage": t.nlist_stage,
           "skin_permille": t.skin_permille, "ms_per_step": t.ms_per_step}
    if cache:
        known = {}
        if os.path.exists(cache):
            try:
                known = json.load(open(cache))
            except (OSError, ValueError):
                known = {}
        known[key] = out
        with open(cache, "w") as f:
            json.dump(known, f, indent=1, sort_keys=True)
    return out


def _tuning(self) -> dict:
    t = PsphTuning()
    self._check(self._lib.psph_get_tuning(self._ctx, C.byref(t)))
    return {"pair_block": t.pair_block, "cell_split": t.cell_split, "nlist_stage": t.nlist_stage,
            "skin_permille": t.skin_permille, "ms_per_step": t.ms_per_step}


def _set_tuning(self, pair_block: int = 128, cell_split: int = 1, nlist_stage: int | None = None,
                skin_permille: int | None = None):
    """Launch setting; nlist_stage / skin_permille None keep the context's
    staging depth / list skin (thousandths of the support, FP32C form)."""
    cur = PsphTuning()
    self._check(self._lib.psph_get_tuning(self._ctx, C.byref(cur)))
    if nlist_stage is None:
        nlist_stage = cur.nlist_stage
    if skin_permille is None:
        skin_permille = cur.skin_permille
    t = PsphTuning(pair_block, cell_split, nlist_stage, skin_permille, 0.0)
    self._check(self._lib.psph_set_tuning(self._ctx, C.byref(t)))


def _list_rebuilds(self) -> int:
    """Steps since upload that ran the cell sort and the neighbour lists."""
    return int(self._lib.psph_list_rebuilds(self._ctx))


for _cls in (GpuDomain, GpuEnsemble):
    _cls.autotune = _autotune
    _cls.tuning = _tuning
    _cls.set_tuning = _set_tuning
    _cls.list_rebuilds = _list_rebuilds
    _cls.attach_closure = _attach_closure
    _cls.closure_stats = _closure_stats
    _cls.closure_features = _closure_features
