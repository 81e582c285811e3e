"""Learned eddy-viscosity closure: host side of the psph_mlp_* / psph_closure_*
calls (include/psph.h).

`ClosureNet` owns one network on the GPU: seeded initial weights, the training
set, Adam training by the library's own forward/backward kernels, inference
on the tensor cores, and save/load of the weights. A trained network goes into
a simulation with `GpuDomain.attach_closure(net, dx)`: every LES fluid particle
then takes its eddy viscosity from the network instead of the Smagorinsky term
of Mat1 (Source/Particle.cpp:157-160), which stays as the fallback for inputs
outside the training range.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import PsphError, load_library

NIN = 6
NPARAMS = 8833
NNORM = 24
# shear rate and vorticity enter in units of the acoustic rate Cs / h
FEATURES = ("log_shear_rate_h_over_cs", "strain_rate_r3", "log_vorticity_h_over_cs", "density_ratio", "h_over_dx",
            "neighbours")


def default_network_path() -> str:
    """The network shipped with the package: trained by
    `python -m persiansph_gb300.closure_train --steps 6000` (eight fine plain
    runs at dx = 10 mm box-filtered to dx = 20 mm; its report lies beside it)."""
    import os
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "closure_dam3d.npz")


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class ClosureNet:
    def __init__(self, seed: int = 0):
        self._lib = load_library()
        self._h = C.c_void_p()
        self._check(self._lib.psph_mlp_create(C.c_uint64(seed), C.byref(self._h)))

    def _check(self, st: int):
        if st != 0:
            msg = self._lib.psph_mlp_last_error(self._h).decode() if self._h else ""
            raise PsphError(st, msg)

    def close(self):
        if self._h:
            self._lib.psph_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- parameters --------------------------------------------------------------
    def get(self):
        p = np.zeros(NPARAMS, np.float32)
        nrm = np.zeros(NNORM, np.float32)
        self._check(self._lib.psph_mlp_get_params(self._h, _fp(p), _fp(nrm)))
        return p, nrm

    def set(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        nrm = None if norm is None else np.ascontiguousarray(norm, np.float32)
        self._check(self._lib.psph_mlp_set_params(self._h, _fp(p) if p is not None else None,
                                                  _fp(nrm) if nrm is not None else None))

    def save(self, path: str, **meta):
        p, nrm = self.get()
        np.savez(path, params=p, norm=nrm, **meta)

    @classmethod
    def load(cls, path: str) -> "ClosureNet":
        d = np.load(path)
        net = cls(0)
        net.set(d["params"], d["norm"])
        return net

    # -- training ------------------------------------------------------------------
    def set_data(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, NIN)
        y = np.ascontiguousarray(y, np.float32).reshape(-1)
        assert len(x) == len(y)
        self._check(self._lib.psph_mlp_set_data(self._h, _fp(x), _fp(y), len(y)))

    def set_weights(self, w=None):
        """Per-sample loss weights of the training set (None: uniform)."""
        if w is None:
            self._check(self._lib.psph_mlp_set_weights(self._h, None))
            return
        w = np.ascontiguousarray(w, np.float32).reshape(-1)
        self._check(self._lib.psph_mlp_set_weights(self._h, _fp(w)))

    def train(self, steps: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(max(steps, 1), np.float32)
        self._check(self._lib.psph_mlp_train(self._h, int(steps), int(batch), float(lr), C.c_uint64(seed),
                                             _fp(losses)))
        return losses[:steps]

    def loss_grad(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, NIN)
        y = np.ascontiguousarray(y, np.float32).reshape(-1)
        g = np.zeros(NPARAMS, np.float32)
        loss = C.c_double(0.0)
        self._check(self._lib.psph_mlp_loss_grad(self._h, _fp(x), _fp(y), len(y), C.byref(loss), _fp(g)))
        return loss.value, g

    def infer(self, x, tensor_cores: bool = True) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, NIN)
        c = np.zeros(len(x), np.float32)
        self._check(self._lib.psph_mlp_infer(self._h, _fp(x), len(x), _fp(c), int(tensor_cores)))
        return c


# ---------------------------------------------------------------------------
# training data from fine runs of the plain method
# ---------------------------------------------------------------------------
def les_case(dx, aspect=None, c0=40.0, L=0.3, H=None, W=1.0, TL=1.6, TH=1.0, TW=1.0):
    """3D dam break with the LES option on (CSmag 0.17): an L x H x W column,
    H = aspect * L unless given, in a TL x TH x TW tank."""
    from . import scenarios
    H = aspect * L if H is None else H
    dom, dt, info = scenarios.dam_break_3d(dx=dx, L=L, H=H, W=W, TL=TL, TH=TH, TW=TW, c0=c0)
    p = dom.particles
    p.set("les", 1)
    p.set("csmag", 0.17)
    info.update({"dx": dx, "L": L, "H": H, "W": W, "TL": TL, "TH": TH, "TW": TW, "c0": c0})
    return dom, dt, info


def fine_snapshots(cases, dx_f, times, precision=1):
    """Runs the cases (dicts of les_case arguments) as one ensemble at lattice
    spacing dx_f and returns, per case, the fluid state at each time:
    [{"t", "x", "v", "density"}...]."""
    from .solver import GpuEnsemble
    doms = [les_case(dx_f, **c) for c in cases]
    cfgs = []
    for dom, dt, _ in doms:
        cfg = dom.config(dt)
        cfg.precision = precision
        cfgs.append(cfg)
    ens = GpuEnsemble(cfgs)
    ens.upload([d.particles for d, _, _ in doms], initial=True)
    out = [[] for _ in cases]
    for t in times:
        ens.step(1 << 30, t_stop=np.full(len(cases), t))
        for q in range(len(cases)):
            f = ens.download_fields(q, ("x", "v", "density", "is_free"))
            fl = f["is_free"] == 1
            out[q].append({"t": ens.integrator(q).time, "x": f["x"][fl], "v": f["v"][fl],
                           "density": f["density"][fl]})
    ens.close()
    return out, [info for _, _, info in doms]


def box_filter(x, v, rho, dx_c):
    """Box filter of a particle field onto the cells of a dx_c lattice: per
    occupied cell its centre, particle count, mean velocity, mean density and
    the subgrid stress tau = mean(v v) - mean(v) mean(v) (xx, yy, zz, xy, xz, yz)."""
    ijk = np.floor(x / dx_c).astype(np.int64)
    keys, inv = np.unique(ijk, axis=0, return_inverse=True)
    inv = inv.ravel()
    cnt = np.bincount(inv).astype(np.float64)
    mean = lambda a: np.bincount(inv, weights=a) / cnt
    ub = np.stack([mean(v[:, d]) for d in range(3)], 1)
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    tau = np.stack([mean(v[:, a] * v[:, b]) - ub[:, a] * ub[:, b] for a, b in pairs], 1)
    return {"centre": (keys + 0.5) * dx_c, "count": cnt, "v": ub, "density": mean(rho), "tau": tau}


def coarse_from_filter(case, dx_c, filt, occupancy):
    """Particle set of the coarse lattice: the coarse case's walls plus one fluid
    particle per cell with at least `occupancy` of its fine lattice sites
    filled, carrying the filtered velocity and density."""
    from .particles import ParticleSet
    dom, dt, info = les_case(dx_c, **case)
    p = dom.particles
    wall = p.get("is_free") == 0
    tmpl = int(np.flatnonzero(~wall)[0])
    keep = filt["count"] >= occupancy
    nf = int(keep.sum())
    out = ParticleSet(int(wall.sum()) + nf)
    for name, arr in p.arrays().items():
        out._arr[name] = np.ascontiguousarray(np.concatenate([arr[wall], np.repeat(arr[tmpl:tmpl + 1], nf, 0)]))
    nw = int(wall.sum())
    out.get("x")[nw:] = filt["centre"][keep]
    out.get("v")[nw:] = filt["v"][keep]
    out.get("vb")[nw:] = filt["v"][keep]
    out.get("density")[nw:] = filt["density"][keep]
    out.get("densityb")[nw:] = filt["density"][keep]
    return out, dom.config(dt), nw, keep


def closure_samples(cset, cfg, dx_c, nw, tau, net=None, precision=1, s_min=1e-3, c_max=1.0):
    """Features of the coarse particles from one step of the runtime kernels,
    and the target coefficient c* = nu*/(h^2 ShearRate) with nu* the eddy
    viscosity that best matches the filtered subgrid stress,
    nu* = max(0, -tau_dev : D / (2 D : D)), D = StrainRate / 2."""
    from .solver import GpuDomain
    cfg.precision = precision
    gd = GpuDomain(cfg)
    gd.upload(cset, initial=True)
    gd.attach_closure(net if net is not None else ClosureNet(0), dx_c)
    gd.step(1)
    feats = gd.closure_features()[nw:]
    sr = gd.download_fields(("strain_rate",))["strain_rate"][nw:].reshape(-1, 3, 3)
    gd.close()
    D = 0.5 * sr
    T = np.zeros_like(D)
    for k, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
        T[:, a, b] = tau[:, k]
        T[:, b, a] = tau[:, k]
    Tdev = T - np.trace(T, axis1=1, axis2=2)[:, None, None] / 3.0 * np.eye(3)
    dd = np.einsum("nij,nij->n", D, D)
    td = np.einsum("nij,nij->n", Tdev, D)
    shear = np.sqrt(2.0 * dd)
    h = cset.get("h")[nw:]
    with np.errstate(divide="ignore", invalid="ignore"):
        nu = np.maximum(0.0, -td / (2.0 * dd))
        c = nu / (h * h * shear)
    ok = (shear > s_min) & np.isfinite(c)
    return feats[ok], np.minimum(c[ok], c_max).astype(np.float32), {"h": h[ok], "shear": shear[ok], "nu": nu[ok]}


def dataset(cases, dx_f, dx_c, times, precision=1):
    """(features, targets, per-sample h and shear, case index) over the cases'
    snapshots."""
    snaps, infos = fine_snapshots(cases, dx_f, times, precision)
    m3 = round(dx_c / dx_f) ** 3
    X, Y, H, S, C = [], [], [], [], []
    for q, case in enumerate(cases):
        for sn in snaps[q]:
            filt = box_filter(sn["x"], sn["v"], sn["density"], dx_c)
            cset, cfg, nw, keep = coarse_from_filter(case, dx_c, filt, 0.5 * m3)
            x, y, aux = closure_samples(cset, cfg, dx_c, nw, filt["tau"][keep], precision=precision)
            X.append(x); Y.append(y); H.append(aux["h"]); S.append(aux["shear"]); C.append(np.full(len(y), q))
    return np.concatenate(X), np.concatenate(Y), np.concatenate(H), np.concatenate(S), np.concatenate(C)


def apriori_errors(net, x, y, h, shear, c_const=None, csmag=0.17):
    """Relative L2 errors of the eddy viscosity against the filtered target for
    the network, the Smagorinsky model of Mat1 (nu = (CSmag h)^2 SBar,
    SBar = 2 ShearRate) and, if given, a constant coefficient."""
    nu_t = y.astype(np.float64) * h * h * shear
    norm = np.linalg.norm(nu_t)
    c_net = net.infer(x, tensor_cores=True).astype(np.float64)
    out = {"network": float(np.linalg.norm(c_net * h * h * shear - nu_t) / norm),
           "smagorinsky": float(np.linalg.norm((csmag * h) ** 2 * 2.0 * shear - nu_t) / norm)}
    if c_const is not None:
        out["constant"] = float(np.linalg.norm(c_const * h * h * shear - nu_t) / norm)
    return out
