"""Host-side particle storage: structure-of-arrays mirror of SPH::Particle.

The reference keeps one heap object per particle (Source/Particle.h:29-149).
Here the same fields live in numpy arrays, one per field, created on first
write; unwritten fields read as the Particle constructor's defaults
(Source/Particle.cpp:25-117). `Particle` gives the reference's per-object
attribute names (`dom.Particles[i].Density = ...`) as views into the arrays.
"""
from __future__ import annotations

import numpy as np

from .abi import ALL_FIELDS, F64_FIELDS, INT_FIELDS, TEN_FIELDS, VEC_FIELDS, field_dtype, field_shape

# Particle constructor defaults that are not zero (Source/Particle.cpp:25-117).
DEFAULTS = {"is_free": 1, "fpmassc": 1.0, "bingham_m": 300.0, "csmag": 0.17, "tin": 4.0}

# Reference attribute name -> field name.
REF_NAMES = {
    "ID": "id", "Material": "material", "IsFree": "is_free", "NoSlip": "no_slip", "PresEq": "pres_eq",
    "Shepard": "shepard", "LES": "les", "VisM": "vis_m", "Fail": "fail", "x": "x", "v": "v", "va": "va",
    "vb": "vb", "a": "a", "NSv": "nsv", "VXSPH": "vxsph", "Density": "density", "Densitya": "densitya",
    "Densityb": "densityb", "dDensity": "ddensity", "Pressure": "pressure", "Mass": "mass", "h": "h",
    "Cs": "cs", "P0": "p0", "RefDensity": "ref_density", "FPMassC": "fpmassc", "Alpha": "alpha",
    "Beta": "beta", "Mu": "mu", "MuRef": "mu_ref", "T0": "t0", "m": "bingham_m", "CSmag": "csmag",
    "TI": "ti", "TIn": "tin", "TIInitDist": "ti_init_dist", "G": "g_mod", "K": "k_mod", "Sigmay": "sigmay",
    "c": "cohesion", "phi": "phi", "psi": "psi", "ZWab": "zwab", "SumDen": "sumden",
    "SumKernel": "sumkernel", "ShearRate": "shear_rate", "SBar": "sbar", "Sigma": "sigma",
    "Sigmaa": "sigmaa", "Sigmab": "sigmab", "ShearStress": "shear_stress", "ShearStressa": "shear_stressa",
    "ShearStressb": "shear_stressb", "Strain": "strain", "Straina": "straina", "Strainb": "strainb",
    "StrainRate": "strain_rate", "RotationRate": "rotation_rate", "TIR": "tir",
    "SeepageType": "seepage_type", "VarPorosity": "var_porosity", "IsSat": "is_sat", "n0": "n0", "k": "k",
    "k2": "k2", "d": "d", "RhoF": "rho_f", "V": "volume", "S": "s", "InOut": "in_out",
}


class ParticleSet:
    """Lazily materialised SoA particle arrays."""

    def __init__(self, n: int = 0):
        self.n = int(n)
        self._arr: dict[str, np.ndarray] = {}

    # -- storage -------------------------------------------------------------
    def has(self, name: str) -> bool:
        return name in self._arr

    def get(self, name: str) -> np.ndarray:
        """Array for `name`, created with defaults on first access."""
        arr = self._arr.get(name)
        if arr is None:
            arr = np.zeros(field_shape(name, self.n), dtype=field_dtype(name))
            if name in DEFAULTS:
                arr[...] = DEFAULTS[name]
            if name == "ref_density" and "density" in self._arr:
                arr[...] = self._arr["density"]
            self._arr[name] = arr
        return arr

    def set(self, name: str, values) -> None:
        if name not in ALL_FIELDS:
            raise KeyError(name)
        arr = self.get(name)
        arr[...] = values

    def arrays(self) -> dict:
        return self._arr

    def materialize(self, names=ALL_FIELDS) -> dict:
        return {f: self.get(f) for f in names}

    # -- growth / deletion ----------------------------------------------------
    def append(self, n_new: int, fields: dict) -> None:
        """Appends n_new particles; `fields` gives arrays for some fields."""
        old = self.n
        total = old + n_new
        names = set(self._arr) | set(fields)
        if "density" in fields and "ref_density" not in fields:
            # RefDensity = Density0 at construction (Source/Particle.cpp:64)
            fields = dict(fields)
            fields["ref_density"] = fields["density"]
            names.add("ref_density")
        prev = dict(self._arr)
        for name in names:
            new = np.zeros(field_shape(name, total), dtype=field_dtype(name))
            if name in DEFAULTS:
                new[...] = DEFAULTS[name]
            if name in prev:
                new[:old] = prev[name]
            elif name == "ref_density" and "density" in prev:
                new[:old] = prev["density"]
            if name in fields:
                new[old:] = fields[name]
            self._arr[name] = new
        self.n = total

    def keep(self, mask: np.ndarray) -> None:
        """Keeps particles where mask is true, preserving order (Array::DelItems)."""
        for name in list(self._arr):
            self._arr[name] = np.ascontiguousarray(self._arr[name][mask])
        self.n = int(np.count_nonzero(mask))

    def copy(self) -> "ParticleSet":
        out = ParticleSet(self.n)
        out._arr = {k: v.copy() for k, v in self._arr.items()}
        return out


class Particle:
    """Per-particle view with the reference's attribute names."""

    __slots__ = ("_set", "_i")

    def __init__(self, pset: ParticleSet, i: int):
        object.__setattr__(self, "_set", pset)
        object.__setattr__(self, "_i", i)

    def __getattr__(self, ref_name):
        f = REF_NAMES.get(ref_name)
        if f is None:
            raise AttributeError(ref_name)
        v = self._set.get(f)[self._i]
        if f in INT_FIELDS:
            return bool(v) if f in ("is_free", "no_slip", "shepard", "les", "var_porosity", "is_sat") else int(v)
        return v if (f in VEC_FIELDS or f in TEN_FIELDS) else float(v)

    def __setattr__(self, ref_name, value):
        f = REF_NAMES.get(ref_name)
        if f is None:
            raise AttributeError(ref_name)
        self._set.get(f)[self._i] = value


class ParticleList:
    """Sequence view of Domain::Particles."""

    def __init__(self, pset: ParticleSet):
        self._set = pset

    def __len__(self):
        return self._set.n

    def Size(self):
        return self._set.n

    def __getitem__(self, i):
        if i < 0:
            i += self._set.n
        if not 0 <= i < self._set.n:
            raise IndexError(i)
        return Particle(self._set, i)

    def __iter__(self):
        for i in range(self._set.n):
            yield Particle(self._set, i)


__all__ = ["ParticleSet", "Particle", "ParticleList", "REF_NAMES", "DEFAULTS", "F64_FIELDS"]
