"""ctypes mirror of the C ABI in include/psph.h.

The structures here must match include/psph.h field for field; the ABI tests
check the sizes against the compiled library. `load_library()` loads the CUDA
library built in-tree by `persiansph_gb300.build` and fails loudly when it is
missing: there is no CPU fallback behind this API.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

# Field lists in include/psph.h order.
BASE_INT_FIELDS = ("id", "material", "is_free", "no_slip", "pres_eq", "shepard", "les", "vis_m", "fail")
VEC_FIELDS = ("x", "v", "va", "vb", "a", "nsv", "vxsph")
BASE_F64_FIELDS = (
    "density", "densitya", "densityb", "ddensity", "pressure", "mass", "h", "cs", "p0", "ref_density",
    "fpmassc", "alpha", "beta", "mu", "mu_ref", "t0", "bingham_m", "csmag", "ti", "tin", "ti_init_dist",
    "g_mod", "k_mod", "sigmay", "cohesion", "phi", "psi", "zwab", "sumden", "sumkernel", "shear_rate", "sbar",
)
TEN_FIELDS = (
    "sigma", "sigmaa", "sigmab", "shear_stress", "shear_stressa", "shear_stressb", "strain", "straina",
    "strainb", "strain_rate", "rotation_rate", "tir",
)
# soil-water interaction fields, after the tensors in the struct
SEEP_INT_FIELDS = ("seepage_type", "var_porosity", "is_sat")
SEEP_F64_FIELDS = ("n0", "k", "k2", "d", "rho_f", "volume", "s")
FLOW_INT_FIELDS = ("in_out",)
INT_FIELDS = BASE_INT_FIELDS + SEEP_INT_FIELDS + FLOW_INT_FIELDS
F64_FIELDS = BASE_F64_FIELDS + SEEP_F64_FIELDS
ALL_FIELDS = INT_FIELDS + VEC_FIELDS + F64_FIELDS + TEN_FIELDS

# status codes (psph_status)
PSPH_OK = 0
# psph_set_flow_profile: which hook (Domain::InCon / OutCon) and the C callback type
PSPH_FLOW_IN, PSPH_FLOW_OUT = 1, 2
FlowFn = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)
# psph_set_step_hooks: where a hook runs (Domain::GeneralBefore / GeneralAfter) and the C callback type
PSPH_HOOK_BEFORE, PSPH_HOOK_AFTER = 1, 2
HookFn = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_void_p)
STATUS_NAMES = {
    0: "PSPH_OK", 1: "PSPH_ERR_INVALID_ARGUMENT", 2: "PSPH_ERR_UNSUPPORTED", 3: "PSPH_ERR_CUDA",
    4: "PSPH_ERR_OUT_OF_MEMORY", 5: "PSPH_ERR_NONFINITE", 6: "PSPH_ERR_DT_COLLAPSE", 7: "PSPH_ERR_CFL",
    8: "PSPH_ERR_CELL_OVERFLOW", 9: "PSPH_ERR_NO_DEVICE", 10: "PSPH_ERR_STATE", 11: "PSPH_ERR_NOT_FOUND",
}


class PsphConfig(C.Structure):
    _fields_ = [
        ("dimension", C.c_int32), ("kernel_type", C.c_int32), ("vis_eq", C.c_int32),
        ("gradient_type", C.c_int32), ("scheme", C.c_int32), ("periodic", C.c_int32 * 3),
        ("swi_type", C.c_int32), ("shepard_step", C.c_int32), ("precision", C.c_int32),
        ("wall_pressure_mode", C.c_int32), ("gravity", C.c_double * 3), ("body_force", C.c_double * 3),
        ("xsph", C.c_double), ("sqrt_h_a", C.c_double), ("R", C.c_double), ("dom_max", C.c_double * 3),
        ("dom_min", C.c_double * 3), ("dt", C.c_double), ("time", C.c_double), ("fsi", C.c_int32),
        ("in_out_flow", C.c_int32), ("mass_conservation", C.c_int32), ("reserved", C.c_int32 * 5),
        ("initial_dist", C.c_double), ("bc_cellfac", C.c_double), ("in_v", C.c_double * 3),
        ("in_density", C.c_double), ("out_v", C.c_double * 3), ("out_density", C.c_double),
    ]


class PsphGrid(C.Structure):
    _fields_ = [
        ("blpf", C.c_double * 3), ("trpr", C.c_double * 3), ("cell_size", C.c_double * 3),
        ("dom_size", C.c_double * 3), ("hmax", C.c_double), ("rhomax", C.c_double), ("cellfac", C.c_double),
        ("cell_no", C.c_int32 * 3), ("pad", C.c_int32),
    ]


class PsphIntegrator(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("deltat", C.c_double), ("deltatint", C.c_double), ("deltatmin", C.c_double),
        ("steps", C.c_int64), ("first_step", C.c_int32), ("ct", C.c_int32), ("shepard_counter", C.c_int32),
        ("pad", C.c_int32),
    ]


class PsphTuning(C.Structure):
    _fields_ = [("pair_block", C.c_int32), ("cell_split", C.c_int32), ("nlist_stage", C.c_int32),
                ("skin_permille", C.c_int32), ("ms_per_step", C.c_double)]


class PsphParticles(C.Structure):
    _fields_ = (
        [("n", C.c_int64)]
        + [(f, C.POINTER(C.c_int32)) for f in BASE_INT_FIELDS]
        + [(f, C.POINTER(C.c_double)) for f in VEC_FIELDS]
        + [(f, C.POINTER(C.c_double)) for f in BASE_F64_FIELDS]
        + [(f, C.POINTER(C.c_double)) for f in TEN_FIELDS]
        + [(f, C.POINTER(C.c_int32)) for f in SEEP_INT_FIELDS]
        + [(f, C.POINTER(C.c_double)) for f in SEEP_F64_FIELDS]
        + [(f, C.POINTER(C.c_int32)) for f in FLOW_INT_FIELDS]
    )


def field_shape(name: str, n: int):
    if name in VEC_FIELDS:
        return (n, 3)
    if name in TEN_FIELDS:
        return (n, 3, 3)
    return (n,)


def field_dtype(name: str):
    return np.int32 if name in INT_FIELDS else np.float64


def particles_struct(arrays: dict, n: int, fields=None) -> PsphParticles:
    """Builds a PsphParticles pointing into numpy arrays (kept alive by the caller).

    Arrays must be C-contiguous with the dtype/shape of `field_shape`; a field
    missing from `arrays` (or not in `fields`) is passed as NULL.
    """
    s = PsphParticles()
    s.n = n
    for f in ALL_FIELDS:
        if fields is not None and f not in fields:
            continue
        arr = arrays.get(f)
        if arr is None:
            continue
        if not arr.flags["C_CONTIGUOUS"] or arr.dtype != field_dtype(f) or arr.shape[0] < n:
            raise ValueError(f"field {f}: need a C-contiguous {field_dtype(f).__name__} array of {n} rows")
        ptype = C.POINTER(C.c_int32) if f in INT_FIELDS else C.POINTER(C.c_double)
        setattr(s, f, arr.ctypes.data_as(ptype))
    return s


_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "libpsph_gb300.so"


def library_path() -> str:
    """The in-tree build, or the file PSPH_LIBRARY names (another build of the
    same sources, e.g. with different tuning flags)."""
    return os.environ.get("PSPH_LIBRARY") or os.path.join(_HERE, "_build", LIB_NAME)


_lib = None


def load_library():
    """Loads the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


def _declare(lib):
    P = C.POINTER
    ctx = C.c_void_p
    lib.psph_abi_version.restype = C.c_int
    lib.psph_device_check.argtypes = [P(C.c_int)]
    lib.psph_create.argtypes = [P(PsphConfig), P(ctx)]
    lib.psph_destroy.argtypes = [ctx]
    lib.psph_destroy.restype = None
    lib.psph_last_error.argtypes = [ctx]
    lib.psph_last_error.restype = C.c_char_p
    lib.psph_set_stream.argtypes = [ctx, C.c_void_p]
    lib.psph_set_grid.argtypes = [ctx, P(PsphGrid)]
    lib.psph_set_integrator.argtypes = [ctx, P(PsphIntegrator)]
    lib.psph_upload.argtypes = [ctx, P(PsphParticles), C.c_int]
    lib.psph_step.argtypes = [ctx, C.c_int64, C.c_double, P(C.c_int64)]
    lib.psph_num_particles.argtypes = [ctx]
    lib.psph_num_particles.restype = C.c_int64
    lib.psph_download.argtypes = [ctx, P(PsphParticles)]
    lib.psph_original_index.argtypes = [ctx, P(C.c_int64)]
    lib.psph_get_grid.argtypes = [ctx, P(PsphGrid)]
    lib.psph_get_integrator.argtypes = [ctx, P(PsphIntegrator)]
    lib.psph_set_flow_profile.argtypes = [ctx, C.c_int, FlowFn, C.c_void_p]
    lib.psph_set_step_hooks.argtypes = [ctx, HookFn, C.c_void_p, C.c_int]
    lib.psph_patch.argtypes = [ctx, P(PsphParticles)]
    lib.psph_pairs_export.argtypes = [ctx, C.c_int, P(C.c_int64), C.c_int64, P(C.c_int64)]
    lib.psph_enable_timing.argtypes = [ctx, C.c_int]
    lib.psph_phase_times.argtypes = [ctx, P(C.c_double), C.c_int, P(C.c_int)]
    lib.psph_last_launch_count.argtypes = [ctx]
    lib.psph_last_launch_count.restype = C.c_int64
    lib.psph_list_rebuilds.argtypes = [ctx]
    lib.psph_list_rebuilds.restype = C.c_int64
    lib.psph_step_timed.argtypes = [ctx, C.c_int64, P(C.c_double), P(C.c_int64)]
    lib.psph_pair_count.argtypes = [ctx, P(C.c_uint64)]
    lib.psph_probe_fp64_peak.argtypes = [P(C.c_double)]
    lib.psph_pairs_export_noalloc.argtypes = [ctx, C.c_int, C.c_void_p, C.c_int64, P(C.c_int64)]
    names3 = P(C.c_char_p)
    dp = P(C.c_double)
    lib.psph_output_request.argtypes = [ctx, C.c_char_p, names3]
    lib.psph_output_write.argtypes = [ctx, C.c_char_p, names3, dp, dp, dp]
    lib.psph_output_flush.argtypes = [ctx]
    lib.psph_batch_create.argtypes = [P(PsphConfig), C.c_int, P(ctx)]
    lib.psph_batch_size.argtypes = [ctx]
    lib.psph_batch_size.restype = C.c_int
    lib.psph_batch_upload.argtypes = [ctx, P(PsphParticles), C.c_int]
    lib.psph_batch_step.argtypes = [ctx, C.c_int64, P(C.c_double), P(C.c_int64)]
    lib.psph_batch_num_particles.argtypes = [ctx, C.c_int]
    lib.psph_batch_num_particles.restype = C.c_int64
    lib.psph_batch_download.argtypes = [ctx, C.c_int, P(PsphParticles)]
    lib.psph_batch_original_index.argtypes = [ctx, C.c_int, P(C.c_int64)]
    lib.psph_batch_get_grid.argtypes = [ctx, C.c_int, P(PsphGrid)]
    lib.psph_batch_get_integrator.argtypes = [ctx, C.c_int, P(PsphIntegrator)]
    fp = P(C.c_float)
    lib.psph_mlp_create.argtypes = [C.c_uint64, P(C.c_void_p)]
    lib.psph_mlp_destroy.argtypes = [C.c_void_p]
    lib.psph_mlp_destroy.restype = None
    lib.psph_mlp_last_error.argtypes = [C.c_void_p]
    lib.psph_mlp_last_error.restype = C.c_char_p
    lib.psph_get_tuning.argtypes = [ctx, P(PsphTuning)]
    lib.psph_set_tuning.argtypes = [ctx, P(PsphTuning)]
    lib.psph_autotune.argtypes = [ctx, C.c_int64, P(PsphTuning)]
    for name in ("psph_get_tuning", "psph_set_tuning", "psph_autotune"):
        getattr(lib, name).restype = C.c_int
    lib.psph_mlp_set_params.argtypes = [C.c_void_p, fp, fp]
    lib.psph_mlp_get_params.argtypes = [C.c_void_p, fp, fp]
    lib.psph_mlp_set_data.argtypes = [C.c_void_p, fp, fp, C.c_int64]
    lib.psph_mlp_set_weights.argtypes = [C.c_void_p, fp]
    lib.psph_mlp_train.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_float, C.c_uint64, fp]
    lib.psph_mlp_loss_grad.argtypes = [C.c_void_p, fp, fp, C.c_int64, P(C.c_double), fp]
    lib.psph_mlp_infer.argtypes = [C.c_void_p, fp, C.c_int64, fp, C.c_int]
    lib.psph_closure_attach.argtypes = [ctx, C.c_void_p, C.c_double]
    lib.psph_closure_stats.argtypes = [ctx, P(C.c_uint64), P(C.c_uint64)]
    lib.psph_closure_features.argtypes = [ctx, fp]
    for name in ("psph_mlp_create", "psph_mlp_set_params", "psph_mlp_get_params", "psph_mlp_set_data",
                 "psph_mlp_set_weights",
                 "psph_mlp_train", "psph_mlp_loss_grad", "psph_mlp_infer", "psph_closure_attach",
                 "psph_closure_stats", "psph_closure_features"):
        getattr(lib, name).restype = C.c_int
    for name in ("psph_device_check", "psph_create", "psph_set_stream", "psph_set_grid", "psph_set_integrator",
                 "psph_upload", "psph_step", "psph_download", "psph_original_index", "psph_get_grid", "psph_get_integrator",
                 "psph_set_flow_profile", "psph_set_step_hooks", "psph_patch",
                 "psph_pairs_export", "psph_enable_timing", "psph_phase_times", "psph_step_timed", "psph_pair_count",
                 "psph_probe_fp64_peak", "psph_pairs_export_noalloc", "psph_batch_create", "psph_batch_upload",
                 "psph_batch_step", "psph_batch_download", "psph_batch_original_index", "psph_batch_get_grid",
                 "psph_batch_get_integrator", "psph_output_request", "psph_output_write", "psph_output_flush"):
        getattr(lib, name).restype = C.c_int


def flow_callback(fn, errors: list):
    """A psph_flow_fn calling fn(position) -> (velocity, density), the Python
    form of a Domain::InCon / OutCon hook; exceptions are collected in errors
    (a C callback cannot raise) for the caller to re-raise."""
    def cb(x, v, den, _user):
        try:
            vel, d = fn(np.array([x[0], x[1], x[2]]))
            v[0], v[1], v[2] = float(vel[0]), float(vel[1]), float(vel[2])
            den[0] = float(d)
        except BaseException as e:  # noqa: BLE001 - re-raised by the caller
            errors.append(e)
    return FlowFn(cb)


NO_FLOW_FN = C.cast(None, FlowFn)
NO_HOOK_FN = C.cast(None, HookFn)


def step_hook_callback(hooks: dict, run, errors: list):
    """A psph_hook_fn / oracle hook calling run(hooks[where]) for the points
    present in hooks; exceptions are collected in errors and stop the step."""
    def cb(_ctx, where, _user):
        fn = hooks.get(where)
        if fn is None:
            return 0
        try:
            run(fn)
            return 0
        except BaseException as e:  # noqa: BLE001 - re-raised by the caller
            errors.append(e)
            return 1
    return HookFn(cb)


class PsphError(RuntimeError):
    """A non-zero psph_status, carrying the library's message (the reference
    throws `Fatal` at these points)."""

    def __init__(self, code: int, message: str):
        self.code = code
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
