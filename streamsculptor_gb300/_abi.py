"""ctypes mirror of include/streamsculptor_gb300.h and the library loader.

The Python facade calls the CUDA library only through these C-ABI entry
points (plain pointers and sizes).  There is no CPU fallback: if the library
is missing the import of any compute entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

SS_ABI_VERSION = 8
SS_MAX_COMPONENTS = 16

SS_OK = 0
SS_ERR_INVALID_ARGUMENT = -1
SS_ERR_CUDA = -2
SS_ERR_NONFINITE = -3
SS_ERR_WORKSPACE = -4
SS_ERR_UNSUPPORTED = -5

SS_NFW = 1
SS_TRIAXIAL_NFW = 2
SS_MIYAMOTO_NAGAI = 3
SS_HERNQUIST = 4
SS_PLUMMER = 5
SS_ISOCHRONE = 6
SS_SH_EXPANSION = 7
SS_BAR = 8
SS_DEHNEN_BAR = 9
SS_UNIFORM_ACCEL = 10
SS_POWERLAW_CUTOFF = 11
SS_ZHAO = 12
SS_SHEXP_LMAX = 8

SS_CENTER_ORIGIN = 0
SS_CENTER_TRACK = 1
SS_GROWS = 4

SS_SH_PLUMMER = 1
SS_SH_HERNQUIST = 2
SS_SH_GRID = 3

SS_RELEASE_FARDAL = 0
SS_RELEASE_CHEN25 = 1

VP = C.c_void_p
DP = C.POINTER(C.c_double)


class ss_component(C.Structure):
    _fields_ = [("kind", C.c_int32), ("center", C.c_int32), ("p", C.c_double * 6)]


class ss_track(C.Structure):
    _fields_ = [("knots", VP), ("slopes", VP), ("t0", C.c_double), ("dt", C.c_double),
                ("n_knots", C.c_int64), ("linear", C.c_int32), ("reserved", C.c_int32)]


class ss_subhalos(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("n", C.c_int64),
                ("m", VP), ("a", VP), ("x0", VP), ("v", VP), ("t0", VP), ("t_window", C.c_double),
                ("grid", VP), ("grid_u0", VP), ("grid_du", VP), ("n_grid", C.c_int64)]


class ss_expansion(C.Structure):
    _fields_ = [("l_max", C.c_int32), ("n_knots", C.c_int32), ("log_r0", C.c_double), ("dlog_r", C.c_double),
                ("coef", VP)]


class ss_potential(C.Structure):
    _fields_ = [("G", C.c_double), ("n_components", C.c_int32), ("reserved", C.c_int32),
                ("comp", ss_component * SS_MAX_COMPONENTS), ("track", ss_track),
                ("subhalos", ss_subhalos), ("expansion", ss_expansion), ("frame_velocity", ss_track),
                ("growth", ss_track)]


class ss_stream_cfg(C.Structure):
    _fields_ = [("t0", C.c_double), ("dt", C.c_double), ("n_steps", C.c_int64),
                ("n_particles", C.c_int64), ("particles_per_release", C.c_int32),
                ("steps_per_release", C.c_int32), ("snap_stride", C.c_int32), ("reserved", C.c_int32),
                ("first_particle", C.c_int64), ("snap_pitch", C.c_int64),
                ("stream_particles", C.c_int64), ("subhalos_per_stream", C.c_int32), ("reserved2", C.c_int32)]


class ss_release_cfg(C.Structure):
    _fields_ = [("n_release", C.c_int64), ("n_draw", C.c_int32), ("model", C.c_int32),
                ("kvals", C.c_double * 8), ("chen_mean", C.c_double * 6), ("chen_L", C.c_double * 36)]


class ss_pert_cfg(C.Structure):
    _fields_ = [("t0", C.c_double), ("dt", C.c_double), ("n_steps", C.c_int64),
                ("n_particles", C.c_int64), ("particles_per_release", C.c_int32),
                ("steps_per_release", C.c_int32), ("ncol", C.c_int32), ("save_stride", C.c_int32)]


SS_MLP_WIDTH = 128
SS_MLP_NPARAM = 128 * 4 + 128 + 3 * (128 * 128 + 128) + 128 + 1


SS_MLP_BASE_MAX = 256


class ss_mlp(C.Structure):
    _fields_ = [("params", VP), ("in_scale", C.c_float * 4), ("in_shift", C.c_float * 4),
                ("out_scale", C.c_float), ("out_shift", C.c_float),
                ("base", VP), ("base_n", C.c_int32), ("reserved", C.c_int32), ("base_u0", C.c_double),
                ("base_du", C.c_double)]


STRUCTS = [ss_potential, ss_stream_cfg, ss_release_cfg, ss_pert_cfg, ss_component, ss_track, ss_subhalos,
           ss_expansion, ss_mlp]

# name -> (restype, argtypes)
SIGNATURES = {
    "ss_abi_version": (C.c_int, []),
    "ss_last_error": (C.c_char_p, []),
    "ss_abi_sizeof": (C.c_int64, [C.c_int]),
    "ss_kernel_launches": (C.c_int64, []),
    "ss_potential_eval": (C.c_int, [C.POINTER(ss_potential), VP, C.c_int64, VP, C.c_double, VP, VP, VP, VP]),
    "ss_orbit_f64": (C.c_int, [C.POINTER(ss_potential), VP, C.c_int64, C.c_double, C.c_double, C.c_int64,
                               C.c_int64, VP, VP]),
    "ss_orbit_ensemble_f64": (C.c_int, [C.POINTER(ss_potential), VP, C.c_int64, C.c_double, VP, C.c_double,
                                        C.c_int64, C.c_int64, C.c_int32, VP, VP]),
    "ss_orbit_shoot_workspace_bytes": (C.c_int64, [C.c_int64]),
    "ss_orbit_shoot_slices": (C.c_int64, [C.c_int64]),
    "ss_orbit_shoot_f64": (C.c_int, [C.POINTER(ss_potential), VP, C.c_double, C.c_double, C.c_int64, C.c_int64, VP,
                                     VP, C.c_int64, C.c_double, VP]),
    "ss_track_slopes": (C.c_int, [VP, C.c_int64, C.c_double, VP, VP]),
    "ss_release_f64": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_release_cfg), VP, VP, VP, VP, VP, VP, VP]),
    "ss_stream_f64": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg), VP, VP, VP, VP, VP]),
    "ss_stream_workspace_bytes": (C.c_int64, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg)]),
    "ss_stream_f32k": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg), VP, VP, VP, VP, VP,
                                 C.c_int64, VP]),
    "ss_stream_f32k_noalloc": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg), VP, VP, VP, VP, VP]),
    "ss_subhalo_eval": (C.c_int, [C.POINTER(ss_subhalos), C.c_double, VP, C.c_int64, C.c_double, VP, VP, VP,
                                  VP, VP]),
    "ss_pert_term": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_subhalos), C.c_int, C.c_double, VP, VP, VP]),
    "ss_pert_workspace_bytes": (C.c_int64, [C.POINTER(ss_pert_cfg), C.c_int, C.c_int64]),
    "ss_pert_response": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_subhalos), C.POINTER(ss_pert_cfg),
                                   C.c_int, VP, VP, VP, VP, VP, C.c_int64, VP]),
    "ss_stream_f32k_ckpt": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg), VP, VP, VP, VP, C.c_int32,
                                      VP]),
    "ss_stream_adjoint_f32": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg), VP, C.c_int32, VP, VP, VP,
                                        VP]),
    "ss_release_vjp": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_release_cfg), VP, VP, VP, VP, VP, VP, VP, VP,
                                 VP]),
    "ss_prog_tangents_workspace_bytes": (C.c_int64, [C.c_int64, C.c_int32]),
    "ss_prog_tangents_f64": (C.c_int, [C.POINTER(ss_potential), VP, VP, C.c_double, C.c_int32, C.c_int32, VP, VP,
                                       VP, VP, VP, C.c_int64, VP]),
    "ss_binned_sums": (C.c_int, [VP, VP, C.c_int64, C.c_int32, VP, C.c_int32, VP, VP, VP]),
    "ss_peak_fma": (C.c_int, [C.c_int, C.c_int64, DP, VP, VP]),
    "ss_math_f64": (C.c_int, [C.c_int, VP, C.c_int64, VP, VP, VP]),
    "ss_copy_rows_async": (C.c_int, [VP, VP, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int, VP]),
    "ss_pert_track_bytes": (C.c_int64, [C.POINTER(ss_pert_cfg), C.c_int]),
    "ss_pert_base_track": (C.c_int, [C.POINTER(ss_potential), C.POINTER(ss_pert_cfg), C.c_int, VP, VP, VP, C.c_int64,
                                     VP]),
    "ss_pert_response_track": (C.c_int, [C.POINTER(ss_subhalos), C.c_double, C.POINTER(ss_pert_cfg), C.c_int, VP, VP,
                                         VP, VP]),
    "ss_mlp_eval_workspace_bytes": (C.c_int64, [C.c_int64]),
    "ss_mlp_eval": (C.c_int, [C.POINTER(ss_mlp), VP, C.c_int64, VP, VP, VP, C.c_int64, VP]),
    "ss_mlp_train_workspace_bytes": (C.c_int64, [C.c_int64]),
    "ss_mlp_loss_grad": (C.c_int, [C.POINTER(ss_mlp), VP, VP, VP, VP, VP, C.c_int64, VP, VP, VP, C.c_int64, VP]),
    "ss_mlp_train_backend": (C.c_int, [C.c_int]),
    "ss_mlp_fit_workspace_bytes": (C.c_int64, [C.c_int64]),
    "ss_mlp_fit": (C.c_int, [C.POINTER(ss_mlp), VP, VP, VP, VP, VP, VP, C.c_int64, VP, C.c_int64, C.c_int64,
                             C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, VP, VP, VP, VP, C.c_int64,
                             VP]),
    "ss_mlp_adam": (C.c_int, [VP, VP, VP, VP, C.c_int64, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float,
                              VP]),
    "ss_mlp_grad_bf16": (C.c_int, [C.POINTER(ss_mlp), VP, C.c_int64, VP, VP, VP]),
    "ss_stream_mlp_workspace_bytes": (C.c_int64, [C.POINTER(ss_stream_cfg)]),
    "ss_stream_mlp_bf16": (C.c_int, [C.POINTER(ss_mlp), C.POINTER(ss_stream_cfg), VP, VP, VP, VP, VP, C.c_int64,
                                     VP]),
    "ss_stream_mlp_judged_workspace_bytes": (C.c_int64, [C.POINTER(ss_potential), C.POINTER(ss_stream_cfg)]),
    "ss_stream_mlp_judged_bf16": (C.c_int, [C.POINTER(ss_mlp), C.POINTER(ss_potential), C.POINTER(ss_stream_cfg),
                                            C.c_float, C.c_int32, VP, VP, VP, VP, VP, VP, C.c_int64, VP]),
}

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libssgb300.so")

_lib = None
_lock = threading.Lock()


class SSError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, name: str, code: int, msg: str):
        super().__init__(f"{name} failed ({code}): {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libssgb300.so (raises if it is missing: there is no fallback)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"streamsculptor_gb300 CUDA library not found at {p}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (nvcc, sm_103a)")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.ss_abi_version() != SS_ABI_VERSION:
            raise RuntimeError("libssgb300.so ABI version mismatch")
        for i, st in enumerate(STRUCTS):
            if lib.ss_abi_sizeof(i) != C.sizeof(st):
                raise RuntimeError(f"ABI struct size mismatch for {st.__name__}: "
                                   f"C {lib.ss_abi_sizeof(i)} vs ctypes {C.sizeof(st)}")
        if path is None:
            _lib = lib
        return lib


def call(name: str, *args) -> int:
    """Call entry point `name`; raise SSError on a negative status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc < 0:
        msg = lib.ss_last_error().decode(errors="replace")
        raise SSError(name, rc, msg)
    return rc
