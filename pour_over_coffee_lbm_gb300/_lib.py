"""ctypes binding of libpog.so (the C ABI declared in include/pog.h).

There is no CPU path: if the library cannot be built or loaded, every call raises.
"""
import ctypes
import os
import threading

from . import build as _build
from .params import PogParams, PogParticleParams

_lock = threading.Lock()
_lib = None

POG_OK = 0
ERRORS = {-1: "POG_E_ARG", -2: "POG_E_CUDA", -3: "POG_E_NAN", -4: "POG_E_INJECTED",
          -5: "POG_E_RANGE", -6: "POG_E_STATE"}

# (name, restype, argtypes) for every entry point of include/pog.h
_P = ctypes.POINTER(PogParams)
_PP = ctypes.POINTER(PogParticleParams)
_v = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_f = ctypes.c_float
SIGNATURES = [
    ("pog_version", _i, []),
    ("pog_last_error", ctypes.c_char_p, []),
    ("pog_launch_count", _ll, [_i]),
    ("pog_validate_params", _i, [_P]),
    ("pog_build_flags", _i, [_P, _v, _v]),
    ("pog_init_equilibrium", _i, [_P, _v, _v, _f, _f, _f, _f, _v]),
    ("pog_pour_advance", _i, [_P, _v]),
    ("pog_field_stats", _i, [_P, _v, _v, _v, _v, _v, _v, _v]),
    ("pog_filter_particles", _i, [_P, _v, _v, _v, _v, _i, _v, ctypes.c_uint32, _ll, _v]),
    ("pog_filter_update", _i, [_P, _v, _v, _v, _v]),
    ("pog_pressure_force", _i, [_P, _v, _v, _v, _f, _f, _v]),
    ("pog_density_drive", _i, [_P, _v, _v, _v, _f, _f, _f, _f, _v]),
    ("pog_phase_chemical_potential", _i, [_P, _v, _f, _v, _v]),
    ("pog_phase_normals", _i, [_P, _v, _v, _v, _v]),
    ("pog_phase_surface_tension", _i, [_P, _v, _v, _v, _v, _v, _f, _v, _v, _v, _v]),
    ("pog_phase_update", _i, [_P, _v, _v, _v, _v, _v, _f, _f, _f, _f, _v, _v, _v]),
    ("pog_phase_properties", _i, [_P, _v, _f, _f, _v, _v, _v]),
    ("pog_pour_phase", _i, [_P, _v, _v, _f, _v]),
    ("pog_step", _i, [_P, _v, _v, _ll, _i, _v, _v, _v, _v, _v, _v, _v, _v, _v]),
    ("pog_step_push", _i, [_P, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v]),
    ("pog_export_natural", _i, [_P, _v, _v, _ll, _v, _i, _v]),
    ("pog_import_natural", _i, [_P, _v, _i, _v, _v, _v]),
    ("pog_macroscopic", _i, [_P, _v, _v, _ll, _v, _v, _v, _v, _v]),
    ("pog_particles_bin_scratch_bytes", ctypes.c_size_t, [_i]),
    ("pog_particles_bin", _i, [_P, _v, _v, _i, _v, _v, _v, _v]),
    ("pog_particles_couple", _i, [_P, _PP, _v, _v, _v, _v, _v, _i, _v, _v, _v, _v, _v, _v]),
    ("pog_particles_clear_deposit", _i, [_P, _v, _i, _v, _v, _v, _v]),
    ("pog_zero", _i, [_v, ctypes.c_size_t, _v]),
    ("pog_drag_from_fixed", _i, [_P, _v, _v, _v]),
    ("pog_drag_from_fixed_cells", _i, [_P, _v, _v, _i, _v, _v, _v]),
    ("pog_adjoint_step", _i, [_P, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v, _v]),
    ("pog_adjoint_scratch_bytes", ctypes.c_size_t, [_P]),
    ("pog_device_status", _i, [_i]),
    ("pog_particles_bin_noalloc", _i, [_P, _v, _v, _i, _v, _v, _v]),
    ("pog_wall_list", _i, [_P, _v, _v, ctypes.c_int32, _v, _v]),
    ("pog_outflow_fixed", _i, [_P, _v, _v, _v, _v]),
]


class PogError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "POG_E?"), code, msg))
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libpog.so (building it in-tree with nvcc when absent or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing:
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError("libpog.so is missing; run pour_over_coffee_lbm_gb300.build.build()")
        lib = ctypes.CDLL(_build.LIB)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(code: int):
    if code != POG_OK:
        msg = load().pog_last_error()
        raise PogError(code, msg.decode() if msg else "")
    return code


def ptr(t):
    """Device pointer of a tensor as an int (ctypes passes it as void*), or None -> NULL."""
    if t is None:
        return None
    return t.data_ptr()


_raw_stream = None


def stream_handle(stream=None):
    """The CUDA stream handle (int) of `stream`, default torch's current stream.  The default
    path reads the raw handle of the current device's current stream directly (a per-step call:
    torch.cuda.current_stream() costs several microseconds of Python)."""
    global _raw_stream
    if stream is not None:
        return stream.cuda_stream
    if _raw_stream is None:
        import torch
        get_raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
        get_dev = getattr(torch._C, "_cuda_getDevice", None)
        if get_raw is not None and get_dev is not None:
            _raw_stream = lambda: get_raw(get_dev())  # noqa: E731
        else:
            _raw_stream = lambda: torch.cuda.current_stream().cuda_stream  # noqa: E731
    return _raw_stream()
