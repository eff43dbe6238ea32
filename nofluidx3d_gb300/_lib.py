"""ctypes binding of the native library libnfx.so (C ABI declared in include/nfx.h).

The library is built in-tree by nofluidx3d_gb300.build. There is no fallback: if the library
is missing or cannot be loaded, or no CUDA device is visible, calls raise NfxError.
"""

from __future__ import annotations

import ctypes as C
import re
import threading
from pathlib import Path

from . import build as _build

NFX_OK = 0
ERR_NAMES = {1: "NFX_ERR_ARG", 2: "NFX_ERR_CUDA", 3: "NFX_ERR_STATE", 4: "NFX_ERR_NOMEM", 5: "NFX_ERR_NODEVICE"}

MODEL_MR, MODEL_SVK, MODEL_SVKK, MODEL_VP = 0, 1, 2, 3
CONTACT_SUBSTRATE, CONTACT_PLANE, CONTACT_SPHERE, CONTACT_SPHERE_INTEGRAL = 0, 1, 2, 3
STATUS_NONFINITE, STATUS_INVERTED, STATUS_CURVE_FULL = 1, 2, 4
FIELD_VON_MISES, FIELD_PRESSURE, FIELD_PLASTIC_STRAIN = 0, 1, 2


class NfxError(RuntimeError):
    """A libnfx call failed; .code is the NFX_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None

_vp = C.c_void_p
_i64 = C.c_int64
_SIGS = {
    "nfx_version": ([], C.c_int),
    "nfx_plan_check": ([_i64, _i64, _vp, _vp, C.c_int, C.POINTER(_i64), C.POINTER(_i64)], C.c_int),
    "nfx_last_error": ([C.c_char_p, C.c_size_t], C.c_int),
    "nfx_create": ([C.c_int, C.POINTER(_vp)], C.c_int),
    "nfx_destroy": ([_vp], C.c_int),
    "nfx_set_mesh": ([_vp, _i64, _i64, _vp, _vp], C.c_int),
    "nfx_set_tetra": ([_vp, C.c_int, C.c_double, C.c_double, C.c_double], C.c_int),
    "nfx_set_viscoplastic": ([_vp, _vp], C.c_int),
    "nfx_add_contact": ([_vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                         C.POINTER(C.c_int)], C.c_int),
    "nfx_set_contact_table": ([_vp, C.c_int, _i64, _i64, _vp], C.c_int),
    "nfx_set_integrator": ([_vp, C.c_double, C.c_int], C.c_int),
    "nfx_set_integrator_lumped": ([_vp, C.c_double, C.c_double], C.c_int),
    "nfx_set_record": ([_vp, C.c_int, _i64, _i64], C.c_int),
    "nfx_step": ([_vp, _i64], C.c_int),
    "nfx_record_now": ([_vp], C.c_int),
    "nfx_sync": ([_vp], C.c_int),
    "nfx_get_time": ([_vp, C.POINTER(_i64)], C.c_int),
    "nfx_get_points": ([_vp, _vp], C.c_int),
    "nfx_set_points": ([_vp, _vp], C.c_int),
    "nfx_get_velocities": ([_vp, _vp], C.c_int),
    "nfx_set_velocities": ([_vp, _vp], C.c_int),
    "nfx_get_force_old": ([_vp, _vp], C.c_int),
    "nfx_set_force_old": ([_vp, _vp], C.c_int),
    "nfx_get_tet_field": ([_vp, C.c_int, _vp], C.c_int),
    "nfx_get_plastic_tensor": ([_vp, _vp], C.c_int),
    "nfx_set_plastic_tensor": ([_vp, _vp], C.c_int),
    "nfx_checkpoint_size": ([_vp, C.POINTER(_i64)], C.c_int),
    "nfx_checkpoint_save": ([_vp, _vp, _i64], C.c_int),
    "nfx_checkpoint_load": ([_vp, _vp, _i64], C.c_int),
    "nfx_get_curve": ([_vp, _vp, _i64, C.POINTER(_i64)], C.c_int),
    "nfx_indenter_force": ([_vp, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "nfx_status": ([_vp, C.POINTER(C.c_uint32), C.c_int], C.c_int),
    "nfx_time_steps": ([_vp, _i64, C.POINTER(C.c_float)], C.c_int),
    "nfx_profile_steps": ([_vp, _i64, C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
    "nfx_profile_tet_pass": ([_vp, C.c_int, C.POINTER(C.c_float)], C.c_int),
    "nfx_mesh_info": ([_vp, C.POINTER(_i64), C.POINTER(_i64)], C.c_int),
    "nfx_snapshot": ([_vp, _vp, _vp, _i64, C.POINTER(_i64)], C.c_int),
    "nfx_snapshot_wait": ([_vp], C.c_int),
    "nfx_host_alloc": ([C.c_size_t, C.POINTER(_vp)], C.c_int),
    "nfx_host_free": ([_vp], C.c_int),
    "nfx_divide_check": ([C.c_int, _i64, _vp, _vp, _vp], C.c_int),
    "nfx_indenter_force_noalloc": ([C.c_int, _i64, _vp, C.c_int, C.c_double, C.c_double, C.c_double, _vp, _vp],
                                   C.c_int),
    "nfx_batch_create": ([C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
    "nfx_batch_destroy": ([_vp], C.c_int),
    "nfx_batch_add_cell": ([_vp, _i64, _i64, _vp, _vp, C.POINTER(C.c_int)], C.c_int),
    "nfx_batch_add_cell_like": ([_vp, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "nfx_batch_set_tetra": ([_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double], C.c_int),
    "nfx_batch_set_viscoplastic": ([_vp, C.c_int, _vp], C.c_int),
    "nfx_batch_add_contact": ([_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.POINTER(C.c_int)], C.c_int),
    "nfx_batch_set_integrator": ([_vp, C.c_int, C.c_double, C.c_int], C.c_int),
    "nfx_batch_set_integrator_lumped": ([_vp, C.c_int, C.c_double, C.c_double], C.c_int),
    "nfx_batch_set_record": ([_vp, C.c_int, _i64, _i64], C.c_int),
    "nfx_batch_finalize": ([_vp], C.c_int),
    "nfx_batch_step": ([_vp, _i64], C.c_int),
    "nfx_batch_time_steps": ([_vp, _i64, C.POINTER(C.c_float)], C.c_int),
    "nfx_batch_record_now": ([_vp], C.c_int),
    "nfx_batch_indenter_force": ([_vp, C.c_int, _vp], C.c_int),
    "nfx_batch_get_curve": ([_vp, C.c_int, _vp, _i64, C.POINTER(_i64)], C.c_int),
    "nfx_batch_get_points": ([_vp, C.c_int, _vp], C.c_int),
    "nfx_batch_set_points": ([_vp, C.c_int, _vp], C.c_int),
    "nfx_batch_status": ([_vp, C.POINTER(C.c_uint32), C.c_int], C.c_int),
    "nfx_batch_cell_status": ([_vp, _vp, C.c_int], C.c_int),
    "nfx_batch_info": ([_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), C.POINTER(C.c_int)], C.c_int),
    "nfx_batch_tuning": ([_vp, _vp, _vp, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "nfx_batch_buckets": ([_vp, C.c_int, C.POINTER(C.c_int), _vp, _vp, _vp], C.c_int),
    "nfx_mlp_create": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i64, C.POINTER(_vp)], C.c_int),
    "nfx_mlp_destroy": ([_vp], C.c_int),
    "nfx_mlp_num_params": ([_vp, C.POINTER(_i64)], C.c_int),
    "nfx_mlp_set_output_gain": ([_vp, C.c_int, C.c_float], C.c_int),
    "nfx_mlp_set_params": ([_vp, _vp], C.c_int),
    "nfx_mlp_get_params": ([_vp, _vp], C.c_int),
    "nfx_mlp_get_grads": ([_vp, _vp], C.c_int),
    "nfx_mlp_forward": ([_vp, _vp, _i64, _vp], C.c_int),
    "nfx_mlp_backward": ([_vp, _vp, _vp, _vp, _i64, C.c_float, _vp, _vp], C.c_int),
    "nfx_mlp_adamw": ([_vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float], C.c_int),
    "nfx_mlp_train": ([_vp, _vp, _vp, _vp, _i64, _i64, _i64, _vp, C.c_uint64, _vp], C.c_int),
    "nfx_mlp_fit_inputs": ([_vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp], C.c_int),
}


def header_symbols() -> list[str]:
    """Names of the functions include/nfx.h declares."""
    text = (_build.INCLUDE / "nfx.h").read_text()
    return sorted(set(re.findall(r"^\s*int\s+(nfx_\w+)\s*\(", text, flags=re.M)))


def load(build_if_needed: bool = True):
    """Load libnfx.so (building it first when sources are newer). Raises NfxError on failure."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build_if_needed else _build.lib_path()
        if not Path(path).exists():
            raise NfxError(2, f"native library not built: {path}")
        lib = C.CDLL(str(path))
        for name, (args, res) in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
        return lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().nfx_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != NFX_OK:
        raise NfxError(rc, last_error())


def library_path() -> Path:
    return _build.lib_path()
