"""ctypes binding of libjld.so, the C ABI declared in include/jld.h.

The library is built in-tree by jerald_gb300.build (nvcc, sm_103a).  Loading
fails loudly when it is missing: there is no CPU or library fallback for any
operation of this package.
"""
from __future__ import annotations

import ctypes as ct
import os
from pathlib import Path

from .build import LIB

_c_void_p = ct.c_void_p
_i32 = ct.c_int32
_i64 = ct.c_int64
_f32 = ct.c_float
_f64 = ct.c_double
_size = ct.c_size_t

# name -> argument types (every entry point returns int status unless noted)
_SIGS = {
    "jld_init_layout": [_i32, _i32],
    "jld_clean": [_i32],
    "jld_ppaint_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p],
    "jld_ppaint_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p],
    "jld_ppaint_box_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _f32, _i32, _i32, _i32, _c_void_p, _c_void_p],
    "jld_ppaint_box_acc_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _f32, _i32, _i32, _i32, _c_void_p,
                               _c_void_p],
    "jld_snap_prep_f32": [_c_void_p, _c_void_p, _i64, _f32, _c_void_p, _i32, _c_void_p, _c_void_p, _c_void_p,
                          _c_void_p, _c_void_p, _i64, _f64, _f64, _f64, _f64, _c_void_p, _c_void_p],
    "jld_ppaint_box_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _f64, _i64, _i64, _i64, _c_void_p, _c_void_p],
    "jld_ppaint_box_method_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _f32, _i32, _i32, _i32, _c_void_p, _i32,
                                  _c_void_p],
    "jld_cell_keys_f32": [_c_void_p, _c_void_p, _i64, _i32, _i32, _i32, _c_void_p, _c_void_p],
    "jld_cell_keys_f64": [_c_void_p, _c_void_p, _i64, _i64, _i64, _i64, _c_void_p, _c_void_p],
    "jld_preadout_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p, _i32, _c_void_p],
    "jld_preadout_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _i32, _c_void_p],
    "jld_preadout_box_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p, _i32, _c_void_p],
    "jld_preadout_box_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _i32, _c_void_p],
    "jld_ppaint3d_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p],
    "jld_ppaint3d_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p],
    "jld_ppaint3d_box_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p],
    "jld_ppaint3d_box_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p],
    "jld_preadout3d_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p, _i32, _c_void_p],
    "jld_preadout3d_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _i32, _c_void_p],
    "jld_preadout3d_box_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _i32, _i32, _i32, _c_void_p, _i32,
                               _c_void_p],
    "jld_preadout3d_box_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _i32,
                               _c_void_p],
    "jld_buildplan_f32": [_i32, _i32, _i32, _c_void_p],
    "jld_buildplan_f64": [_i32, _i32, _i32, _c_void_p],
    "jld_pfft_f32": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _c_void_p, _size],
    "jld_pfft_f64": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _c_void_p, _size],
    "jld_pfft_c_f32": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _size],
    "jld_pfft_c_f64": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _size],
    "jld_pifft_f32": [_c_void_p, _c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _size],
    "jld_pifft_f64": [_c_void_p, _c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _size],
    "jld_pifft_c_f32": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _size],
    "jld_pifft_c_f64": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p, _c_void_p, _size],
    "jld_pfft_c_static_f32": [_c_void_p, _c_void_p, _i32, _i32, _i32, _c_void_p],
    "jld_ldl_prepare_f32": [_i32, _i32, _i32, _c_void_p],
    "jld_ldl_step_f32": [_c_void_p, _c_void_p, _i64, _i32, _i32, _i32, _c_void_p, _i32, _i32, _i32, _i32, _i32,
                         _c_void_p, _c_void_p, _c_void_p, _c_void_p, _size, _c_void_p],
    "jld_ldl_step_ext_f32": [_c_void_p, _c_void_p, _i64, _i32, _i32, _i32, _c_void_p, _i32, _i32, _i32, _i32,
                             _i32, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _size, _c_void_p],
    "jld_ldl_step_hi_f32": [_c_void_p, _c_void_p, _i64, _i32, _i32, _i32, _c_void_p, _i32, _i32, _i32, _i32,
                            _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _size, _c_void_p],
    "jld_ldl_positions_f32": [_c_void_p, _i32, _i32, _i32, _i64, _i32, _i32, _c_void_p],
    "jld_ldl_error_word_f32": [_c_void_p, _i32, _i32, _i32, _i64, _i32, _c_void_p],
    "jld_ldl_order_f32": [_c_void_p, _i32, _i32, _i32, _i64, _i32, _c_void_p],
    "jld_graph_kernel_nodes": [_c_void_p, _c_void_p],
    "jld_copy_from_host": [_c_void_p, _c_void_p, _c_void_p, _size, _i32],
    "jld_fft_pipe_status": [_c_void_p, _i32],
    "jld_wait_selftest": [_c_void_p, _i32, _c_void_p],
    "jld_cell_sort_f32": [_c_void_p, _c_void_p, _i64, _i32, _i32, _i32, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                          _size],
    "jld_ppaint_sorted_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _f32, _i32, _i32, _i32, _c_void_p, _c_void_p,
                              _c_void_p, _c_void_p],
    "jld_ppaint_box_sorted_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _f32, _i32, _i32, _i32, _c_void_p,
                                  _c_void_p, _c_void_p, _size],
}
_RESTYPES = {
    "jld_version": ct.c_char_p,
    "jld_status_string": ct.c_char_p,
    "jld_last_error": ct.c_char_p,
    "jld_fft_workspace_f32": _size,
    "jld_fft_workspace_f64": _size,
    "jld_ldl_workspace_f32": _size,
    "jld_ldl_workspace_opt_f32": _size,
    "jld_ldl_workspace_hi_f32": _size,
    "jld_cell_sort_workspace": _size,
    "jld_ppaint_box_sorted_workspace": _size,
}
_EXTRA_ARGS = {
    "jld_ldl_workspace_f32": [_i32, _i32, _i32, _i64, _i32],
    "jld_ldl_workspace_opt_f32": [_i32, _i32, _i32, _i64, _i32, _i32],
    "jld_ldl_workspace_hi_f32": [_i32, _i32, _i32, _i64, _i32, _i32],
    "jld_status_string": [ct.c_int],
    "jld_fft_workspace_f32": [_i32, _i32, _i32],
    "jld_fft_workspace_f64": [_i32, _i32, _i32],
    "jld_cell_sort_workspace": [_i64],
    "jld_ppaint_box_sorted_workspace": [_i64],
    "jld_version": [],
    "jld_last_error": [],
}


class JLDError(RuntimeError):
    """A libjld entry point returned a nonzero status."""

    def __init__(self, name: str, status: int, msg: str):
        super().__init__(f"{name}: {msg} (status {status})")
        self.status = status


_lib = None


def lib_path() -> Path:
    return Path(os.environ.get("JLD_LIB", str(LIB)))


def load():
    """Loads libjld.so once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not path.exists():
        raise RuntimeError(
            f"{path} not found: build the CUDA library first (python -m jerald_gb300.build); "
            "this package has no CPU fallback")
    lib = ct.CDLL(str(path))
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ct.c_int
    for name, rt in _RESTYPES.items():
        fn = getattr(lib, name)
        fn.argtypes = _EXTRA_ARGS[name]
        fn.restype = rt
    _lib = lib
    return lib


def call(name: str, *args) -> None:
    """Calls an int-returning entry point and raises JLDError on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        msg = lib.jld_last_error().decode(errors="replace") or lib.jld_status_string(st).decode()
        raise JLDError(name, st, msg)


def exported_names() -> list[str]:
    return sorted(set(_SIGS) | set(_RESTYPES))
