"""ctypes binding of libaugur_gb300.so (the C ABI declared in include/augur_pm.h).

The product path has no fallback: if the library is missing or a call fails, a
RuntimeError says why. Build it with ``python -m augur_gb300.build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libaugur_gb300.so"

AUGUR_MODE_PERIODIC = 0
AUGUR_MODE_ISOLATED_SOFTENED = 1

_vp, _i64, _i32, _f32, _f64 = C.c_void_p, C.c_int64, C.c_int, C.c_float, C.c_double

# name -> (restype, argtypes); every symbol include/*.h declares is listed here
SIGNATURES = {
    "augur_status_string": (C.c_char_p, [_i32]),
    "augur_version": (_i32, []),
    "augur_pm_plan_create": (_i32, [C.POINTER(_vp), _i32, _i32, _i64, _i32, _f64, _f64, _f64]),
    "augur_pm_plan_destroy": (_i32, [_vp]),
    "augur_pm_plan_workspace_bytes": (_i64, [_vp]),
    "augur_pm_plan_get_tiles": (_i32, [_vp, _vp]),
    "augur_pm_plan_set_tiles": (_i32, [_vp, _vp]),
    "augur_pm_plan_bind_force_grid": (_i32, [_vp, _vp]),
    "augur_pm_set_kernel_mlp": (_i32, [_vp, _vp, _i32, _vp, _i32, _i32, _f64, _f64, _vp]),
    "augur_pm_reset_kernel": (_i32, [_vp, _vp]),
    "augur_pm_pair_acc": (_i32, [_vp, _vp, _vp, _vp, _i64, _f64, _i32, _vp, _i32, _vp, _i32, _i32, _f64, _vp, _vp]),
    "augur_pm_cell_index": (_i32, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "augur_pm_deposit": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _vp]),
    "augur_pm_poisson": (_i32, [_vp, _vp, _vp, _vp]),
    "augur_pm_gather": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "augur_pm_force": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "augur_pm_step": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _f32, _i32, _vp]),
    "augur_pm_step_host": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _f32, _i32, _vp]),
    "augur_pm_run": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _f32, _i32, _vp, _vp]),
    "augur_pm_run_begin": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _f32, _vp]),
    "augur_pm_run_steps": (_i32, [_vp, _i32, _vp]),
    "augur_pm_batch_create": (_i32, [C.POINTER(_vp), _vp, _i32]),
    "augur_pm_batch_run_steps": (_i32, [_vp, _i32, _vp]),
    "augur_pm_batch_size": (_i32, [_vp]),
    "augur_pm_batch_destroy": (_i32, [_vp]),
    "augur_pm_run_end": (_i32, [_vp, _vp, _vp, _vp, _vp]),
    "augur_pm_run_profile": (_i32, [_vp, _i32, _vp, _i32, _vp]),
    "augur_pm_run_load": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _f32, _vp]),
    "augur_pm_run_grid": (_i32, [_vp, _vp, _i32, _vp]),
    "augur_pm_force_grid": (_vp, [_vp]),
    "augur_pm_run_kick": (_i32, [_vp, _f32, _i32, _vp, _vp, _f32, _vp]),
    "augur_pm_run_unload": (_i32, [_vp, _vp, _vp, _vp]),
    "augur_pm_last_launches": (_i64, [_vp]),
    "augur_pm_check": (_i32, [_vp, _vp]),
    "augur_direct_sum_fp64": (_i32, [_vp, _vp, _i64, _vp, _vp, _i64, _i32, _f64, _f64, _vp, _vp]),
    "augur_energy_fp64": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp]),
    "augur_direct_sum_fp64_noalloc": (_i32, [_vp, _vp, _i64, _vp, _vp, _i64, _i32, _f64, _vp, _vp]),
    # include/augur_field2d.h
    "augur_field2d_scatter_work_bytes": (C.c_size_t, [_i32]),
    "augur_field2d_scatter": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _f64, _f64, _vp, _vp, _vp]),
    "augur_field2d_inputs": (_i32, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "augur_unet2d_param_count": (_i64, [_i32, _i32, _i32, _i32]),
    "augur_unet2d_prepared_count": (_i64, [_i32, _i32, _i32, _i32]),
    "augur_unet2d_prepare": (_i32, [_vp, _i32, _i32, _i32, _i32, _vp, _vp]),
    "augur_unet2d_work_bytes": (C.c_size_t, [_i32, _i32, _i32, _i32]),
    "augur_unet2d_forward": (_i32, [_vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _vp, C.c_size_t, _vp]),
    "augur_field2d_accel": (_i32, [_vp, _vp, _i32, _f64, _vp, _vp]),
    "augur_field2d_finish_work_bytes": (C.c_size_t, []),
    "augur_field2d_finish": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "augur_field2d_drift": (_i32, [_vp, _vp, _vp, _i64, _f64, _vp, _vp, _vp]),
    "augur_field2d_kick": (_i32, [_vp, _vp, _vp, _i64, _f64, _vp, _vp, _vp]),
    "augur_tick2d_work_bytes": (C.c_size_t, [_i32]),
    "augur_tick2d_drift_scatter": (_i32, [_vp, _vp, _i64, _i32, _i32, _f64, _f64, _f64, _i32, _i32, _f64, _f64, _vp,
                                          _vp, _vp]),
    "augur_tick2d_drift": (_i32, [_vp, _vp, _i64, _i32, _i32, _f64, _f64, _f64, _vp]),
    "augur_tick2d_mean_acc": (_i32, [_vp, _vp, _i32, _f64, _i64, _vp, _vp, _vp]),
    "augur_tick2d_gather_kick": (_i32, [_vp, _vp, _vp, _i64, _i32, _i32, _f64, _f64, _vp, _i32, _f64, _i32, _f64,
                                        _f64, _vp]),
    # include/augur_cnn.h
    "augur_cnn_conv_tc": (_i32, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _f32, _vp, _vp, _vp]),
    "augur_cnn_conv_in": (_i32, [_vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp]),
    "augur_cnn_conv_in_tc": (_i32, [_vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp]),
    "augur_cnn_wgrad": (_i32, [_i32, _vp, _vp, _i32, _i32, _vp, _i32, _vp, _vp, _vp]),
    "augur_cnn_set_wait_budget": (C.c_uint, [C.c_uint]),
    "augur_cnn_prep_weights": (_i32, [_vp, _i32, _i32, _i32, _i32, _i32, _vp, _vp]),
    "augur_cnn_input": (_i32, [_vp, _vp, _i64, _f32, _f32, _vp, _vp]),
    "augur_cnn_adamw": (_i32, [_vp, _vp, _vp, _vp, _i32, _f32, _f32, _f32, _f32, _f32, _i32, _vp]),
    "augur_cnn_gather_transpose": (_i32, [_vp, _vp, _i64, _i32, _f64, _vp, _vp]),
    "augur_cnn_pack_dout": (_i32, [_vp, _i64, _f32, _vp, _vp]),
    "augur_cnn_gelu_bwd": (_i32, [_vp, _vp, _i64, _vp, _vp]),
}



class Tiles(C.Structure):
    """augur_pm_tiles: launch geometry of a plan's kernels (results do not depend on it)."""
    _fields_ = [("deposit_rows_y", C.c_int), ("deposit_rows_z", C.c_int), ("deposit_chunk", C.c_int),
                ("green_tile_y", C.c_int), ("c2r_rows", C.c_int), ("fft_rows", C.c_int),
                ("deposit_aggregate", C.c_int)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}

    @classmethod
    def from_dict(cls, d: dict) -> "Tiles":
        return cls(**{k: int(d[k]) for k, _ in cls._fields_})


_lib = None


def load() -> C.CDLL:
    """Load the library once; raises RuntimeError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"augur_gb300 native library not built: {LIB_PATH} is missing "
                           "(run python -m augur_gb300.build)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            if name in OPTIONAL:
                continue
            raise RuntimeError(f"{LIB_PATH.name} does not export {name}")
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


OPTIONAL: set[str] = set()


def status_text(rc: int) -> str:
    return load().augur_status_string(rc).decode()


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed: {status_text(rc)} (status {rc})")


def register(name: str, restype, argtypes, optional: bool = False) -> None:
    """Declare an additional exported symbol (used by sibling modules)."""
    SIGNATURES[name] = (restype, argtypes)
    if optional:
        OPTIONAL.add(name)
    if _lib is not None:
        fn = getattr(_lib, name, None)
        if fn is not None:
            fn.restype, fn.argtypes = restype, argtypes
