"""ctypes binding of libexactdiag_gb300.so (declared in include/exactdiag_gb300.h).

There is no CPU fallback: if the library is missing the import of any device
operation raises, naming the build step.
"""

from __future__ import annotations

import ctypes
import pathlib

from exactdiag_gb300 import build as _build

ED_OK = 0
ED_F64, ED_C128, ED_F32, ED_C64 = 0, 1, 2, 3

ERRORS = {
    -1: "invalid argument",
    -2: "device allocation failed",
    -3: "CUDA error",
    -4: "basis not built",
    -5: "sector too large",
    -6: "internal consistency check failed",
    -7: "device wait timed out",
}

# Every symbol include/exactdiag_gb300.h declares, with its ctypes signature.
_c = ctypes
_vp = _c.c_void_p
_i64p = _c.POINTER(_c.c_int64)
_d4 = _c.POINTER(_c.c_double)
SIGNATURES = {
    "ed_sector_create": (_c.c_int, [_c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.POINTER(_vp)]),
    "ed_sector_destroy": (_c.c_int, [_vp]),
    "ed_basis_build": (_c.c_int, [_vp, _vp]),
    "ed_basis_size": (_c.c_int, [_vp, _i64p]),
    "ed_sector_set_launch": (_c.c_int, [_vp, _c.c_int, _c.c_int]),
    "ed_sector_get_launch": (_c.c_int, [_vp, _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]),
    "ed_sector_set_step_shape": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int]),
    "ed_sector_get_step_shape": (_c.c_int, [_vp, _c.POINTER(_c.c_int), _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]),
    "ed_sector_set_segment_window": (_c.c_int, [_vp, _c.c_int]),
    "ed_sector_get_segment_window": (_c.c_int, [_vp, _c.POINTER(_c.c_int)]),
    "ed_sector_row_kinds": (_c.c_int, [_vp, _c.POINTER(_c.c_int)]),
    "ed_sector_kind_rows": (_c.c_int, [_vp, _c.POINTER(_c.c_int64)]),
    "ed_sector_step_launches": (_c.c_int, [_vp, _c.POINTER(_c.c_int)]),
    "ed_position_correlations": (_c.c_int, [_vp, _c.c_int, _vp, _c.c_int, _c.c_int, _c.POINTER(_c.c_int), _c.POINTER(_c.c_double), _vp]),
    "ed_singlet_correlations": (_c.c_int, [_vp, _c.c_int, _vp, _c.POINTER(_c.c_int), _c.POINTER(_c.c_double), _vp]),
    "ed_sector_is_real": (_c.c_int, [_vp, _c.POINTER(_c.c_int)]),
    "ed_basis_export": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "ed_hv": (_c.c_int, [_vp, _d4, _c.c_int, _vp, _vp, _vp]),
    "ed_hv_mode": (_c.c_int, [_vp, _d4, _c.c_int, _vp, _vp, _c.c_int, _vp]),
    "ed_lanczos_step": (_c.c_int, [_vp, _d4, _c.c_int, _vp, _vp, _vp, _vp, _vp]),
    "ed_lanczos_hv": (_c.c_int, [_vp, _d4, _c.c_int, _vp, _vp, _vp, _vp, _vp]),
    "ed_lanczos_update": (_c.c_int, [_vp, _c.c_int, _vp, _vp, _vp, _vp]),
    "ed_accumulate": (_c.c_int, [_vp, _c.c_int, _vp, _c.c_double, _c.c_double, _vp, _vp]),
    "ed_accumulate_many": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.POINTER(_c.c_void_p), _c.POINTER(_c.c_double), _vp, _vp]),
    "ed_normalize": (_c.c_int, [_vp, _c.c_int, _vp, _vp, _vp]),
    "ed_continued_fraction": (_c.c_int, [_vp, _vp, _c.c_int, _vp, _c.c_int, _c.c_double, _c.c_double, _c.c_double,
                                         _vp, _vp]),
    "ed_excitation_apply": (_c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _vp, _vp, _vp]),
    "ed_batch_lanczos": (_c.c_int, [_c.POINTER(_vp), _c.c_int, _d4, _c.c_int, _c.POINTER(_vp), _c.c_int, _vp,
                                    _c.c_int, _vp]),
    "ed_project_out": (_c.c_int, [_vp, _c.c_int, _vp, _c.c_int, _vp, _vp, _vp]),
    "ed_project_out_noalloc": (_c.c_int, [_vp, _c.c_int, _vp, _c.c_int, _vp, _vp, _vp]),
    "ed_last_error_string": (_c.c_char_p, []),
}

_LIB = None


class EngineError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, func: str, status: int, detail: str):
        super().__init__(f"{func} failed: {ERRORS.get(status, status)} ({detail})")
        self.status = status


def library_path() -> pathlib.Path:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load the engine library; raise when it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise ImportError(f"{path} is missing: build it with exactdiag_gb300.build.build() (nvcc, sm_103a)")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(func: str, status: int) -> None:
    if status != ED_OK:
        detail = load().ed_last_error_string()
        raise EngineError(func, status, detail.decode() if detail else "")


def weights_array(w) -> ctypes.Array:
    arr = (ctypes.c_double * 4)(*[float(v) for v in w])
    return arr
