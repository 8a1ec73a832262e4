"""ctypes binding of libspecfem3d_gb300.so.

This is the binding a Python (or ctypes-speaking) caller uses; a Fortran solver
links the same symbols directly (they carry gfortran's `name_` mangling).
Loading fails loudly when the library has not been built: there is no CPU
fallback behind this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

P = ctypes.c_void_p
_INT_P = ctypes.POINTER(ctypes.c_int)
_LIB = None

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "specfem3d_gb300.h")


def header_signatures(path: str = HEADER) -> dict:
    """{name: (return type, [argument declarations])} of every function declared
    in include/specfem3d_gb300.h."""
    import re
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(void\s*\*\s*|void\s+|int\s+)(\w+)\s*\(([^;{]*?)\)\s*;", txt):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(2)] = (m.group(1).replace(" ", "").strip(), args)
    return out


# the reference-named entry points: void, every argument by reference
_FC_VOID = {n: len(a) for n, (r, a) in header_signatures().items() if n.endswith("_") and r == "void"}


def lib_path() -> str:
    return _build.lib_path()


def load() -> ctypes.CDLL:
    """Load the CUDA library (raises if it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run specfem3d_gb300.build.build() (needs nvcc); "
                           "there is no CPU fallback for the GPU path")
    L = ctypes.CDLL(path)
    for name, n in _FC_VOID.items():
        f = getattr(L, name)
        f.restype = None
        f.argtypes = [P] * n
    L.sf3d_last_error.restype = ctypes.c_int
    L.sf3d_last_error.argtypes = [ctypes.c_char_p, ctypes.c_int]
    L.sf3d_clear_error.restype = None
    L.sf3d_version.restype = ctypes.c_int
    L.sf3d_set_stf_table.restype = ctypes.c_int
    L.sf3d_set_stf_table.argtypes = [P, P, ctypes.c_int, ctypes.c_int]
    L.sf3d_set_sources.restype = ctypes.c_int
    L.sf3d_set_sources.argtypes = [P, ctypes.c_int, P, P, P, ctypes.c_int]
    L.sf3d_iterate_time.restype = ctypes.c_int
    L.sf3d_iterate_time.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_int]
    L.sf3d_get_seismograms.restype = ctypes.c_int
    L.sf3d_get_seismograms.argtypes = [P, P]
    L.sf3d_get_extra_kernels_f64.restype = ctypes.c_int
    L.sf3d_get_extra_kernels_f64.argtypes = [P, P, P]
    L.sf3d_get_seismograms_kind.restype = ctypes.c_int
    L.sf3d_get_seismograms_kind.argtypes = [P, ctypes.c_int, P]
    L.sf3d_last_timing.restype = ctypes.c_int
    L.sf3d_last_timing.argtypes = [P, P, P, P, P]
    L.sf3d_set_stiffness_variant.restype = ctypes.c_int
    L.sf3d_set_stiffness_variant.argtypes = [P, ctypes.c_int]
    L.sf3d_set_geometry_precision.restype = ctypes.c_int
    L.sf3d_set_geometry_precision.argtypes = [P, ctypes.c_int]
    L.sf3d_set_geometry_format.restype = ctypes.c_int
    L.sf3d_set_geometry_format.argtypes = [P, ctypes.c_int]
    L.sf3d_geometry_pack_info.restype = ctypes.c_int
    L.sf3d_geometry_pack_info.argtypes = [P, P, P]
    L.sf3d_autotune_stiffness.restype = ctypes.c_int
    L.sf3d_autotune_stiffness.argtypes = [P, ctypes.c_int, P, P]
    for name in ("sf3d_gradient_forward", "sf3d_gradient_backward"):
        getattr(L, name).restype = ctypes.c_int
        getattr(L, name).argtypes = [P, ctypes.c_float]
    L.sf3d_gradient_setup.restype = ctypes.c_int
    L.sf3d_gradient_setup.argtypes = [P, ctypes.c_int, ctypes.c_int, P]
    L.sf3d_gradient_set_residual.restype = ctypes.c_int
    L.sf3d_gradient_set_residual.argtypes = [P, P]
    L.sf3d_gradient_get.restype = ctypes.c_int
    L.sf3d_gradient_get.argtypes = [P, P, P, P]
    L.sf3d_gradient_set_fused.restype = ctypes.c_int
    L.sf3d_gradient_set_fused.argtypes = [P, ctypes.c_int]
    L.sf3d_gradient_release.restype = ctypes.c_int
    L.sf3d_gradient_release.argtypes = [P]
    L.sf3d_field_maxabs_noalloc.restype = ctypes.c_int
    L.sf3d_field_maxabs_noalloc.argtypes = [P, ctypes.c_long, P, P]
    L.sf3d_check_bounded_wait.restype = ctypes.c_int
    L.sf3d_check_bounded_wait.argtypes = [ctypes.c_double, P, P]
    L.sf3d_batch_prepare.restype = ctypes.c_int
    L.sf3d_batch_prepare.argtypes = [P, ctypes.c_int, P, P, P, ctypes.c_int, ctypes.c_int, P]
    L.sf3d_batch_set_tiling.restype = ctypes.c_int
    L.sf3d_batch_set_tiling.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.sf3d_batch_set_halves.restype = ctypes.c_int
    L.sf3d_batch_set_halves.argtypes = [P, ctypes.c_int]
    L.sf3d_batch_autotune.restype = ctypes.c_int
    L.sf3d_batch_autotune.argtypes = [P, ctypes.c_int, P, P, P, P]
    L.sf3d_batch_iterate.restype = ctypes.c_int
    L.sf3d_batch_iterate.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int]
    for name in ("sf3d_batch_timing",):
        getattr(L, name).restype = ctypes.c_int
        getattr(L, name).argtypes = [P, P, P]
    for name in ("sf3d_batch_get_seismograms", "sf3d_batch_get_displ"):
        getattr(L, name).restype = ctypes.c_int
        getattr(L, name).argtypes = [P, P]
    L.sf3d_batch_release.restype = ctypes.c_int
    L.sf3d_batch_release.argtypes = [P]
    L.sf3d_synchronize.restype = ctypes.c_int
    L.sf3d_synchronize.argtypes = [P]
    L.sf3d_device_ptr.restype = P
    L.sf3d_device_ptr.argtypes = [P, ctypes.c_char_p]
    L.sf3d_check_stability.restype = ctypes.c_int
    L.sf3d_check_stability.argtypes = [P, ctypes.c_float, P]
    L.sf3d_get_kernels_f64.restype = ctypes.c_int
    L.sf3d_get_kernels_f64.argtypes = [P, P, P, P]
    L.sf3d_get_kernels_ac_f64.restype = ctypes.c_int
    L.sf3d_get_kernels_ac_f64.argtypes = [P, P, P]
    L.sf3d_set_acoustic_kernel_pairing.restype = ctypes.c_int
    L.sf3d_set_acoustic_kernel_pairing.argtypes = [P, ctypes.c_int]
    _LIB = L
    return L


def exported_symbols():
    return list(header_signatures())


class SF3DError(RuntimeError):
    pass


def check() -> None:
    """Raise SF3DError if the library recorded an error (and clear it)."""
    L = load()
    buf = ctypes.create_string_buffer(512)
    code = L.sf3d_last_error(buf, 512)
    if code != 0:
        L.sf3d_clear_error()
        raise SF3DError(f"specfem3d_gb300 error {code}: {buf.value.decode()}")


# ---------------------------------------------------------------------------
# by-reference argument helpers
# ---------------------------------------------------------------------------

class Args:
    """Keeps the ctypes scalars / arrays of one call alive and hands out pointers."""

    def __init__(self):
        self._keep = []

    def i(self, v) -> int:
        c = ctypes.c_int(int(v))
        self._keep.append(c)
        return ctypes.addressof(c)

    def f(self, v) -> int:
        c = ctypes.c_float(float(v))
        self._keep.append(c)
        return ctypes.addressof(c)

    def a(self, arr, dtype) -> int:
        if arr is None:
            arr = np.zeros(1, dtype)
        arr = np.ascontiguousarray(arr, dtype=dtype)
        self._keep.append(arr)
        return arr.ctypes.data

    def ai(self, arr) -> int:
        return self.a(arr, np.int32)

    def af(self, arr) -> int:
        return self.a(arr, np.float32)

    def ad(self, arr) -> int:
        return self.a(arr, np.float64)
