"""Gaussian smoothing of sensitivity kernels (xsmooth_sem,
tomography/postprocess_sensitivity_kernels/smooth_sem.F90) through the device
entry points prepare_smooth_gpu / compute_smooth_gpu / get_smooth_gpu."""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import abi
from .meshgen import NGLL3, WGLL


def smoothing_parameters(sigma_h: float, sigma_v: float, elemsize_max_glob: float):
    """(sigma_h2, sigma_v2, sigma_h3, sigma_v3) in single precision as
    smooth_sem.F90:524-559 sets them: sigma2 = 2 sigma^2, search radius
    3 sigma + max(sigma_h, sigma_v) / 2, the latter at least sqrt(3) x the
    largest element."""
    f = np.float32
    sh, sv = f(sigma_h), f(sigma_v)
    element_size = f(max(sh, sv) * f(0.5))
    if element_size < f(math.sqrt(3.0)) * f(elemsize_max_glob):
        element_size = f(f(math.sqrt(3.0)) * f(elemsize_max_glob))
    return (f(2.0) * sh * sh, f(2.0) * sv * sv, f(f(3.0) * sh + element_size), f(f(3.0) * sv + element_size))


def integ_factor(db: dict) -> np.ndarray:
    """J w_i w_j w_k per element GLL point (smooth_sem.F90:920-940), float32."""
    n = int(db["nspec"])
    irr = np.asarray(db["irregular_element_number"])
    jac = np.empty((n, NGLL3), np.float32)
    reg = irr == 0
    jac[reg] = np.float32(db["jacobian_regular"])
    if (~reg).any():
        jac[~reg] = np.asarray(db["jacobian"], np.float32).reshape(-1, NGLL3)[irr[~reg] - 1]
    w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1).astype(np.float32)
    return (jac * w3[None, :]).reshape(-1)


def smooth(db: dict, xyz_elem: np.ndarray, kernels: np.ndarray, sigma_h: float, sigma_v: float,
           elemsize_max_glob: float | None = None) -> np.ndarray:
    """Smoothed kernels (nker, nspec * 125) of one slice (kernels (nker, nspec * 125),
    xyz_elem (nspec, 125, 3))."""
    L = abi.load()
    A = abi.Args()
    kern = np.ascontiguousarray(np.asarray(kernels, np.float32).reshape(-1, int(db["nspec"]) * NGLL3))
    nker, nspec = kern.shape[0], int(db["nspec"])
    if elemsize_max_glob is None:
        from .hexmesh import element_size_max
        elemsize_max_glob = float(element_size_max(xyz_elem).max())
    h2, v2, h3, v3 = smoothing_parameters(sigma_h, sigma_v, elemsize_max_glob)
    x, y, z = (np.ascontiguousarray(xyz_elem[..., d].reshape(-1), np.float32) for d in range(3))
    handle = ctypes.c_long(0)
    L.prepare_smooth_gpu_(ctypes.addressof(handle), A.af(x), A.af(y), A.af(z), A.f(h2), A.f(v2), A.f(h3), A.f(v3),
                          A.i(nspec), A.i(nker))
    abi.check()
    L.compute_smooth_gpu_(ctypes.addressof(handle), A.af(kern), A.af(integ_factor(db)), A.af(x), A.af(y), A.af(z),
                          A.i(nspec))
    abi.check()
    out = np.zeros_like(kern)
    L.get_smooth_gpu_(ctypes.addressof(handle), out.ctypes.data)
    abi.check()
    return out
