"""Misfit post-processing through the C ABI: adjoint sources from seismograms and
the summation of event kernels, computed on the device in FP64.

The reference does this with host tools: utils/adjoint_sources/{waveform,traveltime,
amplitude}/create_adjsrc_*.f90 (one ASCII trace at a time) and
src/tomography/sum_kernels.f90 (one proc*_kernel.bin per event and slice).  Here the
traces of all receivers and components, or the kernels of all events, go through
one call."""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi

KINDS = {"waveform": 0, "traveltime": 1, "amplitude": 2}


def _lib():
    L = abi.load()
    L.sf3d_adjoint_sources.restype = ctypes.c_int
    L.sf3d_adjoint_sources.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.sf3d_sum_kernels.restype = ctypes.c_int
    L.sf3d_sum_kernels.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p]
    return L


def adjoint_sources(kind: str, syn, dat, dt: float, t0: float, ts: float, te: float, component: int = 0):
    """(adj, norms) for traces (nrec, 3, nstep): kind "waveform" (needs dat),
    "traveltime" or "amplitude"; component 0 for all, 1-3 for one."""
    L = _lib()
    syn = np.ascontiguousarray(syn, np.float64)
    nrec, three, nstep = syn.shape
    assert three == 3
    d = None if dat is None else np.ascontiguousarray(dat, np.float64)
    adj = np.zeros_like(syn)
    norms = np.zeros((nrec, 3))
    rc = L.sf3d_adjoint_sources(KINDS[kind], nrec, nstep, dt, t0, ts, te, int(component), syn.ctypes.data,
                                None if d is None else d.ctypes.data, adj.ctypes.data, norms.ctypes.data)
    if rc != 0:
        abi.check()
    return adj, norms


def sum_kernels(kernels, masks=None):
    """(total FP64, total rounded to FP32, norms) of a list of equally sized event kernels."""
    L = _lib()
    ks = [np.ascontiguousarray(k, np.float32).reshape(-1) for k in kernels]
    n = ks[0].size
    assert all(k.size == n for k in ks)
    kp = (ctypes.c_void_p * len(ks))(*[k.ctypes.data for k in ks])
    ms = None
    mp = None
    if masks is not None:
        ms = [np.ascontiguousarray(m, np.float32).reshape(-1) for m in masks]
        mp = (ctypes.c_void_p * len(ms))(*[m.ctypes.data for m in ms])
    total = np.zeros(n)
    total32 = np.zeros(n, np.float32)
    norms = np.zeros(len(ks))
    rc = L.sf3d_sum_kernels(len(ks), n, kp, mp, total.ctypes.data, total32.ctypes.data, norms.ctypes.data)
    if rc != 0:
        abi.check()
    return total, total32, norms
