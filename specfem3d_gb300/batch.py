"""Many shots on one mesh through the sf3d_batch_* C ABI.

The reference runs independent shots as separate simulations
(NUMBER_OF_SIMULTANEOUS_RUNS, src/shared/parallel.f90:2171-2260).  Here the
shots of a configuration (``cfg['shots']``) share one prepared mesh; their
wavefields are stacked shot-innermost on the device and advance together.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi, meshgen
from .meshgen import NGLL3, Block
from .solver import GPUSolver


def shot_sources(db: dict, cfg: dict):
    """(ispec_selected_source (S,), sourcearrays (S,3,5,5,5) Fortran layout, stf (S, nstep))
    of every shot of ``cfg['shots']`` on the mesh of ``db``."""
    shots = cfg["shots"]
    S = len(shots)
    B = Block(cfg)
    dtype = db["kappastore"].dtype.type
    isp = np.zeros(S, np.int32)
    sa = np.zeros((NGLL3, 3, S), np.float32)  # Fortran (S, 3, 125): shot index fastest
    stf = np.zeros((S, int(cfg["nstep"])))
    for s, shot in enumerate(shots):
        d = {k: db[k] for k in ("irregular_element_number", "xix", "xiy", "xiz", "etax", "etay", "etaz",
                                 "gammax", "gammay", "gammaz", "xix_regular")}
        c = dict(cfg)
        c["sources"] = [shot]
        c["receivers"] = []
        meshgen._sources_receivers(c, B, d, dtype)
        isp[s] = d["ispec_selected_source"][0]
        sa[:, :, s] = np.asarray(d["sourcearrays"], np.float32).reshape(NGLL3, 3)
        stf[s] = np.asarray(d["stf"]).reshape(-1)
    return isp, sa.reshape(-1), stf


class BatchSolver:
    """All shots of ``cfg['shots']`` on the mesh of ``db`` (elastic, no attenuation)."""

    def __init__(self, db: dict, cfg: dict, nlength: int | None = None):
        self.cfg = cfg
        self.nstep = int(cfg["nstep"])
        self.nlength = int(nlength or self.nstep)
        self.solver = GPUSolver(db, cfg, nlength=1)
        self.L, self.mp = self.solver.L, self.solver.mp
        self.nshots = len(cfg["shots"])
        self.nrec = int(db["nrec"])
        self.nglob = int(db["nglob"])
        self.deltat = self.solver.deltat
        isp, sa, stf = shot_sources(db, cfg)
        stf_f = np.ascontiguousarray(stf.T)  # Fortran (S, nstep): shot index fastest
        nbytes = ctypes.c_double()
        rc = self.L.sf3d_batch_prepare(self.mp, self.nshots, isp.ctypes.data, sa.ctypes.data, stf_f.ctypes.data,
                                       self.nstep, self.nlength, ctypes.addressof(nbytes))
        if rc != 0:
            abi.check()
        self.device_bytes = nbytes.value
        self.it = 1

    def set_tiling(self, shots_per_block: int, elements_per_block: int, shots_per_thread: int = 1):
        if self.L.sf3d_batch_set_tiling(self.mp, int(shots_per_block), int(elements_per_block),
                                        int(shots_per_thread)) != 0:
            abi.check()

    def set_halves(self, halves: int):
        """1: all shots in every launch; 2: two shot halves overlapped on two streams."""
        if self.L.sf3d_batch_set_halves(self.mp, int(halves)) != 0:
            abi.check()

    def autotune(self, reps: int = 3) -> dict:
        """Time every stiffness kernel and tiling at rest (per-point kernels: shots per
        thread x shots per CTA x elements per CTA; pencil kernel: shots per CTA) and keep
        the fastest; shots_per_thread 0 in the result is the pencil kernel."""
        ms = (ctypes.c_float * 27)()
        sb, eb, spt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        if self.L.sf3d_batch_autotune(self.mp, int(reps), ms, ctypes.addressof(sb), ctypes.addressof(eb),
                                      ctypes.addressof(spt)) != 0:
            abi.check()
        table = {}
        for v, t in enumerate((1, 4)):
            for a, s in enumerate((1, 2, 4, 8)):
                for b, e in enumerate((1, 2, 4)):
                    x = ms[(v * 4 + a) * 3 + b]
                    if x >= 0:
                        table[f"{t}x{s}x{e}"] = round(float(x), 4)
        for q, lanes in enumerate((8, 16, 32)):
            if ms[24 + q] >= 0:
                table[f"pencil{lanes}"] = round(float(ms[24 + q]), 4)
        return {"shots_per_thread": spt.value, "shots_per_block": sb.value, "elements_per_block": eb.value,
                "kernel": "pencil" if spt.value == 0 else "per-point", "ms": table}

    def run(self, nsteps: int, steps_per_graph: int = 50) -> float:
        """nsteps steps of every shot; returns the device time in ms."""
        rc = self.L.sf3d_batch_iterate(self.mp, self.it, self.it + nsteps - 1, float(self.deltat),
                                       int(steps_per_graph))
        if rc != 0:
            abi.check()
        self.it += nsteps
        ms, n = ctypes.c_float(), ctypes.c_int()
        self.L.sf3d_batch_timing(self.mp, ctypes.addressof(ms), ctypes.addressof(n))
        self.last_launches = n.value
        return ms.value

    def seismograms(self) -> np.ndarray:
        """(nshots, nrec, 3, nlength) displacement traces."""
        out = np.zeros(3 * self.nrec * self.nshots * self.nlength, np.float32)
        if self.nrec:
            if self.L.sf3d_batch_get_seismograms(self.mp, out.ctypes.data) != 0:
                abi.check()
        return out.reshape(self.nlength, self.nshots, self.nrec, 3).transpose(1, 2, 3, 0)

    def displacement(self) -> np.ndarray:
        """(nshots, NGLOB, 3) displacement of every shot."""
        out = np.zeros(3 * self.nglob * self.nshots, np.float32)
        if self.L.sf3d_batch_get_displ(self.mp, out.ctypes.data) != 0:
            abi.check()
        return out.reshape(self.nglob, 3, self.nshots).transpose(2, 0, 1)

    def close(self):
        if self.solver is not None:
            self.solver.close()
            self.solver = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
