"""Waveform-misfit gradients through the checkpointed discrete-adjoint C ABI.

The reference obtains sensitivity kernels from a SIMULATION_TYPE=3 run: the
adjoint wavefield, driven by adjoint sources read from SEM/*.adj files, is
propagated next to a backward reconstruction of the forward field, and
compute_kernels.f90:67-226 accumulates rho/kappa/mu kernels, which
save_adjoint_kernels.f90:325-343 scales to relative kernels.  Here the forward
field is recomputed from HBM checkpoints instead (the scheme of
iterate_time_undoatt.F90:29-632) and the adjoint is the exact transpose of the
discrete Newmark step, so the result is the derivative of the discrete misfit:

    J(m) = 1/2 sum_shots sum_receivers sum_n dt |s_n(m) - d_n|^2

with respect to rho, kappa and mu at every GLL point (FP64 accumulation).
``relative_kernels`` converts it to the reference's K_m = m dJ/dm form.

Model perturbations act on the per-point stores (rhostore, kappastore,
mustore) and the mass matrix; the Stacey impedances (rho_vp, rho_vs) are held
fixed, so the gradient is exact for every direction.
"""
from __future__ import annotations

import ctypes
import types

import numpy as np

from . import abi, meshgen
from .meshgen import NGLL3, Block
from .solver import GPUSolver


# ----------------------------------------------------------------- model space
def gll_coordinates(cfg: dict):
    """x, y, z of every GLL point, shape (nspec, 125) each."""
    B = Block(cfg)
    return B.gll_coords(np.arange(B.nspec))


def gaussian_blob(cfg: dict, center, radius: float, amplitude: float) -> np.ndarray:
    """Relative perturbation amplitude * exp(-|x - c|^2 / radius^2) per GLL point (nspec, 125)."""
    x, y, z = gll_coordinates(cfg)
    r2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
    return amplitude * np.exp(-r2 / radius ** 2)


def smooth_direction(cfg: dict, seed: int, corr_len: float = 1000.0) -> np.ndarray:
    """Seeded smooth random field per GLL point (nspec, 125), unit RMS: white noise
    filtered with a Gaussian of the given correlation length."""
    from . import models
    f, origin = models.gaussian_field(cfg, corr_len=corr_len, spacing=corr_len / 8.0, seed=seed, std=1.0,
                                      clip=np.inf)
    x, y, z = gll_coordinates(cfg)
    d = models.sample(f, origin, x.reshape(-1), y.reshape(-1), z.reshape(-1)).reshape(x.shape)
    return d / np.sqrt(np.mean(d ** 2))


def perturbed_database(db: dict, cfg: dict, dln_rho=None, dln_kappa=None, dln_mu=None) -> dict:
    """Copy of ``db`` with rho, kappa, mu scaled by (1 + dln) per GLL point and the
    mass matrices recomputed; the Stacey impedances stay those of ``db``."""
    new = dict(db)
    dtype = db["kappastore"].dtype.type
    for name, d in (("rhostore", dln_rho), ("kappastore", dln_kappa), ("mustore", dln_mu)):
        if d is not None:
            new[name] = (db[name].astype(np.float64) * (1.0 + np.asarray(d, np.float64).reshape(-1))).astype(dtype)
    if dln_rho is not None:
        shape = types.SimpleNamespace(nspec=int(db["nspec"]), nglob=int(db["nglob"]))
        meshgen._mass(cfg, shape, new, dtype)
    return new


def shot_database(db: dict, cfg: dict, shot: int) -> dict:
    """Copy of ``db`` whose source is shot ``shot`` of ``cfg['shots']`` (mesh and
    model shared with ``db``; only the source arrays and stf are recomputed)."""
    new = dict(db)
    meshgen._sources_receivers(shot_config(cfg, shot), Block(cfg), new, db["kappastore"].dtype.type)
    return new


def background_material(cfg: dict):
    """(rho, vp, vs) per GLL point of the background model (layers plus the
    configuration's random perturbation, if any)."""
    from . import models
    if cfg.get("perturbation"):
        return models.perturbed_material(cfg, **cfg["perturbation"])
    lay = np.asarray(cfg["elem_layer"], np.int64)
    L = cfg["layers"]
    return tuple(np.repeat(np.asarray([m[k] for m in L], np.float32)[lay], NGLL3) for k in ("rho", "vp", "vs"))


def true_material(cfg: dict):
    """Background with the configuration's Gaussian blob applied to vs."""
    rho, vp, vs = background_material(cfg)
    b = cfg["blob"]
    blob = gaussian_blob(cfg, b["center"], b["radius"], b["dlnvs"]).reshape(-1)
    return rho, vp, (vs.astype(np.float64) * (1.0 + blob)).astype(np.float32)


def misfit(seis: np.ndarray, obs: np.ndarray, dt: float):
    """L2 waveform misfit (FP64) and dJ/d(seismogram sample), both from (nrec, 3, nstep) traces."""
    r = seis.astype(np.float64) - obs.astype(np.float64)
    return 0.5 * dt * float(np.sum(r * r)), dt * r


def relative_kernels(db: dict, grad: dict) -> dict:
    """K_m = m dJ/dm per GLL point (the reference's rho/kappa/mu kernel convention
    up to the volume weighting, which the per-point gradient already carries)."""
    n = int(db["nspec"])
    return {k: grad[k] * db[s].reshape(n, NGLL3).astype(np.float64)
            for k, s in (("rho", "rhostore"), ("kappa", "kappastore"), ("mu", "mustore"))}


# ----------------------------------------------------------------- device runs
class MisfitGradient:
    """One shot: forward from rest with checkpoints every ``checkpoint_every``
    steps, then the adjoint sweep for a given residual."""

    def __init__(self, db: dict, cfg: dict, checkpoint_every: int = 200, fused: bool = True):
        cfg = dict(cfg)
        cfg["record"] = ("displ",)
        self.cfg, self.db = cfg, db
        self.nstep = int(cfg["nstep"])
        self.solver = GPUSolver(db, cfg, nlength=self.nstep)
        self.L = self.solver.L
        # the fastest stiffness build for this mesh, timed at rest (a few ms)
        self.stiffness_variant, _ = self.solver.autotune_stiffness()
        nbytes = ctypes.c_double()
        rc = self.L.sf3d_gradient_setup(self.solver.mp, self.nstep, int(checkpoint_every), ctypes.addressof(nbytes))
        if rc != 0:
            abi.check()
        self.device_bytes = nbytes.value
        if self.L.sf3d_gradient_set_fused(self.solver.mp, int(bool(fused))) != 0:
            abi.check()

    @property
    def dt(self) -> float:
        return float(self.solver.deltat)

    def set_shot(self, db: dict):
        """Next shot on the same mesh and model: ``db`` carries its sources."""
        self.solver.set_sources(db)

    def forward(self) -> np.ndarray:
        """Seismograms (nrec, 3, nstep) of the forward run from rest."""
        if self.L.sf3d_gradient_forward(self.solver.mp, float(self.solver.deltat)) != 0:
            abi.check()
        self.forward_ms = self.solver.last_timing()["total_ms"]
        return self.solver.seismograms()

    def gradient(self, residual: np.ndarray) -> dict:
        """dJ/drho, dJ/dkappa, dJ/dmu per GLL point (nspec, 125) for dJ/ds = residual (nrec, 3, nstep)."""
        res = np.ascontiguousarray(np.asarray(residual, np.float64).transpose(2, 0, 1), dtype=np.float32)
        if self.L.sf3d_gradient_set_residual(self.solver.mp, res.ctypes.data) != 0:
            abi.check()
        if self.L.sf3d_gradient_backward(self.solver.mp, float(self.solver.deltat)) != 0:
            abi.check()
        self.backward_ms = self.solver.last_timing()["total_ms"]
        n = self.solver.nspec
        out = {k: np.zeros((n, NGLL3), np.float64) for k in ("rho", "kappa", "mu")}
        if self.L.sf3d_gradient_get(self.solver.mp, out["rho"].ctypes.data, out["kappa"].ctypes.data,
                                    out["mu"].ctypes.data) != 0:
            abi.check()
        return out

    def close(self):
        if self.solver is not None:
            self.solver.close()
            self.solver = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shot_config(cfg: dict, shot: int) -> dict:
    """The configuration of one shot of a multi-shot workload (``cfg['shots']``)."""
    c = dict(cfg)
    if cfg.get("shots"):
        c["sources"] = [cfg["shots"][shot]]
    return c


def misfit_gradient(db_of_shot, cfg: dict, observed, checkpoint_every: int = 200, fused: bool = True):
    """Sum over shots of the misfit and its gradient.  ``db_of_shot(i)`` returns the
    database of shot i (same mesh and model, shot i's source); ``observed[i]`` its
    observed traces (nrec, 3, nstep)."""
    total = 0.0
    grad = None
    timing = []
    # one device set-up for every shot (mesh, model, autotuned stiffness build and
    # gradient buffers are shared); each shot replaces only the sources
    mg = MisfitGradient(db_of_shot(0), shot_config(cfg, 0), checkpoint_every, fused)
    try:
        for i, obs in enumerate(observed):
            if i > 0:
                mg.set_shot(db_of_shot(i))
            seis = mg.forward()
            J, res = misfit(seis, obs, mg.dt)
            g = mg.gradient(res)
            timing.append((mg.forward_ms, mg.backward_ms))
            total += J
            if grad is None:
                grad = g
            else:
                for k in grad:
                    grad[k] += g[k]
    finally:
        mg.close()
    return total, grad, timing
