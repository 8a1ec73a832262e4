"""Constant-Q attenuation with N_SLS = 3 standard linear solids.

Computes the arrays the viscoelastic stiffness kernel consumes, following
shared/get_attenuation_model.f90 and specfem3D/prepare_attenuation.f90:

* the absorption band from the mesh's minimum resolved period
  (shared/check_mesh_resolution.f90:200-280; get_attenuation_periods,
  get_attenuation_tau_sigma, get_attenuation_source_freq :702-810);
* strain relaxation times tau_eps fitted to a constant Q over 100 log-spaced
  frequencies by a Nelder-Mead search (attenuation_invert_by_simplex
  :976-1058; the search is scipy's Matlab-compatible fmin with the same
  coefficients, initial simplex and 1e-4 tolerances);
* factor_common(_kappa), the unrelaxed-modulus scale factors
  (get_attenuation_property_values / get_attenuation_scale_factor :599-694)
  and the second-order Runge-Kutta coefficients alpha/beta/gamma
  (get_attenuation_memory_values :464-493).
"""
from __future__ import annotations

import math

import numpy as np
from scipy.optimize import fmin

N_SLS = 3
NGLL3 = 125
ATTENUATION_COMP_MAXIMUM = 9000.0
ATTENUATION_F0_REFERENCE = 18.0  # the reference's default Par_file value
PI_SIMPLEX = 3.14159265358979


def min_resolved_period(cfg: dict, db: dict) -> float:
    """Largest per-element resolved period (single precision): (max edge /4) / min(vp,vs) * 5
    (check_mesh_resolution.f90, get_elem_minmaxsize: longest of the 12 edges).
    Meshes other than blocks give the edge per element as db["elem_size_max"]."""
    f32 = np.float32
    nspec = db["nspec"]
    if "elem_size_max" in db:
        emax = np.asarray(db["elem_size_max"], f32)
        return _resolved(db, emax)
    nx, ny = cfg["nx"], cfg["ny"]
    xl = np.array([cfg["x0"] + (cfg["x1"] - cfg["x0"]) * e / nx for e in range(nx + 1)])
    yl = np.array([cfg["y0"] + (cfg["y1"] - cfg["y0"]) * e / ny for e in range(ny + 1)])
    zl = np.asarray(cfg["zlev"])
    dx = (xl[1:] - xl[:-1]).astype(f32)
    dy = (yl[1:] - yl[:-1]).astype(f32)
    dz = (zl[1:] - zl[:-1]).astype(f32)
    e = np.arange(nspec)
    emax = np.maximum(np.maximum(dx[e % nx], dy[(e // nx) % ny]), dz[e // (nx * ny)]).astype(f32)
    return _resolved(db, emax)


def _resolved(db: dict, emax) -> float:
    f32 = np.float32
    nspec = db["nspec"]
    kap = db["kappastore"].reshape(nspec, NGLL3)
    mu = db["mustore"].reshape(nspec, NGLL3)
    rho = db["rhostore"].reshape(nspec, NGLL3)
    vp = np.sqrt((kap + f32(4.0 / 3.0) * mu) / rho).astype(f32)
    vs = np.sqrt(mu / rho).astype(f32)
    vmin = np.minimum(vp.min(axis=1), vs.min(axis=1))
    return float(((emax / f32(4.0)) / vmin * f32(5.0)).max())


def band(min_resolved: float):
    minp = float(np.float32(np.float32(0.99) * np.float32(min_resolved)))
    maxp = minp * 10.0 ** 1.75
    f1, f2 = 1.0 / maxp, 1.0 / minp
    e1, e2 = math.log10(f1), math.log10(f2)
    d = (e2 - e1) / (N_SLS - 1.0)
    tau_sigma = np.array([1.0 / (PI_SIMPLEX * 2.0 * 10 ** (e1 + i * d)) for i in range(N_SLS)])
    f_c = 10.0 ** (0.5 * (math.log10(f1) + math.log10(f2)))
    return tau_sigma, f_c, minp, maxp


def tau_eps_for_q(Q: float, tau_sigma, minp: float, maxp: float):
    f1, f2 = 1.0 / maxp, 1.0 / minp
    e1, e2 = math.log10(f1), math.log10(f2)
    logf = e1 + np.arange(100) * (e2 - e1) / 99.0
    w = 2.0 * PI_SIMPLEX * 10.0 ** logf
    iQ = 1.0 / Q
    ts = np.asarray(tau_sigma)

    def misfit(te):
        den = 1.0 + (w[:, None] ** 2) * ts[None, :] ** 2
        A = ((1.0 + (w[:, None] ** 2) * te[None, :] * ts[None, :]) / den).sum(axis=1)
        B = (w[:, None] * (te[None, :] - ts[None, :]) / den).sum(axis=1)
        return float(np.sum(np.abs(B / A - iQ) / iQ))

    x0 = ts + ts * 2.0 / Q
    return fmin(misfit, x0, xtol=1e-4, ftol=1e-4, maxiter=200 * N_SLS, maxfun=200 * N_SLS, disp=False)


def factors(Q: float, tau_sigma, f_c: float, minp: float, maxp: float, f0_ref: float = ATTENUATION_F0_REFERENCE):
    Q = min(max(float(Q), 1.0), ATTENUATION_COMP_MAXIMUM)
    te = tau_eps_for_q(Q, tau_sigma, minp, maxp)
    ratio = te / tau_sigma
    one_minus_sum_beta = float(ratio.sum())
    beta = ratio - 1.0
    mu0 = 1.0 + 2.0 * math.log(f_c / f0_ref) / (math.pi * Q)
    x1 = 1.0 + np.sum(beta / N_SLS)
    x2 = 1.0 + np.sum(beta / (1.0 + 1.0 / (2.0 * math.pi * f_c * tau_sigma) ** 2) / N_SLS)
    scale = (x1 / x2) * mu0
    if not 0.5 <= scale <= 1.5:
        raise ValueError("unreliable correction factor in attenuation model")
    return beta, one_minus_sum_beta, scale


def memory_values(tau_sigma_f32, dt):
    """alpha/beta/gamma of the second-order RK memory-variable update (FP32)."""
    f = np.float32
    ts = np.asarray(tau_sigma_f32, f)
    d = f(dt)
    ti = f(-1) / ts
    d2, d3, d4 = d * d, d * d * d, d * d * d * d
    al = f(1.0) + d * ti + d2 * (ti * ti) / f(2) + d3 * (ti * ti * ti) / f(6) + d4 * (ti * ti * ti * ti) / f(24)
    be = d / f(2) + d2 * ti / f(3) + d3 * (ti * ti) / f(8) + d4 * (ti * ti * ti) / f(24)
    ga = d / f(2) + d2 * ti / f(6) + d3 * (ti * ti) / f(24)
    return al.astype(f), be.astype(f), ga.astype(f)


def setup(cfg: dict, db: dict) -> dict:
    """Attenuation arrays for a layered block; mustore/kappastore become unrelaxed."""
    f32 = np.float32
    tau_sigma, f_c, minp, maxp = band(min_resolved_period(cfg, db))
    tau_f = tau_sigma.astype(f32)
    tauinv = (f32(1) / tau_f).astype(np.float64)
    nspec = db["nspec"]
    lay = np.asarray(cfg["elem_layer"], np.int64)
    nl = len(cfg["layers"])
    fcm_l = np.zeros((nl, N_SLS), f32)
    fck_l = np.zeros((nl, N_SLS), f32)
    smu_l = np.ones(nl, f32)
    skap_l = np.ones(nl, f32)
    for li, m in enumerate(cfg["layers"]):
        bm, om, sm = factors(float(f32(m["Qmu"])), tau_sigma, f_c, minp, maxp)
        bk, ok, sk = factors(float(f32(m.get("Qkappa", 9999.0))), tau_sigma, f_c, minp, maxp)
        fcm_l[li] = ((2.0 * bm * tauinv) / om).astype(f32)
        fck_l[li] = ((bk * tauinv) / ok).astype(f32)
        smu_l[li], skap_l[li] = f32(sm), f32(sk)
    # (N_SLS,5,5,5,NSPEC): sls fastest
    fcm = np.broadcast_to(fcm_l[lay][:, None, :], (nspec, NGLL3, N_SLS)).reshape(-1)
    fck = np.broadcast_to(fck_l[lay][:, None, :], (nspec, NGLL3, N_SLS)).reshape(-1)
    smu = np.repeat(smu_l[lay], NGLL3)
    skap = np.repeat(skap_l[lay], NGLL3)
    al, be, ga = memory_values(tau_f, cfg["dt"])
    return dict(factor_common=np.ascontiguousarray(fcm), factor_common_kappa=np.ascontiguousarray(fck),
                mustore=(db["mustore"] * smu).astype(f32), kappastore=(db["kappastore"] * skap).astype(f32),
                # relaxed moduli and the unrelaxed scaling, as the databases keep
                # them (mustore / kappastore, attenuation.bin scale_factor(_kappa))
                mustore_relaxed=db["mustore"], kappastore_relaxed=db["kappastore"],
                scale_factor=smu.astype(f32), scale_factor_kappa=skap.astype(f32),
                alphaval=al, betaval=be, gammaval=ga, tau_sigma=tau_f, f_c_source=f_c, attenuation=1)
