"""Velocity-model helpers for the synthetic workloads.

``gaussian_perturbation`` builds the seeded, Gaussian-correlated relative
perturbation of the benchmark definition: white noise on a regular grid,
filtered in the Fourier domain with a Gaussian of the given correlation length,
scaled to a 2.5 % standard deviation and clipped at +-5 %, then sampled at the
GLL points by trilinear interpolation.
"""
from __future__ import annotations

import numpy as np

from .meshgen import Block, NGLL3


def gaussian_field(cfg: dict, corr_len: float = 1000.0, spacing: float = 100.0, seed: int = 7,
                   std: float = 0.025, clip: float = 0.05):
    x0, x1, y0, y1 = cfg["x0"], cfg["x1"], cfg["y0"], cfg["y1"]
    z0, z1 = float(cfg["zlev"][0]), float(cfg["zlev"][-1])
    # the generation grid spans at least eight correlation lengths per axis, so
    # the normalisation does not depend on the size of the block
    span = 8.0 * corr_len
    nx = int(np.ceil(max(x1 - x0, span) / spacing)) + 1
    ny = int(np.ceil(max(y1 - y0, span) / spacing)) + 1
    nz = int(np.ceil(max(z1 - z0, span) / spacing)) + 1
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((nz, ny, nx))
    kx = np.fft.fftfreq(nx, d=spacing) * 2 * np.pi
    ky = np.fft.fftfreq(ny, d=spacing) * 2 * np.pi
    kz = np.fft.fftfreq(nz, d=spacing) * 2 * np.pi
    k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    filt = np.exp(-k2 * corr_len ** 2 / 4.0)
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * filt))
    f = f / f.std() * std
    f = np.clip(f, -clip, clip)
    return f, (x0, y0, z0, spacing)


def sample(field, origin, x, y, z):
    """Trilinear interpolation of the grid field at points (x, y, z)."""
    x0, y0, z0, h = origin
    nz, ny, nx = field.shape
    fx = np.clip((x - x0) / h, 0, nx - 1 - 1e-9)
    fy = np.clip((y - y0) / h, 0, ny - 1 - 1e-9)
    fz = np.clip((z - z0) / h, 0, nz - 1 - 1e-9)
    ix, iy, iz = fx.astype(np.int64), fy.astype(np.int64), fz.astype(np.int64)
    tx, ty, tz = fx - ix, fy - iy, fz - iz
    out = np.zeros_like(fx)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (tx if dx else 1 - tx) * (ty if dy else 1 - ty) * (tz if dz else 1 - tz)
                out += w * field[iz + dz, iy + dy, ix + dx]
    return out


def perturbed_material(cfg: dict, corr_len: float = 1000.0, seed: int = 7):
    """(rho, vp, vs) per GLL point (125*nspec, float32): layer values, with the
    relative perturbation applied to vp and vs of the solid elements."""
    B = Block(cfg)
    lay = np.asarray(cfg["elem_layer"], np.int64)
    L = cfg["layers"]
    rho = np.repeat(np.asarray([m["rho"] for m in L], np.float64)[lay], NGLL3)
    vp = np.repeat(np.asarray([m["vp"] for m in L], np.float64)[lay], NGLL3)
    vs = np.repeat(np.asarray([m["vs"] for m in L], np.float64)[lay], NGLL3)
    field, origin = gaussian_field(cfg, corr_len=corr_len, seed=seed)
    pert = np.zeros_like(vp)
    chunk = 1 << 16
    for s in range(0, B.nspec, chunk):
        e = np.arange(s, min(B.nspec, s + chunk))
        x, y, z = B.gll_coords(e)
        pert[s * NGLL3:(s + len(e)) * NGLL3] = sample(field, origin, x.reshape(-1), y.reshape(-1), z.reshape(-1))
    solid = vs > 0
    vp = np.where(solid, vp * (1 + pert), vp)
    vs = np.where(solid, vs * (1 + pert), vs)
    return rho.astype(np.float32), vp.astype(np.float32), vs.astype(np.float32)


# ----------------------------------------------------------------------------- anisotropy
_VOIGT = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]      # 1..6 = xx yy zz yz xz xy
ANISO_NAMES = ["c11store", "c12store", "c13store", "c14store", "c15store", "c16store", "c22store", "c23store",
               "c24store", "c25store", "c26store", "c33store", "c34store", "c35store", "c36store", "c44store",
               "c45store", "c46store", "c55store", "c56store", "c66store"]
_UPPER = [(a, b) for a in range(6) for b in range(a, 6)]       # c11 c12 .. c16 c22 .. c66


def tilted_ti(rho, vp, vs, eps: float = 0.05, gamma: float = 0.04, delta: float = 0.02,
              tilt_deg: float = 30.0, azimuth_deg: float = 20.0) -> np.ndarray:
    """(n, 6, 6) Voigt stiffness of a tilted transversely isotropic medium: the
    hexagonal tensor of Thomsen's parameters about a symmetry axis tilted from
    vertical by tilt_deg in the vertical plane at azimuth_deg (C33 = rho vp^2,
    C44 = rho vs^2, C11 = C33 (1 + 2 eps), C66 = C44 (1 + 2 gamma),
    C13 = sqrt((C33 - C44)(C33 (1 + 2 delta) - C44)) - C44)."""
    rho, vp, vs = (np.asarray(v, np.float64).reshape(-1) for v in (rho, vp, vs))
    c33, c44 = rho * vp * vp, rho * vs * vs
    c11, c66 = c33 * (1 + 2 * eps), c44 * (1 + 2 * gamma)
    c13 = np.sqrt(np.maximum((c33 - c44) * (c33 * (1 + 2 * delta) - c44), 0.0)) - c44
    C = np.zeros((len(rho), 6, 6))
    C[:, 0, 0] = C[:, 1, 1] = c11
    C[:, 2, 2] = c33
    C[:, 0, 1] = C[:, 1, 0] = c11 - 2 * c66
    C[:, 0, 2] = C[:, 2, 0] = C[:, 1, 2] = C[:, 2, 1] = c13
    C[:, 3, 3] = C[:, 4, 4] = c44
    C[:, 5, 5] = c66
    t, a = np.radians(tilt_deg), np.radians(azimuth_deg)
    Ry = np.array([[np.cos(t), 0, np.sin(t)], [0, 1, 0], [-np.sin(t), 0, np.cos(t)]])
    Rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    R = Rz @ Ry
    # Voigt -> 4th order tensor, rotate, back
    T = np.zeros((len(rho), 3, 3, 3, 3))
    for I, (i, j) in enumerate(_VOIGT):
        for J, (k, l) in enumerate(_VOIGT):
            for (p, q) in {(i, j), (j, i)}:
                for (r, s) in {(k, l), (l, k)}:
                    T[:, p, q, r, s] = C[:, I, J]
    T = np.einsum("ip,jq,kr,ls,npqrs->nijkl", R, R, R, R, T, optimize=True)
    out = np.zeros_like(C)
    for I, (i, j) in enumerate(_VOIGT):
        for J, (k, l) in enumerate(_VOIGT):
            out[:, I, J] = T[:, i, j, k, l]
    return out


def make_anisotropic(db: dict, voigt: np.ndarray) -> dict:
    """Copy of db with ANISOTROPY on: the 21 c_ij per GLL point from (npt, 6, 6)
    Voigt matrices (c11 c12 ... c66, upper triangle row by row)."""
    out = dict(db)
    v = np.asarray(voigt, np.float64)
    for name, (a, b) in zip(ANISO_NAMES, _UPPER):
        out[name] = v[:, a, b].astype(np.float32)
    out["anisotropy"] = 1
    return out


def isotropic_voigt(kappa, mu) -> np.ndarray:
    """(n, 6, 6) Voigt matrices of isotropic media (lambda + 2 mu, lambda, mu)."""
    k, m = (np.asarray(v, np.float64).reshape(-1) for v in (kappa, mu))
    lam = k - 2.0 * m / 3.0
    C = np.zeros((len(k), 6, 6))
    for i in range(3):
        for j in range(3):
            C[:, i, j] = lam
        C[:, i, i] = lam + 2 * m
        C[:, 3 + i, 3 + i] = m
    return C
