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
