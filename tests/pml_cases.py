"""Block configurations for the C-PML tests: a homogeneous block of 312.5 m cubes
with a moment-tensor source and four surface receivers inside the layers'
interior, and the same source and receivers in a block three times as wide and
deep (its boundaries too far to reflect within the compared time window)."""
import numpy as np

H = 312.5


def block(n: int, nz: int, off: float, nstep: int, dt: float = 0.008):
    from specfem3d_gb300 import configs
    M = configs.random_moment_tensor(np.random.default_rng(3))
    cfg = dict(nx=n, ny=n, x0=-off, x1=n * H - off, y0=-off, y1=n * H - off,
               zlev=[float(-nz * H + q * H) for q in range(nz + 1)], elem_layer=None,
               layers=[dict(rho=2400.0, vp=3000.0, vs=1700.0)], dt=None, nstep=nstep, stacey=True,
               sources=[dict(type="cmt", x=1875.0 + 17, y=1875.0 - 11, z=-937.5 + 23, M=M, stf="ricker", f0=2.0)],
               receivers=[(1875.0 + dx, 1875.0 + dy, 0.0) for dx in (-500.0, 300.0) for dy in (-400.0, 450.0)])
    cfg = configs.finish(cfg)
    cfg["dt"] = dt
    return cfg
