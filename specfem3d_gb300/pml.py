"""C-PML absorbing layers for block meshes: the set-up the reference does in
xgenerate_databases and at the start of xspecfem3D, restated for the GPU path.

* CPML elements and regions (the layers of ``nel`` elements along the x, y and
  bottom faces of the block; the top stays a free surface): faces X/Y/Z_ONLY,
  edges XY/XZ/YZ_ONLY, corners XYZ, numbered as setup/constants.h.in:240-246;
* damping profiles d, K, alpha per GLL point and the separation of the
  parameters that the recursive convolution needs
  (generate_databases/pml_set_local_dampingcoeff.f90:30-1700, 1942-2023):
  K = 1, d = -(NPOWER+1) vp_max log(Rcoef) / (2 width) dist^(1.2 NPOWER),
  alpha = ALPHA_MAX (1 - dist) with ALPHA_MAX = pi f0 (0.9, 1, 1.1 along x, y, z);
* recursive convolution coefficients alpha/beta (9 each), A-bar (5) and the
  strain coefficients (18) per GLL point (specfem3D/prepare_timerun.F90:
  prepare_timerun_pml and compute_convolution_coef; pml_compute_accel_contribution.f90:
  l_parameter_computation; pml_compute_memory_variables.f90: lijk / lx / ly /
  lz_parameter_computation);
* the elastic mass matrix with the PML terms (shared/define_mass_matrices.f90:
  define_mass_matrices_pml_elastic), which replaces the Stacey-augmented one.

Arithmetic is float32 where the reference uses CUSTOM_REAL and float64 where it
writes dble(), so the coefficients are those of a CUSTOM_REAL = 4 build.
"""
from __future__ import annotations

import numpy as np

NGLL3 = 125
X_ONLY, Y_ONLY, Z_ONLY, XY_ONLY, XZ_ONLY, YZ_ONLY, XYZ = 1, 2, 3, 4, 5, 6, 7
NPOWER = 1.0
RCOEF = 0.001
THETA = np.float32(1.0 / 8.0)
f32 = np.float32

# damped axes (x, y, z) of each region
_AXES = {X_ONLY: (1, 0, 0), Y_ONLY: (0, 1, 0), Z_ONLY: (0, 0, 1), XY_ONLY: (1, 1, 0), XZ_ONLY: (1, 0, 1),
         YZ_ONLY: (0, 1, 1), XYZ: (1, 1, 1)}


def block_regions(cfg: dict, nel: int) -> np.ndarray:
    """CPML region (0: interior) of every element of a block configuration with
    ``nel`` element layers along xmin, xmax, ymin, ymax and the bottom."""
    from .meshgen import Block
    B = Block(cfg)
    ex, ey, ez = B.elem_xyz(np.arange(B.nspec))
    ax = (ex < nel) | (ex >= B.nx - nel)
    ay = (ey < nel) | (ey >= B.ny - nel)
    az = ez < nel
    code = np.zeros(B.nspec, np.int32)
    table = {(1, 0, 0): X_ONLY, (0, 1, 0): Y_ONLY, (0, 0, 1): Z_ONLY, (1, 1, 0): XY_ONLY, (1, 0, 1): XZ_ONLY,
             (0, 1, 1): YZ_ONLY, (1, 1, 1): XYZ}
    for key, v in table.items():
        code[(ax == bool(key[0])) & (ay == bool(key[1])) & (az == bool(key[2]))] = v
    return code


def _profile(dist, vp, width):
    """pml_damping_profile_l (pml_set_local_dampingcoeff.f90:1942-1983), CUSTOM_REAL = 4."""
    return f32(-((NPOWER + 1.0) * float(vp) * np.log(RCOEF) / (2.0 * float(width))) * float(dist) ** (1.2 * NPOWER))


def _sep_two(a, b, two):
    """seperate_two_changeable_value (pml_set_local_dampingcoeff.f90:1989-2002)."""
    if a >= b:
        return f32(b + two), b
    return a, f32(a + two)


def _sep_one(a, b, two, four):
    """seperate_two_value_with_one_changeable (:2008-2023): returns the new a."""
    return f32(b + two) if a >= b else f32(b + four)


def damping_profiles(db: dict, xyz: np.ndarray, regions: np.ndarray, f0: float):
    """(K, d, alpha) arrays (3, nspec_cpml, 125) float32 (x, y, z), CPML_to_spec
    (1-based), the layer widths and min_distance_between_CPML_parameter."""
    cpml = np.nonzero(regions)[0]
    reg = regions[cpml]
    n = len(cpml)
    ib = np.asarray(db["ibool"]).reshape(-1, NGLL3).astype(np.int64) - 1
    xs = np.zeros((int(db["nglob"]), 3), np.float32)
    xs[ib.reshape(-1)] = np.asarray(xyz, np.float32).reshape(-1, 3)
    lo, hi = xs.min(axis=0), xs.max(axis=0)
    origin = (lo + hi) / f32(2)
    P = xs[ib[cpml]]                                    # (n, 125, 3)
    # widths: distance from each outer face to the closest CPML point of the regions
    # damped along that axis (:200-260)
    width = np.zeros(3, np.float32)
    inner_lo, inner_hi = lo.copy(), hi.copy()
    for a in range(3):
        damped = np.array([_AXES[r][a] for r in reg], bool)
        if not damped.any():
            continue
        v = P[damped][..., a].reshape(-1)
        pos = v[v - origin[a] > 0]
        neg = v[v - origin[a] <= 0]
        if len(pos):
            inner_hi[a] = pos.min()
        if len(neg):
            inner_lo[a] = neg.max()
        width[a] = max(hi[a] - inner_hi[a], inner_lo[a] - lo[a])
    o_lo = lo + np.array([inner_lo[a] - lo[a] for a in range(3)], np.float32)
    o_hi = hi - np.array([hi[a] - inner_hi[a] for a in range(3)], np.float32)
    rho = np.asarray(db["rhostore"]).reshape(-1, NGLL3)[cpml]
    vp_max = float((np.asarray(db["rho_vp"]).reshape(-1, NGLL3)[cpml] / rho).max())
    amax = np.array([np.pi * f0 * 0.9, np.pi * f0 * 1.0, np.pi * f0 * 1.1], np.float32)
    K = np.ones((3, n, NGLL3), np.float32)
    d = np.zeros((3, n, NGLL3), np.float32)
    al = np.zeros((3, n, NGLL3), np.float32)
    for a in range(3):
        damped = np.array([_AXES[int(r)][a] for r in reg], bool)
        if not damped.any():
            continue
        c = P[damped][..., a]
        absc = np.where(c - origin[a] > 0, c - o_hi[a], o_lo[a] - c).astype(np.float32)
        dist = (absc / width[a]).astype(np.float32)
        dd = (-((NPOWER + 1.0) * float(vp_max) * np.log(RCOEF) / (2.0 * float(width[a])))
              * dist.astype(np.float64) ** (1.2 * NPOWER)).astype(np.float32)
        aa = (amax[a] * (np.float32(1) - dist)).astype(np.float32)
        dd = np.where(dd < 0, np.float32(0), dd)
        d[a][damped] = dd
        al[a][damped] = aa
    # minimum GLL spacing in the layers and the separation threshold (:1379-1445)
    dmin = np.inf
    Pg = P.reshape(n, 5, 5, 5, 3)                       # [e][k][j][i]
    for sl in ((slice(None), slice(0, 4), slice(0, 4), slice(0, 4)),):
        base = Pg[:, :4, :4, :4]
        for d_ in ((0, 0, 1), (0, 1, 0), (1, 0, 0)):
            nb = Pg[:, d_[0]:4 + d_[0], d_[1]:4 + d_[1], d_[2]:4 + d_[2]]
            dmin = min(dmin, float((((base - nb).astype(np.float32)) ** 2).sum(-1).min()))
    dmin = f32(np.sqrt(f32(dmin)))
    mind = f32(amax[0] * dmin / max(width) / f32(8))
    two, four = f32(mind * 2), f32(mind * 4)
    _separate(reg, K, d, al, mind, two, four)
    return K, d, al, (cpml + 1).astype(np.int32), width, float(mind)


def _separate(reg, K, d, al, mind, two, four):
    """Separation of alpha and beta = alpha + d / K where the recursive convolution
    divides by their differences (pml_set_local_dampingcoeff.f90:1446-1940), applied
    to every point of the edge and corner elements at once (each branch of the
    reference's per-point if-chains becomes a mask)."""
    w = np.where
    pairs = {XY_ONLY: (0, 1), XZ_ONLY: (0, 2), YZ_ONLY: (1, 2)}
    for r, (a0, a1) in pairs.items():
        sel = reg == r
        if not sel.any():
            continue
        ax, ay = al[a0][sel], al[a1][sel]
        kx, ky, dx, dy = K[a0][sel], K[a1][sel], d[a0][sel], d[a1][sel]
        close = np.abs(ax - ay) < mind
        ax, ay = w(close & (ax >= ay), ay + two, ax), w(close & (ax < ay), ax + two, ay)
        bx = (ax + dx / kx).astype(np.float32)
        by = (ay + dy / ky).astype(np.float32)
        c1 = np.abs(bx - ay) < mind
        bx = w(c1, w(bx >= ay, ay + two, ay + four), bx).astype(np.float32)
        c2 = np.abs(by - ax) < mind
        by = w(c2, w(by >= ax, ax + two, ax + four), by).astype(np.float32)
        if ((np.abs(ax - ay) < mind) | (np.abs(bx - ay) < mind) | (np.abs(by - ax) < mind)).any():
            raise ValueError("C-PML parameter separation failed on an edge element")
        d[a0][sel] = ((bx - ax) * kx).astype(np.float32)
        al[a0][sel] = ax
        d[a1][sel] = ((by - ay) * ky).astype(np.float32)
        al[a1][sel] = ay
    sel = reg == XYZ
    if not sel.any():
        return
    a = [al[q][sel].astype(np.float32) for q in range(3)]
    k = [K[q][sel] for q in range(3)]
    dd = [d[q][sel] for q in range(3)]
    # the pairs (x, y), (x, z), (y, z) in the reference's order, each moving the third
    # value off the separated pair when it falls too close
    for (i, j, o) in ((0, 1, 2), (0, 2, 1), (1, 2, 0)):
        close = np.abs(a[i] - a[j]) < mind
        gt = a[i] > a[j]
        ai = w(close & gt, a[j] + two, a[i]).astype(np.float32)
        aj = w(close & ~gt, a[i] + two, a[j]).astype(np.float32)
        a[i], a[j] = ai, aj
        mx, mn = np.maximum(a[i], a[j]), np.minimum(a[i], a[j])
        above = close & (a[o] > mx)
        below = close & ~above & (a[o] < mn)
        between = close & ~above & ~below
        ao = a[o].copy()
        ao = w(above & (np.abs(a[o] - mx) < mind), mx + two, ao)
        lowc = below & (np.abs(a[o] - mn) < mind)
        ai, aj = a[i].copy(), a[j].copy()
        ai = w(lowc & gt, a[o] + four, ai)
        aj = w(lowc & gt, a[o] + two, aj)
        aj = w(lowc & ~gt, a[o] + four, aj)
        ai = w(lowc & ~gt, a[o] + two, ai)
        ai2 = w(between & gt, a[j] + four, ai)
        ao = w(between & gt, a[j] + two, ao)
        aj2 = w(between & ~gt, a[i] + four, aj)
        ao = w(between & ~gt, a[i] + two, ao)
        a[i], a[j], a[o] = ai2.astype(np.float32), aj2.astype(np.float32), ao.astype(np.float32)
    if ((np.abs(a[0] - a[1]) < mind) | (np.abs(a[1] - a[2]) < mind) | (np.abs(a[0] - a[2]) < mind)).any():
        raise ValueError("C-PML alpha separation failed on a corner element")
    b = [(a[q] + dd[q] / k[q]).astype(np.float32) for q in range(3)]
    for q in range(3):
        oth = [a[x] for x in range(3) if x != q]
        mx, mn = np.maximum(oth[0], oth[1]), np.minimum(oth[0], oth[1])
        bq = b[q]
        above = bq > mx
        below = ~above & (bq < mn)
        mid = ~above & ~below
        out = bq.copy()
        out = w(above & (np.abs(bq - mx) < mind), mx + two, out)
        out = w(below & (np.abs(bq - mn) < mind), mx + two, out)
        m1 = mid & (np.abs(bq - mx) < mind)
        out = w(m1, mx + two, out)
        m2 = mid & (np.abs(out - mn) < mind)
        out = w(m2, mn + two, out)
        out = w(m2 & (np.abs(out - mx) < mind), mx + two, out)
        b[q] = out.astype(np.float32)
    for q in range(3):
        d[q][sel] = ((b[q] - a[q]) * k[q]).astype(np.float32)
        al[q][sel] = a[q]


# ------------------------------------------------------------------ convolution coefficients
def convolution_coef(bb, dt, mind):
    """compute_convolution_coef (prepare_timerun.F90:926-1030), second-order scheme."""
    bb = f32(bb)
    dt = f32(dt)
    temp = f32(np.exp(f32(-0.5) * bb * dt))
    c0 = f32(temp * temp)
    if abs(bb) >= mind:
        c1 = f32((f32(1) - temp) / bb)
        c2 = f32(c1 * temp)
    else:
        b2 = f32(bb * bb)
        b3 = f32(b2 * bb)
        dt2, dt3, dt4 = f32(dt ** 2), f32(dt ** 3), f32(dt ** 4)
        c1 = f32(f32(0.5) * dt + (-f32(0.125) * dt2 * bb + f32(1 / 48) * dt3 * b2 - f32(1 / 384) * dt4 * b3))
        c2 = f32(f32(0.5) * dt + (-f32(3 / 8) * dt2 * bb + f32(7 / 48) * dt3 * b2 - f32(5 / 128) * dt4 * b3))
    return c0, c1, c2


def l_parameters(kx, dx, ax, ky, dy, ay, kz, dz, az, region):
    """l_parameter_computation (pml_compute_accel_contribution.f90:445-597): A_0 .. A_5."""
    bx, by, bz = f32(ax + dx / kx), f32(ay + dy / ky), f32(az + dz / kz)
    if region == XYZ:
        A0 = f32(kx * ky * kz)
        A1 = A0 * (bx + by + bz - ax - ay - az)
        A2 = A0 * (bx - ax) * (by - ay - ax) + A0 * (by - ay) * (bz - az - ay) + A0 * (bz - az) * (bx - ax - az)
        A3 = A0 * ax ** 2 * (bx - ax) * (by - ax) * (bz - ax) / ((ay - ax) * (az - ax))
        A4 = A0 * ay ** 2 * (bx - ay) * (by - ay) * (bz - ay) / ((ax - ay) * (az - ay))
        A5 = A0 * az ** 2 * (bx - az) * (by - az) * (bz - az) / ((ay - az) * (ax - az))
    elif region == XY_ONLY:
        A0 = f32(kx * ky)
        A1 = A0 * (bx + by - ax - ay)
        A2 = A0 * (bx - ax) * (by - ay - ax) - A0 * (by - ay) * ay
        A3 = A0 * ax ** 2 * (bx - ax) * (by - ax) / (ay - ax)
        A4 = A0 * ay ** 2 * (bx - ay) * (by - ay) / (ax - ay)
        A5 = f32(0)
    elif region == XZ_ONLY:
        A0 = f32(kx * kz)
        A1 = A0 * (bx + bz - ax - az)
        A2 = A0 * (bx - ax) * (-ax) + A0 * (bz - az) * (bx - ax - az)
        A3 = A0 * ax ** 2 * (bx - ax) * (bz - ax) / (az - ax)
        A4 = f32(0)
        A5 = A0 * az ** 2 * (bx - az) * (bz - az) / (ax - az)
    elif region == YZ_ONLY:
        A0 = f32(ky * kz)
        A1 = A0 * (by + bz - ay - az)
        A2 = A0 * (by - ay) * (bz - az - ay) - A0 * (bz - az) * az
        A3 = f32(0)
        A4 = A0 * ay ** 2 * (by - ay) * (bz - ay) / (az - ay)
        A5 = A0 * az ** 2 * (by - az) * (bz - az) / (ay - az)
    elif region == X_ONLY:
        A0 = kx
        A1, A2, A3, A4, A5 = A0 * (bx - ax), -A0 * ax * (bx - ax), A0 * ax ** 2 * (bx - ax), f32(0), f32(0)
    elif region == Y_ONLY:
        A0 = ky
        A1, A2, A3, A4, A5 = A0 * (by - ay), -A0 * ay * (by - ay), f32(0), A0 * ay ** 2 * (by - ay), f32(0)
    else:
        A0 = kz
        A1, A2, A3, A4, A5 = A0 * (bz - az), -A0 * az * (bz - az), f32(0), f32(0), A0 * az ** 2 * (bz - az)
    return tuple(f32(v) for v in (A0, A1, A2, A3, A4, A5))


def lijk_parameters(kx, dx, ax, ky, dy, ay, kz, dz, az, region, index_ijk):
    """lijk_parameter_computation (pml_compute_memory_variables.f90:912-1070): A_0 .. A_3
    (the arguments arrive permuted by the caller; index_ijk names the permutation)."""
    temp = {123: (X_ONLY, Y_ONLY, Z_ONLY, XY_ONLY, XZ_ONLY, YZ_ONLY),
            132: (X_ONLY, Z_ONLY, Y_ONLY, XZ_ONLY, XY_ONLY, YZ_ONLY),
            231: (Z_ONLY, Y_ONLY, X_ONLY, YZ_ONLY, XZ_ONLY, XY_ONLY)}[index_ijk]
    rx, ry, rz, rxy, rxz, ryz = temp
    bx, by, bz = f32(ax + dx / kx), f32(ay + dy / ky), f32(az + dz / kz)
    if region == XYZ:
        A0 = f32(kx * ky / kz)
        A1 = -A0 * (ax - az) * (ax - bx) * (ax - by) / ((ax - ay) * (ax - bz))
        A2 = -A0 * (ay - az) * (ay - bx) * (ay - by) / ((ay - ax) * (ay - bz))
        A3 = -A0 * (bz - az) * (bz - bx) * (bz - by) / ((bz - ax) * (bz - ay))
    elif region == ryz:
        A0 = f32(ky / kz)
        A1 = f32(0)
        A2 = -A0 * (ay - az) * (ay - by) / (ay - bz)
        A3 = -A0 * (bz - az) * (bz - by) / (bz - ay)
    elif region == rxz:
        A0 = f32(kx / kz)
        A1 = -A0 * (ax - az) * (ax - bx) / (ax - bz)
        A2 = f32(0)
        A3 = -A0 * (bz - az) * (bz - bx) / (bz - ax)
    elif region == rxy:
        A0 = f32(kx * ky)
        A1 = -A0 * (ax - bx) * (ax - by) / (ax - ay)
        A2 = -A0 * (ay - bx) * (ay - by) / (ay - ax)
        A3 = f32(0)
    elif region == rx:
        A0 = kx
        A1, A2, A3 = -A0 * (ax - bx), f32(0), f32(0)
    elif region == ry:
        A0 = ky
        A1, A2, A3 = f32(0), -A0 * (ay - by), f32(0)
    else:                                    # rz
        A0 = f32(1) / kz
        A1, A2, A3 = f32(0), f32(0), -A0 * (bz - az)
    return tuple(f32(v) for v in (A0, A1, A2, A3))


def lq_parameters(k, d, a, region, axis):
    """lx / ly / lz_parameter_computation (pml_compute_memory_variables.f90:1076-1283)."""
    damped = {0: (XYZ, XZ_ONLY, XY_ONLY, X_ONLY), 1: (XYZ, YZ_ONLY, XY_ONLY, Y_ONLY),
              2: (XYZ, YZ_ONLY, XZ_ONLY, Z_ONLY)}[axis]
    if region in damped:
        b = f32(a + d / k)
        return f32(k), f32(-k * (a - b))
    return f32(1), f32(0)


def coefficients(K, d, al, regions_cpml, dt, mind):
    """Per GLL point of every CPML element: alpha (9), beta (9), A-bar (5), strain (18)
    coefficients (prepare_timerun.F90, prepare_timerun_pml), arrays (n, 125, m).
    The per-point routines above applied to all points of a region at once."""
    n = K.shape[1]
    ca = np.zeros((n, NGLL3, 9), np.float32)
    cb = np.zeros((n, NGLL3, 9), np.float32)
    cab = np.zeros((n, NGLL3, 5), np.float32)
    cs = np.zeros((n, NGLL3, 18), np.float32)
    for q in range(3):
        for r, v in enumerate(_convolution_coef_v(al[q], dt, mind)):
            ca[..., 3 * q + r] = v
        for r, v in enumerate(_convolution_coef_v((al[q] + d[q] / K[q]).astype(np.float32), dt, mind)):
            cb[..., 3 * q + r] = v
    kx, ky, kz = K
    dx, dy, dz = d
    ax, ay, az = al
    for region in range(1, 8):
        sel = regions_cpml == region
        if not sel.any():
            continue
        args = [x[sel] for x in (kx, dx, ax, ky, dy, ay, kz, dz, az)]
        lp = _vec(l_parameters, args, region)
        cab[sel] = np.stack(lp[1:], axis=-1)
        (Kx, Dx, Ax, Ky, Dy, Ay, Kz, Dz, Az) = args
        cs[sel, :, 0:4] = np.stack(_vec(lijk_parameters, [Kz, Dz, Az, Ky, Dy, Ay, Kx, Dx, Ax], region, 231), -1)
        cs[sel, :, 4:8] = np.stack(_vec(lijk_parameters, [Kx, Dx, Ax, Kz, Dz, Az, Ky, Dy, Ay], region, 132), -1)
        cs[sel, :, 8:12] = np.stack(_vec(lijk_parameters, [Kx, Dx, Ax, Ky, Dy, Ay, Kz, Dz, Az], region, 123), -1)
        cs[sel, :, 12:14] = np.stack(_vec(lq_parameters, [Kx, Dx, Ax], region, 0), -1)
        cs[sel, :, 14:16] = np.stack(_vec(lq_parameters, [Ky, Dy, Ay], region, 1), -1)
        cs[sel, :, 16:18] = np.stack(_vec(lq_parameters, [Kz, Dz, Az], region, 2), -1)
    return ca, cb, cab, cs


def _vec(fn, arrays, *extra):
    """fn (a per-point routine written with float32 scalars) on float32 arrays: the
    same operations elementwise (numpy float32 arithmetic is per-operation IEEE)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        out = fn(*arrays, *extra)
    return [np.broadcast_to(np.asarray(v, np.float32), arrays[0].shape).astype(np.float32) for v in out]


def _convolution_coef_v(bb, dt, mind):
    """compute_convolution_coef on an array of b values."""
    bb = np.asarray(bb, np.float32)
    dt = f32(dt)
    temp = np.exp(f32(-0.5) * bb * dt).astype(np.float32)
    c0 = (temp * temp).astype(np.float32)
    big = np.abs(bb) >= mind
    with np.errstate(divide="ignore", invalid="ignore"):
        c1 = ((f32(1) - temp) / bb).astype(np.float32)
    c2 = (c1 * temp).astype(np.float32)
    b2 = (bb * bb).astype(np.float32)
    b3 = (b2 * bb).astype(np.float32)
    dt2, dt3, dt4 = f32(dt ** 2), f32(dt ** 3), f32(dt ** 4)
    t1 = (f32(0.5) * dt + (-f32(0.125) * dt2 * bb + f32(1 / 48) * dt3 * b2 - f32(1 / 384) * dt4 * b3)).astype(np.float32)
    t2 = (f32(0.5) * dt + (-f32(3 / 8) * dt2 * bb + f32(7 / 48) * dt3 * b2 - f32(5 / 128) * dt4 * b3)).astype(np.float32)
    return c0, np.where(big, c1, t1).astype(np.float32), np.where(big, c2, t2).astype(np.float32)


def pml_mass(db: dict, regions: np.ndarray, cpml_to_spec, K, d, dt: float) -> np.ndarray:
    """Elastic mass matrix with the PML terms (define_mass_matrices.f90:
    define_mass_matrices_pml_elastic): interior elements rho J w, CPML elements
    rho J w (prod K + dt/2 sum_a d_a prod_{b != a} K_b) over the region's damped axes."""
    from .meshgen import WGLL
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    irr = np.asarray(db["irregular_element_number"])
    w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1)
    jel = np.empty((nspec, NGLL3), np.float64)
    reg = irr == 0
    jel[reg] = np.float32(db["jacobian_regular"])
    if (~reg).any():
        jel[~reg] = np.asarray(db["jacobian"]).reshape(-1, NGLL3)[irr[~reg] - 1]
    rho = np.asarray(db["rhostore"]).reshape(nspec, NGLL3).astype(np.float64)
    ib = np.asarray(db["ibool"]).reshape(nspec, NGLL3).astype(np.int64) - 1
    fac = np.ones((nspec, NGLL3))
    for e_c, ispec in enumerate(np.asarray(cpml_to_spec) - 1):
        ax = _AXES[int(regions[ispec])]
        kk = [K[a, e_c].astype(np.float64) for a in range(3)]
        dd = [d[a, e_c].astype(np.float64) for a in range(3)]
        used = [a for a in range(3) if ax[a]]
        prod = np.ones(NGLL3)
        for a in used:
            prod = prod * kk[a]
        s = np.zeros(NGLL3)
        for a in used:
            t = dd[a].copy()
            for b in used:
                if b != a:
                    t = t * kk[b]
            s += t
        fac[ispec] = prod + s * dt / 2.0
    terms = (jel * w3[None, :] * rho * fac).astype(np.float32).astype(np.float64)
    rmass = np.bincount(ib.reshape(-1), weights=terms.reshape(-1), minlength=nglob).astype(np.float32)
    rmass[rmass <= 0] = 1
    return rmass


def setup(db: dict, cfg: dict, nel: int = 2, f0: float | None = None) -> dict:
    """Copy of a block database with C-PML layers of ``nel`` elements on the x, y and
    bottom faces instead of Stacey conditions: regions, damping profiles, coefficients
    and the PML mass matrix (the outer faces stay in the database: the boundary
    condition zeroes the field there)."""
    from .meshgen import element_coordinates
    out = dict(db)
    regions = block_regions(cfg, nel)
    xyz = element_coordinates(cfg)
    if f0 is None:
        f0 = float(cfg["sources"][0].get("f0", 1.0))
    K, d, al, c2s, width, mind = damping_profiles(db, xyz, regions, f0)
    ca, cb, cab, cs = coefficients(K, d, al, regions[c2s - 1], float(cfg["dt"]), mind)
    rmass = pml_mass(db, regions, c2s, K, d, float(cfg["dt"]))
    inv = (np.float32(1) / rmass).astype(np.float32)
    out.update(pml=1, stacey=0, cpml_regions=regions, cpml_to_spec=c2s, is_cpml=(regions > 0).astype(np.int32),
               pml_K=K, pml_d=d, pml_alpha=al, pml_width=width, pml_min_distance=mind,
               pml_coef_alpha=ca, pml_coef_beta=cb, pml_coef_abar=cab, pml_coef_strain=cs,
               rmass=rmass, rmassx=inv, rmassy=inv.copy(), rmassz=inv.copy())
    return out
