"""Mesh databases of a regular layered block, in the layouts the GPU entry points take.

This module plays the role of xmeshfem3D + xgenerate_databases + the solver's
setup (read_mesh_databases, setup_sources_receivers, prepare_timerun) for the
block meshes of the benchmark workloads, producing exactly the arrays that the
Fortran solver hands to prepare_constants_device / prepare_fields_elastic_device.
It is vectorised numpy written for structured blocks:

* global numbering: the reference sorts GLL coordinates (shared/get_global.f90)
  and renumbers points by first appearance in element order
  (get_global_indirect_addressing, shared/get_global.f90:80-141).  On a
  structured block the first element containing a grid point is known in closed
  form, so the same numbering is computed here without a sort;
* regular/irregular split (generate_databases/calc_jacobian.f90:184-360) and
  the metric of axis-aligned hexahedra;
* materials (generate_databases/get_model.F90:289-301);
* mass matrices with the Stacey term (shared/define_mass_matrices.f90:28-442,
  specfem3D/prepare_timerun.F90:246-388);
* absorbing faces in the order xmin, xmax, ymin, ymax, bottom[, top]
  (generate_databases/get_absorbing_boundary.F90);
* source/receiver location by closest GLL point then local coordinates
  (specfem3D/locate_point.f90), Lagrange interpolants and moment-tensor
  source arrays (specfem3D/compute_arrays_source.f90:29-149);
* source time function tables (specfem3D/comp_source_time_function.f90) with
  t0 from specfem3D/setup_sources_receivers.f90:482-491.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

NGLL = 5
NGLL3 = 125
XIGLL = np.array([-1.0, -math.sqrt(3.0 / 7.0), 0.0, math.sqrt(3.0 / 7.0), 1.0])
WGLL = np.array([0.1, 49.0 / 90.0, 32.0 / 45.0, 49.0 / 90.0, 0.1])


# ----------------------------------------------------------------------------
# GLL interpolation
# ----------------------------------------------------------------------------

def _legendre(z, n):
    p1, p2 = 1.0, z
    if n == 0:
        return 1.0
    for k in range(1, n):
        p1, p2 = p2, ((2 * k + 1) * z * p2 - k * p1) / (k + 1)
    return p2


def derivation_matrices():
    """hprime_xx(i2,i1) = l'_{i1}(xi_{i2}) and hprimewgll_xx = hprime * w(i2), column-major
    (shared/define_derivation_matrices.f90:28-100); weights products wgllwgll_*."""
    N = NGLL - 1
    hp = np.zeros((NGLL, NGLL))
    for i1 in range(NGLL):
        for i2 in range(NGLL):
            if i1 == i2:
                hp[i2, i1] = -N * (N + 1) / 4.0 if i1 == 0 else (N * (N + 1) / 4.0 if i1 == N else 0.0)
            else:
                hp[i2, i1] = _legendre(XIGLL[i2], N) / (_legendre(XIGLL[i1], N) * (XIGLL[i2] - XIGLL[i1]))
    hpw = hp * WGLL[:, None]
    ww = np.outer(WGLL, WGLL)
    col = lambda a: np.asarray(a, np.float32).reshape(-1, order="F")  # noqa: E731
    return dict(hprime_xx=col(hp), hprimewgll_xx=col(hpw), wgllwgll_xy=col(ww), wgllwgll_xz=col(ww),
                wgllwgll_yz=col(ww), hprime_d=hp)


def lagrange(xi: float):
    """Lagrange interpolants and derivatives at xi (shared/lagrange_poly.f90:30-199)."""
    h = np.ones(NGLL)
    hp = np.zeros(NGLL)
    for d in range(NGLL):
        others = [XIGLL[i] for i in range(NGLL) if i != d]
        den = np.prod([XIGLL[d] - o for o in others])
        h[d] = np.prod([xi - o for o in others]) / den
        s = 0.0
        for i, o in enumerate(others):
            s += np.prod([xi - q for jj, q in enumerate(others) if jj != i])
        hp[d] = s / den
    return h, hp


# ----------------------------------------------------------------------------
# the block
# ----------------------------------------------------------------------------

class Block:
    """Structured block geometry: node levels along each axis."""

    def __init__(self, cfg: dict):
        self.nx, self.ny = int(cfg["nx"]), int(cfg["ny"])
        self.xl = np.array([cfg["x0"] + (cfg["x1"] - cfg["x0"]) * e / self.nx for e in range(self.nx + 1)])
        self.yl = np.array([cfg["y0"] + (cfg["y1"] - cfg["y0"]) * e / self.ny for e in range(self.ny + 1)])
        self.zl = np.asarray(cfg["zlev"], np.float64)
        self.nz = len(self.zl) - 1
        self.nspec = self.nx * self.ny * self.nz
        self.NX, self.NY, self.NZ = 4 * self.nx + 1, 4 * self.ny + 1, 4 * self.nz + 1
        self.nglob = self.NX * self.NY * self.NZ
        # GLL coordinates along each axis per element: (n_elem_axis, 5)
        self.xg = self.xl[:-1, None] + (self.xl[1:] - self.xl[:-1])[:, None] * (1 + XIGLL[None, :]) / 2
        self.yg = self.yl[:-1, None] + (self.yl[1:] - self.yl[:-1])[:, None] * (1 + XIGLL[None, :]) / 2
        self.zg = self.zl[:-1, None] + (self.zl[1:] - self.zl[:-1])[:, None] * (1 + XIGLL[None, :]) / 2

    def elem_xyz(self, e):
        e = np.asarray(e)
        return e % self.nx, (e // self.nx) % self.ny, e // (self.nx * self.ny)

    def gll_coords(self, e):
        """(len(e), 125) x, y, z of the GLL points of elements e (i fastest)."""
        ex, ey, ez = self.elem_xyz(e)
        x = np.broadcast_to(self.xg[ex][:, None, None, :], (len(ex), 5, 5, 5)).reshape(len(ex), NGLL3)
        y = np.broadcast_to(self.yg[ey][:, None, :, None], (len(ex), 5, 5, 5)).reshape(len(ex), NGLL3)
        z = np.broadcast_to(self.zg[ez][:, :, None, None], (len(ex), 5, 5, 5)).reshape(len(ex), NGLL3)
        return x, y, z


def element_coordinates(cfg: dict) -> np.ndarray:
    """(nspec, 125, 3) coordinates of every element's GLL points of a block configuration."""
    B = Block(cfg)
    x, y, z = B.gll_coords(np.arange(B.nspec))
    return np.stack([x, y, z], axis=-1)


def _ibool_block(B: Block) -> np.ndarray:
    """First-appearance global numbering of the block's GLL points (1-based).

    A grid point (gx,gy,gz) = (4ex+i, 4ey+j, 4ez+k) first appears in the element
    with the smallest (ez, ey, ex), i.e. owner index o = max(0, ceil(g/4)-1) per
    axis, at local index g - 4o.  Elements own the sub-box of their points not
    shared with a lower-index neighbour ([0..4] on the low side of the block,
    [1..4] elsewhere), and points are numbered by owner element then local
    index i + 5j + 25k, as get_global_indirect_addressing does."""
    nx, ny, nz = B.nx, B.ny, B.nz
    e = np.arange(B.nspec, dtype=np.int64)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    cnt = (np.where(ex == 0, 5, 4) * np.where(ey == 0, 5, 4) * np.where(ez == 0, 5, 4)).astype(np.int64)
    offset = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    ibool = np.empty((B.nspec, NGLL3), np.int32)
    loc = np.arange(NGLL3)
    li, lj, lk = loc % 5, (loc // 5) % 5, loc // 25
    chunk = max(1, (1 << 22) // NGLL3)
    for s in range(0, B.nspec, chunk):
        sl = slice(s, min(B.nspec, s + chunk))
        gx = 4 * ex[sl, None] + li[None, :]
        gy = 4 * ey[sl, None] + lj[None, :]
        gz = 4 * ez[sl, None] + lk[None, :]
        ox = np.maximum(0, (gx + 3) // 4 - 1)
        oy = np.maximum(0, (gy + 3) // 4 - 1)
        oz = np.maximum(0, (gz + 3) // 4 - 1)
        ix, iy, iz = gx - 4 * ox, gy - 4 * oy, gz - 4 * oz
        i0 = np.where(ox == 0, 0, 1)
        j0 = np.where(oy == 0, 0, 1)
        k0 = np.where(oz == 0, 0, 1)
        ni = 5 - i0
        nj = 5 - j0
        own = ox + nx * (oy + ny * oz)
        rank = (ix - i0) + ni * ((iy - j0) + nj * (iz - k0))
        ibool[sl] = (offset[own] + rank + 1).astype(np.int32)
    return ibool.reshape(-1)


def _regularity(B: Block):
    """check_element_regularity (generate_databases/calc_jacobian.f90:184-360) for
    axis-aligned boxes: a cube of the first cube's size whose single-precision
    corner Jacobian has xix == etay == gammaz exactly."""
    ex, ey, ez = B.elem_xyz(np.arange(B.nspec))
    xa = B.xl[ex].astype(np.float32); xb = B.xl[ex + 1].astype(np.float32)
    ya = B.yl[ey].astype(np.float32); yb = B.yl[ey + 1].astype(np.float32)
    za = B.zl[ez].astype(np.float32); zb = B.zl[ez + 1].astype(np.float32)
    d1 = ((xb - xa).astype(np.float64)) ** 2   # edge 1-2 (x)
    d2 = ((zb - za).astype(np.float64)) ** 2   # edge 1-5 (z)
    d3 = ((yb - ya).astype(np.float64)) ** 2   # edge 1-4 (y)
    shape_ok = (np.abs(d2 - d1) < 1e-5 * d1) & (np.abs(d3 - d1) < 1e-5 * d1)
    xxi = 0.5 * (xb.astype(np.float64) - xa.astype(np.float64))
    yeta = 0.5 * (yb.astype(np.float64) - ya.astype(np.float64))
    zga = 0.5 * (zb.astype(np.float64) - za.astype(np.float64))
    jac = xxi * (yeta * zga)
    xix = (yeta * zga / jac).astype(np.float32)
    etay = (xxi * zga / jac).astype(np.float32)
    gaz = (xxi * yeta / jac).astype(np.float32)
    cand = shape_ok & (xix == etay) & (xix == gaz)
    regular = np.zeros(B.nspec, bool)
    idx = np.nonzero(cand)[0]
    xr = jr = 0.0
    if len(idx):
        first = idx[0]
        cube = d1[first]
        regular = cand & (np.abs(d1 - cube) <= 1e-5 * cube)
        regular[:first] = False
        # the regular constants come from the double-precision corner coordinates
        fx, fy, fz = (int(v) for v in B.elem_xyz(first))
        a = 0.5 * (B.xl[fx + 1] - B.xl[fx])
        b = 0.5 * (B.yl[fy + 1] - B.yl[fy])
        c = 0.5 * (B.zl[fz + 1] - B.zl[fz])
        jd = a * (b * c)
        xd, yd, zd = b * c / jd, a * c / jd, a * b / jd
        xr = float(np.float32(xd))
        jr = float(np.float32(1.0 / (xd * (yd * zd - 0.0 * 0.0) - 0.0 * (0.0 * zd - 0.0 * 0.0) + 0.0 * (0.0 * 0.0 - yd * 0.0))))
    irr = np.where(regular, 0, np.cumsum(~regular)).astype(np.int32)
    return irr, xr, jr


def build_database(cfg: dict, material=None, dtype=np.float32) -> dict:
    """All solver arrays of the block (reference layouts, 1-based indices)."""
    B = Block(cfg)
    nspec = B.nspec
    db = dict(nspec=nspec, nglob=B.nglob)
    db["ibool"] = _ibool_block(B)
    irr, xr, jr = _regularity(B)
    nirr = int(irr.max()) if irr.size else 0
    db.update(irregular_element_number=irr, nspec_irregular=nirr, xix_regular=xr, jacobian_regular=jr)
    # metric of irregular elements: constant per axis-aligned box
    elist = np.nonzero(irr)[0]
    ex, ey, ez = B.elem_xyz(elist)
    dx = B.xl[ex + 1] - B.xl[ex]
    dy = B.yl[ey + 1] - B.yl[ey]
    dz = B.zl[ez + 1] - B.zl[ez]
    ne = max(nirr, 1)
    zero = np.zeros(ne * NGLL3, dtype)

    def per_elem(v):
        out = np.zeros((ne, NGLL3), dtype)
        if nirr:
            out[:] = np.asarray(v, dtype)[:, None]
        return out.reshape(-1)

    db["xix"] = per_elem(2.0 / dx)
    db["etay"] = per_elem(2.0 / dy)
    db["gammaz"] = per_elem(2.0 / dz)
    for n in ["xiy", "xiz", "etax", "etaz", "gammax", "gammay"]:
        db[n] = zero.copy()
    db["jacobian"] = per_elem(dx * dy * dz / 8.0)
    # materials
    if material is None and cfg.get("perturbation"):
        from . import models
        material = models.perturbed_material(cfg, **cfg["perturbation"])
    if material is None:
        lay = np.asarray(cfg["elem_layer"], np.int64)
        L = cfg["layers"]
        rho = np.repeat(np.asarray([m["rho"] for m in L], np.float32)[lay], NGLL3)
        vp = np.repeat(np.asarray([m["vp"] for m in L], np.float32)[lay], NGLL3)
        vs = np.repeat(np.asarray([m["vs"] for m in L], np.float32)[lay], NGLL3)
    else:
        # the database's precision (an FP64 database keeps FP64 material values)
        rho, vp, vs = (np.asarray(a, dtype) for a in material)
    r, p, s = rho.astype(dtype), vp.astype(dtype), vs.astype(dtype)
    # fluid elements: zero shear velocity (generate_databases/get_model.F90 sets
    # ispec_is_acoustic for vs == 0)
    db["ispec_is_acoustic"] = (np.asarray(vs, np.float32).reshape(nspec, NGLL3) == 0).all(axis=1).astype(np.int32)
    db["rhostore"] = r
    db["kappastore"] = r * (p * p - dtype(4.0 / 3.0) * s * s)
    db["mustore"] = r * s * s
    db["rho_vp"] = r * p
    db["rho_vs"] = r * s
    # absorbing faces, fluid-solid coupling faces, free surface
    _absorbing(cfg, B, db, dtype)
    _coupling_and_free_surface(cfg, B, db, dtype)
    # mass matrices
    _mass(cfg, B, db, dtype)
    db.update(derivation_matrices())
    # sources / receivers / stf
    _sources_receivers(cfg, B, db, dtype)
    db["attenuation"] = int(bool(cfg.get("attenuation", False)))
    if db["attenuation"]:
        from . import attenuation
        db.update(attenuation.setup(cfg, db))
    return db


def _absorbing(cfg, B, db, dtype):
    want = cfg.get("absorbing", ["xmin", "xmax", "ymin", "ymax", "bottom"]) if cfg.get("stacey", True) else []
    e = np.arange(B.nspec)
    ex, ey, ez = B.elem_xyz(e)
    conds = {"xmin": (1, ex == 0), "xmax": (2, ex == B.nx - 1), "ymin": (3, ey == 0), "ymax": (4, ey == B.ny - 1),
             "bottom": (5, ez == 0), "top": (6, ez == B.nz - 1)}
    a = np.arange(5)
    A, Bb = np.meshgrid(a, a, indexing="xy")   # A fastest within face: g = a + 5 b
    A, Bb = A.reshape(-1), Bb.reshape(-1)
    ispecs, ijks, jws, normals = [], [], [], []
    for name in ["xmin", "xmax", "ymin", "ymax", "bottom", "top"]:
        if name not in want:
            continue
        iface, sel = conds[name]
        el = np.nonzero(sel)[0]
        if not len(el):
            continue
        fx, fy, fz = B.elem_xyz(el)
        dx = (B.xl[fx + 1] - B.xl[fx])[:, None]
        dy = (B.yl[fy + 1] - B.yl[fy])[:, None]
        dz = (B.zl[fz + 1] - B.zl[fz])[:, None]
        one = np.ones((len(el), 25), np.int32)
        if iface in (1, 2):
            i = one * (1 if iface == 1 else 5); j = one * (A + 1); k = one * (Bb + 1)
            jac2 = dy * dz / 4.0
            n = np.array([-1.0 if iface == 1 else 1.0, 0.0, 0.0])
        elif iface in (3, 4):
            i = one * (A + 1); j = one * (1 if iface == 3 else 5); k = one * (Bb + 1)
            jac2 = dx * dz / 4.0
            n = np.array([0.0, -1.0 if iface == 3 else 1.0, 0.0])
        else:
            i = one * (A + 1); j = one * (Bb + 1); k = one * (1 if iface == 5 else 5)
            jac2 = dx * dy / 4.0
            n = np.array([0.0, 0.0, -1.0 if iface == 5 else 1.0])
        w = (WGLL[A] * WGLL[Bb])[None, :]
        ispecs.append(el + 1)
        ijks.append(np.stack([i, j, k], axis=-1).reshape(len(el), 25, 3))
        jws.append((jac2 * w).astype(dtype))
        normals.append(np.broadcast_to(n.astype(dtype), (len(el), 25, 3)))
    if ispecs:
        db["abs_boundary_ispec"] = np.concatenate(ispecs).astype(np.int32)
        db["abs_boundary_ijk"] = np.concatenate(ijks).astype(np.int32).reshape(-1)
        db["abs_boundary_jacobian2Dw"] = np.concatenate(jws).reshape(-1)
        db["abs_boundary_normal"] = np.ascontiguousarray(np.concatenate(normals)).reshape(-1)
    else:
        db["abs_boundary_ispec"] = np.zeros(0, np.int32)
        db["abs_boundary_ijk"] = np.zeros(0, np.int32)
        db["abs_boundary_jacobian2Dw"] = np.zeros(0, dtype)
        db["abs_boundary_normal"] = np.zeros(0, dtype)
    db["num_abs_boundary_faces"] = len(db["abs_boundary_ispec"])
    db["stacey"] = int(db["num_abs_boundary_faces"] > 0)


def _face_pts(iface):
    """Element-local point indices of face iface (1..6) in face GLL order
    (get_element_face_gll_indices, shared/get_element_face.f90:169-279)."""
    a = np.arange(5)
    A, Bb = np.meshgrid(a, a, indexing="xy")
    A, Bb = A.reshape(-1), Bb.reshape(-1)
    if iface in (1, 2):
        i, j, k = np.full(25, 0 if iface == 1 else 4), A, Bb
    elif iface in (3, 4):
        i, j, k = A, np.full(25, 0 if iface == 3 else 4), Bb
    else:
        i, j, k = A, Bb, np.full(25, 0 if iface == 5 else 4)
    return np.stack([i, j, k], axis=-1)


def _coupling_and_free_surface(cfg, B, db, dtype):
    """Fluid-solid coupling faces seen from the fluid element, normal pointing out
    of the fluid, in element then face order (generate_databases/get_coupling_surfaces.f90:270-380);
    free-surface faces = top faces of the block (face 6)."""
    isac = db["ispec_is_acoustic"].astype(bool)
    nspec = B.nspec
    e = np.arange(nspec)
    ex, ey, ez = B.elem_xyz(e)
    ispecs, ijks, jws, normals = [], [], [], []
    if isac.any() and (~isac).any():
        nb = {1: (ex > 0, e - 1), 2: (ex < B.nx - 1, e + 1), 3: (ey > 0, e - B.nx), 4: (ey < B.ny - 1, e + B.nx),
              5: (ez > 0, e - B.nx * B.ny), 6: (ez < B.nz - 1, e + B.nx * B.ny)}
        flag = np.zeros((nspec, 7), bool)
        for f in range(1, 7):
            has, other = nb[f]
            flag[:, f] = isac & has & ~isac[np.where(has, other, 0)]
        for el in np.nonzero(flag.any(axis=1))[0]:
            fx, fy, fz = (int(v) for v in B.elem_xyz(el))
            dx = B.xl[fx + 1] - B.xl[fx]; dy = B.yl[fy + 1] - B.yl[fy]; dz = B.zl[fz + 1] - B.zl[fz]
            for f in range(1, 7):
                if not flag[el, f]:
                    continue
                pts = _face_pts(f)
                a = np.arange(5)
                A, Bb = np.meshgrid(a, a, indexing="xy")
                w = (WGLL[A.reshape(-1)] * WGLL[Bb.reshape(-1)])
                jac2 = {1: dy * dz, 2: dy * dz, 3: dx * dz, 4: dx * dz, 5: dx * dy, 6: dx * dy}[f] / 4.0
                n = np.zeros(3)
                n[(f - 1) // 2] = -1.0 if f % 2 == 1 else 1.0
                ispecs.append(el + 1)
                ijks.append(pts + 1)
                jws.append(jac2 * w)
                normals.append(np.broadcast_to(n, (25, 3)))
    nc = len(ispecs)
    db["num_coupling_ac_el_faces"] = nc
    db["coupling_ac_el_ispec"] = np.asarray(ispecs, np.int32)
    db["coupling_ac_el_ijk"] = (np.asarray(ijks, np.int32).reshape(-1) if nc else np.zeros(0, np.int32))
    db["coupling_ac_el_jacobian2Dw"] = (np.asarray(jws, dtype).reshape(-1) if nc else np.zeros(0, dtype))
    db["coupling_ac_el_normal"] = (np.asarray(normals, dtype).reshape(-1) if nc else np.zeros(0, dtype))
    top = np.nonzero(ez == B.nz - 1)[0]
    db["num_free_surface_faces"] = len(top)
    db["free_surface_ispec"] = (top + 1).astype(np.int32)
    db["free_surface_ijk"] = np.tile((_face_pts(6) + 1).reshape(-1), len(top)).astype(np.int32)


def _mass(cfg, B, db, dtype):
    """Mass matrices of any hexahedral mesh: per-point Jacobian of irregular
    elements, the regular Jacobian elsewhere."""
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    irr = db["irregular_element_number"]
    w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1)  # i fastest
    jel = np.empty((nspec, NGLL3), np.float64)
    reg = irr == 0
    jel[reg] = np.float32(db["jacobian_regular"])
    if (~reg).any():
        jel[~reg] = db["jacobian"].reshape(-1, NGLL3)[irr[~reg] - 1]
    rho = db["rhostore"].reshape(nspec, NGLL3).astype(np.float64)
    isac = db["ispec_is_acoustic"].astype(bool)
    ib = db["ibool"].reshape(nspec, NGLL3).astype(np.int64) - 1
    terms = (jel * w3[None, :] * rho).astype(dtype).astype(np.float64)
    terms[isac] = 0.0
    rmass = np.bincount(ib.reshape(-1), weights=terms.reshape(-1), minlength=nglob)
    rmass = rmass.astype(dtype)
    if isac.any():
        # rmass_acoustic = 1 / (sum J w / kappa + Stacey term) (define_mass_matrices.f90:120-160, :488-520)
        kap = db["kappastore"].reshape(nspec, NGLL3).astype(np.float64)
        ta = np.zeros_like(terms)
        ta[isac] = (jel[isac] * w3[None, :] / kap[isac]).astype(dtype)
        rma = np.bincount(ib.reshape(-1), weights=ta.reshape(-1), minlength=nglob).astype(dtype)
        db["rmass_acoustic_volume"] = rma.copy()          # the database's rmass_acoustic
        if db["stacey"]:
            nf = db["num_abs_boundary_faces"]
            isp = db["abs_boundary_ispec"] - 1
            ijk = db["abs_boundary_ijk"].reshape(nf, 25, 3) - 1
            pt = ijk[..., 0] + 5 * ijk[..., 1] + 25 * ijk[..., 2]
            q = isp[:, None] * NGLL3 + pt
            sel = isac[isp]
            sn = dtype(0.5 * float(cfg["dt"])) / db["rho_vp"][q[sel]]
            add = db["abs_boundary_jacobian2Dw"].reshape(nf, 25)[sel] * sn
            st = np.bincount(db["ibool"][q[sel]].reshape(-1).astype(np.int64) - 1,
                             weights=add.astype(np.float64).reshape(-1), minlength=nglob).astype(dtype)
            db["rmassz_acoustic"] = st                          # the database's Stacey term
            rma = rma + st
        rma[rma <= 0] = 1
        db["rmass_acoustic"] = (dtype(1) / rma).astype(dtype)
    mx = rmass.copy(); my = rmass.copy(); mz = rmass.copy()
    if db["stacey"]:
        dt2 = dtype(0.5 * float(cfg["dt"]))
        nf = db["num_abs_boundary_faces"]
        isp = db["abs_boundary_ispec"] - 1
        ijk = db["abs_boundary_ijk"].reshape(nf, 25, 3) - 1
        p = ijk[..., 0] + 5 * ijk[..., 1] + 25 * ijk[..., 2]
        q = isp[:, None] * NGLL3 + p
        n = db["abs_boundary_normal"].reshape(nf, 25, 3)
        rvp = db["rho_vp"][q]; rvs = db["rho_vs"][q]
        vn = dt2 * (n[..., 0] + n[..., 1] + n[..., 2])
        jw = db["abs_boundary_jacobian2Dw"].reshape(nf, 25)
        g = db["ibool"][q].astype(np.int64) - 1
        el = ~isac[isp]
        for c, m in enumerate((mx, my, mz)):
            t = rvp * vn * n[..., c] + rvs * (dt2 - vn * n[..., c])
            add = np.bincount(g[el].reshape(-1), weights=(t * jw)[el].astype(np.float64).reshape(-1), minlength=nglob)
            # the database keeps the Stacey terms apart (rmassx/y/z of
            # save_arrays_solver.F90:228-231); the solver adds rmass before inverting
            db["rmass" + "xyz"[c] + "_stacey"] = add.astype(dtype)
            m += add.astype(dtype)
    for m in (mx, my, mz):
        m[m <= 0] = 1
    db["rmass"] = rmass
    db["rmassx"] = (dtype(1) / mx).astype(dtype)
    db["rmassy"] = (dtype(1) / my).astype(dtype)
    db["rmassz"] = (dtype(1) / mz).astype(dtype)


def locate(B: Block, xt: float, yt: float, zt: float, octant=None):
    """Closest GLL point (single-precision coordinates, first strictly-closer wins
    in element order), then local coordinates in that element; a target outside
    that element moves to the first element containing it
    (specfem3D/locate_point.f90:160-300, :422-624).  Returns (ispec 1-based, xi, eta, gamma).

    ``octant`` (3 signs) places a target that lies on element boundaries in the
    element on that side of it along each axis, the element a run partitioned
    differently may have chosen."""
    if octant is not None:
        idx = []
        for v, lv, n, sgn in ((xt, B.xl, B.nx, octant[0]), (yt, B.yl, B.ny, octant[1]), (zt, B.zl, B.nz, octant[2])):
            i = np.searchsorted(lv, v, side="left" if sgn < 0 else "right") - 1
            idx.append(int(np.clip(i, 0, n - 1)))
        ex, ey, ez = idx
        e = ex + B.nx * (ey + B.ny * ez)
        return (e + 1, (2 * xt - B.xl[ex] - B.xl[ex + 1]) / (B.xl[ex + 1] - B.xl[ex]),
                (2 * yt - B.yl[ey] - B.yl[ey + 1]) / (B.yl[ey + 1] - B.yl[ey]),
                (2 * zt - B.zl[ez] - B.zl[ez + 1]) / (B.zl[ez + 1] - B.zl[ez]))
    ex0 = np.searchsorted(B.xl, xt) - 1
    ey0 = np.searchsorted(B.yl, yt) - 1
    ez0 = np.searchsorted(B.zl, zt) - 1
    cx = np.arange(max(0, ex0 - 1), min(B.nx, ex0 + 3))
    cy = np.arange(max(0, ey0 - 1), min(B.ny, ey0 + 3))
    cz = np.arange(max(0, ez0 - 1), min(B.nz, ez0 + 3))
    E = (cx[None, None, :] + B.nx * (cy[None, :, None] + B.ny * cz[:, None, None])).reshape(-1)
    E = np.sort(E)
    x, y, z = B.gll_coords(E)
    d = ((xt - x.astype(np.float32).astype(np.float64)) ** 2 + (yt - y.astype(np.float32).astype(np.float64)) ** 2
         + (zt - z.astype(np.float32).astype(np.float64)) ** 2)
    flat = int(np.argmin(d.reshape(-1)))  # first minimum in (element, k, j, i) order
    e = int(E[flat // NGLL3])

    def local(e):
        ex, ey, ez = (int(v) for v in B.elem_xyz(e))
        xi = (2 * xt - B.xl[ex] - B.xl[ex + 1]) / (B.xl[ex + 1] - B.xl[ex])
        eta = (2 * yt - B.yl[ey] - B.yl[ey + 1]) / (B.yl[ey + 1] - B.yl[ey])
        ga = (2 * zt - B.zl[ez] - B.zl[ez + 1]) / (B.zl[ez + 1] - B.zl[ez])
        return xi, eta, ga

    xi, eta, ga = local(e)
    if max(abs(xi), abs(eta), abs(ga)) > 1 + 1e-9:
        ex = int(np.clip(np.searchsorted(B.xl, xt, side="left") - 1, 0, B.nx - 1))
        ey = int(np.clip(np.searchsorted(B.yl, yt, side="left") - 1, 0, B.ny - 1))
        ez = int(np.clip(np.searchsorted(B.zl, zt, side="left") - 1, 0, B.nz - 1))
        e = ex + B.nx * (ey + B.ny * ez)
        xi, eta, ga = local(e)
    return e + 1, xi, eta, ga


def _sources_receivers(cfg, B, db, dtype, locator=None):
    """Source arrays, receiver interpolants and stf tables; ``locator(x, y, z)`` returns
    (ispec 1-based, xi, eta, gamma) and defaults to the block locator."""
    if locator is None:
        def locator(x, y, z, octant=None):
            return locate(B, x, y, z, octant)
    srcs = cfg.get("sources", [])
    ns = len(srcs)
    sa = np.zeros((ns, 3, NGLL3))
    isel = np.zeros(ns, np.int32)
    loc = np.zeros((ns, 3))
    src_fluid = np.zeros(ns, bool)
    irr = db["irregular_element_number"]
    for i, s in enumerate(srcs):
        e1, xi, eta, ga = locator(float(s["x"]), float(s["y"]), float(s["z"]), s.get("octant"))
        isel[i] = e1
        loc[i] = (xi, eta, ga)
        hx, hpx = lagrange(xi)
        he, hpe = lagrange(eta)
        hg, hpg = lagrange(ga)
        hl = (hg[:, None, None] * he[None, :, None] * hx[None, None, :]).reshape(-1)
        in_fluid = bool(np.asarray(db.get("ispec_is_acoustic", np.zeros(e1, np.int32)))[e1 - 1])
        src_fluid[i] = in_fluid
        if s.get("type", "cmt") == "cmt" and in_fluid:
            # moment tensor in a fluid element: an explosion-equivalent pressure
            # source of the scalar moment (setup_sources_receivers.f90:1187-1212):
            # factor = sqrt(2/3) M0, M0 = sqrt(M:M / 2), interpolated on the element
            Mxx, Myy, Mzz, Mxy, Mxz, Myz = (float(v) for v in s["M"])
            m0 = math.sqrt(Mxx ** 2 + Myy ** 2 + Mzz ** 2 + 2.0 * (Myz ** 2 + Mxz ** 2 + Mxy ** 2)) / math.sqrt(2.0)
            fac = m0 * math.sqrt(2.0) / math.sqrt(3.0)
            for c in range(3):
                sa[i, c] = fac * hl
        elif s.get("type", "cmt") == "cmt":
            ir = irr[e1 - 1]
            if ir:
                m = [db[n].reshape(-1, NGLL3)[ir - 1].astype(np.float64) for n in
                     ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz")]
                dd = [float(np.sum(hl * mm)) for mm in m]
            else:
                xr = float(np.float32(db["xix_regular"]))
                sh = float(np.sum(hl))
                dd = [xr * sh, 0.0, 0.0, 0.0, xr * sh, 0.0, 0.0, 0.0, xr * sh]
            dxis_dx, dxis_dy, dxis_dz, detas_dx, detas_dy, detas_dz, dg_dx, dg_dy, dg_dz = dd
            hxi = (hg[:, None, None] * he[None, :, None] * hpx[None, None, :]).reshape(-1)
            heta = (hg[:, None, None] * hpe[None, :, None] * hx[None, None, :]).reshape(-1)
            hga = (hpg[:, None, None] * he[None, :, None] * hx[None, None, :]).reshape(-1)
            dsx = hxi * dxis_dx + heta * detas_dx + hga * dg_dx
            dsy = hxi * dxis_dy + heta * detas_dy + hga * dg_dy
            dsz = hxi * dxis_dz + heta * detas_dz + hga * dg_dz
            Mxx, Myy, Mzz, Mxy, Mxz, Myz = (float(v) for v in s["M"])
            sa[i, 0] = Mxx * dsx + Mxy * dsy + Mxz * dsz
            sa[i, 1] = Mxy * dsx + Myy * dsy + Myz * dsz
            sa[i, 2] = Mxz * dsx + Myz * dsy + Mzz * dsz
        else:
            f = [float(v) for v in s["F"]]
            for c in range(3):
                sa[i, c] = f[c] * hl
    # Fortran sourcearrays(NSOURCES,NDIM,NGLLX,NGLLY,NGLLZ): source index fastest
    db["sourcearrays"] = np.ascontiguousarray(sa.astype(dtype).transpose(2, 1, 0)).reshape(-1)
    db["ispec_selected_source"] = isel
    db["source_xi_eta_gamma"] = loc
    db["nsources"] = ns
    recs = cfg.get("receivers", [])
    nr = len(recs)
    irec = np.zeros(nr, np.int32)
    hx, he, hg = np.zeros((nr, NGLL)), np.zeros((nr, NGLL)), np.zeros((nr, NGLL))
    rloc = np.zeros((nr, 3))
    for r, (x, y, z) in enumerate(recs):
        e1, xi, eta, ga = locator(float(x), float(y), float(z))
        irec[r] = e1
        rloc[r] = (xi, eta, ga)
        hx[r], _ = lagrange(xi)
        he[r], _ = lagrange(eta)
        hg[r], _ = lagrange(ga)
    db.update(ispec_selected_rec=irec, hxir=hx.reshape(-1), hetar=he.reshape(-1), hgammar=hg.reshape(-1),
              receiver_xi_eta_gamma=rloc, nrec=nr)
    stf, t0 = stf_table(cfg, src_fluid)
    db["stf"] = stf
    db["t0"] = t0


def stf_value(kind: str, t, p):
    """Source time functions (specfem3D/comp_source_time_function.f90): Heaviside
    via the error function with hdur_Gaussian = hdur/1.628 (setup_sources_receivers.f90:439),
    Ricker of dominant frequency f0, Gaussian."""
    t = np.asarray(t, np.float64)
    if kind == "heaviside":
        return 0.5 * (1.0 + erf(t / (p / 1.628)))
    if kind == "ricker":
        a = math.pi ** 2 * p * p
        return (1.0 - 2.0 * a * t * t) * np.exp(-a * t * t)
    hd = p / 1.628
    return np.exp(-t * t / (hd * hd)) / (math.sqrt(math.pi) * hd)


def stf_table(cfg: dict, in_fluid=None):
    """(NSOURCES, NSTEP) FP64 stf at t = (it-1) dt - t0 - tshift
    (compute_add_sources_viscoelastic.F90:80-100), t0 per setup_sources_receivers.f90:482-491.
    Moment-tensor sources in fluid elements (in_fluid) use a Gaussian instead of
    the Heaviside (get_stf_acoustic, compute_add_sources_acoustic.f90:693-821)
    and move t0 to at least 3 (hdur - tshift) (setup_sources_receivers.f90:495-514)."""
    srcs = cfg.get("sources", [])
    dt, nstep = float(cfg["dt"]), int(cfg["nstep"])
    if not srcs:
        return np.zeros((0, nstep)), 0.0
    fluid = [bool(in_fluid[i]) if in_fluid is not None else False for i in range(len(srcs))]
    kinds = [s.get("stf", "ricker") for s in srcs]
    kinds = ["gaussian" if f and k == "heaviside" and s.get("type", "cmt") == "cmt" else k
             for s, k, f in zip(srcs, kinds, fluid)]
    params = [float(s["f0"]) if k == "ricker" else float(s["hdur"]) for s, k in zip(srcs, kinds)]
    tsh = np.array([float(s.get("tshift", 0.0)) for s in srcs])
    tsh = tsh - tsh.min() if len(srcs) > 1 else np.zeros(1)
    if all(k == "ricker" for k in kinds):
        t0 = -1.2 * min(ts - 1.0 / p for ts, p in zip(tsh, params))
    else:
        t0 = -2.0 * min(ts - p for ts, p in zip(tsh, params))
    for f, k, ts, p in zip(fluid, kinds, tsh, params):
        if f and k == "gaussian":
            t0 = max(t0, -3.0 * (ts - p))
    if "t0" in cfg:
        t0 = float(cfg["t0"])
    t = (np.arange(nstep) * dt) - t0
    return np.stack([stf_value(k, t - ts, p) for k, p, ts in zip(kinds, params, tsh)]), t0


def block_colors(cfg: dict) -> np.ndarray:
    """Colour of every element of a block mesh such that no two elements of a colour
    share a GLL point: the parity of the element indices along x, y, z (8 colours).
    Plays the part of get_perm_color (generate_databases) for structured blocks."""
    B = Block(cfg)
    e = np.arange(B.nspec)
    ex, ey, ez = B.elem_xyz(e)
    return ((ex % 2) + 2 * (ey % 2) + 4 * (ez % 2)).astype(np.int32)


def greedy_colors(ibool: np.ndarray, nspec: int, nglob: int) -> np.ndarray:
    """First-fit colouring of elements through shared points (any mesh): element e
    takes the lowest colour not used by an element sharing one of its points."""
    ib = np.asarray(ibool).reshape(nspec, -1) - 1
    used = np.zeros(nglob, np.uint64)          # bit c set: colour c already touches the point
    col = np.zeros(nspec, np.int32)
    for e in range(nspec):
        m = np.bitwise_or.reduce(used[ib[e]])
        c = 0
        while (int(m) >> c) & 1:
            c += 1
        col[e] = c
        used[ib[e]] |= np.uint64(1 << c)
    return col
