"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this module; it is test infrastructure, never the product.  It builds
``liboracle_f32.so`` / ``liboracle_f64.so`` from ``sem_oracle.c`` and restates
the reference's database generation for a regular layered block:

* mesher geometry + GLL coordinates   (generate_databases/calc_jacobian.f90:148-178)
* global numbering                    (shared/get_global.f90:28-141)
* Jacobian, regular/irregular split   (generate_databases/calc_jacobian.f90:28-360)
* materials                           (generate_databases/get_model.F90:289-301)
* mass matrices incl. Stacey term     (shared/define_mass_matrices.f90:28-442,
                                       specfem3D/prepare_timerun.F90:246-388)
* absorbing faces                     (generate_databases/get_absorbing_boundary.F90)
* source/receiver location + arrays   (specfem3D/locate_point.f90,
                                       specfem3D/compute_arrays_source.f90:29-149)
* source time function table          (specfem3D/comp_source_time_function.f90,
                                       specfem3D/setup_sources_receivers.f90:482-491)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SRC = os.path.join(_HERE, "sem_oracle.c")
_LOCK = threading.Lock()
_LIBS: dict = {}

NGLL = 5
NGLL3 = 125
N_SLS = 3


def build(force: bool = False) -> None:
    """Compile both precisions of the oracle with gcc (OpenMP)."""
    os.makedirs(_BUILD, exist_ok=True)
    for tag, extra in (("f32", []), ("f64", ["-DORACLE_DOUBLE"])):
        out = os.path.join(_BUILD, f"liboracle_{tag}.so")
        if (not force and os.path.exists(out)
                and os.path.getmtime(out) >= max(os.path.getmtime(_SRC),
                                                 os.path.getmtime(os.path.join(_HERE, "sem_oracle.h")))):
            continue
        cmd = ["gcc", "-O2", "-fPIC", "-fopenmp", "-shared", *extra, "-o", out, _SRC, "-lm"]
        subprocess.run(cmd, check=True)


def lib(precision: str = "f32") -> ctypes.CDLL:
    with _LOCK:
        if precision not in _LIBS:
            build()
            L = ctypes.CDLL(os.path.join(_BUILD, f"liboracle_{precision}.so"))
            vp = ctypes.c_void_p
            L.orc_sim_new.restype = vp
            L.orc_sim_free.argtypes = [vp]
            L.orc_set_ptr.argtypes = [vp, ctypes.c_char_p, vp]
            L.orc_set_int.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
            L.orc_get_int.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
            L.orc_set_real.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
            L.orc_step.argtypes = [vp]
            L.orc_run.argtypes = [vp, ctypes.c_int]
            L.orc_compute_forces_elastic.argtypes = [vp, ctypes.c_int]
            L.orc_stf.restype = ctypes.c_double
            L.orc_stf.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
            L.orc_get_global.restype = ctypes.c_int
            L.orc_get_global.argtypes = [ctypes.c_long, vp, vp, vp, vp, ctypes.c_double]
            L.orc_mesh_regular.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [vp] * 5
            L.orc_gll_coordinates.argtypes = [ctypes.c_int, vp, vp, vp, vp]
            L.orc_calc_jacobian_all.restype = ctypes.c_int
            L.orc_calc_jacobian_all.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp]
            L.orc_mass_stacey_elastic.argtypes = [ctypes.c_int, ctypes.c_double] + [vp] * 10
            L.orc_invert_mass.argtypes = [ctypes.c_int, vp, vp, vp, vp, ctypes.c_int]
            L.orc_face_geometry.argtypes = [vp, ctypes.c_int, vp, vp, vp]
            L.orc_locate_point.restype = ctypes.c_int
            L.orc_locate_point.argtypes = [ctypes.c_int] + [vp] * 8 + [ctypes.c_double] * 3 + [vp] * 3
            L.orc_lagrange_any.argtypes = [ctypes.c_double, vp, vp, vp]
            L.orc_gll.argtypes = [vp, vp]
            L.orc_derivation_matrices.argtypes = [vp] * 6
            L.orc_source_array_cmt.argtypes = ([ctypes.c_int, vp, vp, ctypes.c_float if precision == "f32" else ctypes.c_double]
                                               + [ctypes.c_double] * 9 + [vp])
            L.orc_source_array_force.argtypes = [ctypes.c_double] * 6 + [vp]
            L.orc_realw_size.restype = ctypes.c_int
            _LIBS[precision] = L
        return _LIBS[precision]


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def real_dtype(precision: str):
    return np.float32 if precision == "f32" else np.float64


class OracleSim:
    """One oracle simulation: numpy arrays handed to the C struct by name."""

    def __init__(self, precision: str = "f32"):
        self.precision = precision
        self.L = lib(precision)
        self.h = self.L.orc_sim_new()
        self._keep: dict = {}

    def __del__(self):
        try:
            self.L.orc_sim_free(self.h)
        except Exception:
            pass

    def set(self, name: str, arr: np.ndarray) -> np.ndarray:
        if not arr.flags.c_contiguous:
            arr = np.ascontiguousarray(arr)
        self._keep[name] = arr
        if self.L.orc_set_ptr(self.h, name.encode(), _p(arr)) != 0:
            raise KeyError(name)
        return arr

    def get(self, name: str) -> np.ndarray:
        return self._keep[name]

    def seti(self, name: str, v: int) -> None:
        if self.L.orc_set_int(self.h, name.encode(), int(v)) != 0:
            raise KeyError(name)

    def geti(self, name: str) -> int:
        v = ctypes.c_int(0)
        if self.L.orc_get_int(self.h, name.encode(), ctypes.byref(v)) != 0:
            raise KeyError(name)
        return v.value

    def setr(self, name: str, v: float) -> None:
        if self.L.orc_set_real(self.h, name.encode(), float(v)) != 0:
            raise KeyError(name)

    def step(self, n: int = 1) -> None:
        self.L.orc_run(self.h, int(n))

    def forces(self, backward: bool = False) -> None:
        self.L.orc_compute_forces_elastic(self.h, int(backward))


# ----------------------------------------------------------------------------
# database generation restated from the reference (regular layered block)
# ----------------------------------------------------------------------------

def gll():
    L = lib("f64")
    x = np.zeros(NGLL)
    w = np.zeros(NGLL)
    L.orc_gll(_p(x), _p(w))
    return x, w


def derivation_matrices(precision: str = "f32"):
    L = lib(precision)
    rd = real_dtype(precision)
    hp, hpw, wxy, wxz, wyz = (np.zeros(25, rd) for _ in range(5))
    hpd = np.zeros(25)
    L.orc_derivation_matrices(_p(hp), _p(hpw), _p(wxy), _p(wxz), _p(wyz), _p(hpd))
    return dict(hprime_xx=hp, hprimewgll_xx=hpw, wgllwgll_xy=wxy, wgllwgll_xz=wxz, wgllwgll_yz=wyz,
                hprime_d=hpd)


def lagrange_any(xi: float):
    L = lib("f64")
    x, _ = gll()
    h = np.zeros(NGLL)
    hp = np.zeros(NGLL)
    L.orc_lagrange_any(float(xi), _p(x), _p(h), _p(hp))
    return h, hp


def stf_table(kind: str, param: float, tshift: float, t0: float, dt: float, nstep: int) -> np.ndarray:
    """FP64 source time function at t = (it-1) dt - t0 - tshift
    (compute_add_sources_viscoelastic.F90:80-100)."""
    L = lib("f64")
    k = {"heaviside": 0, "ricker": 1, "gaussian": 2}[kind]
    return np.array([L.orc_stf(k, (it - 1) * dt - t0 - tshift, param) for it in range(1, nstep + 1)])


def build_database(cfg: dict, precision: str = "f32", material=None) -> dict:
    """Run the restated setup chain for a regular layered block.

    ``cfg`` uses the schema of :func:`specfem3d_gb300.meshgen.normalize_config`.
    ``material`` optionally gives (rho, vp, vs) per GLL point (125*nspec each,
    float32) for models that are not piecewise constant by layer.
    """
    L = lib(precision)
    nx, ny = int(cfg["nx"]), int(cfg["ny"])
    zlev = np.asarray(cfg["zlev"], dtype=np.float64)
    nz = len(zlev) - 1
    nspec = nx * ny * nz
    npt = NGLL3 * nspec
    anchors = np.zeros(24 * nspec)
    xs, ys, zs = np.zeros(npt), np.zeros(npt), np.zeros(npt)
    L.orc_mesh_regular(nx, ny, nz, float(cfg["x0"]), float(cfg["x1"]), float(cfg["y0"]), float(cfg["y1"]),
                       _p(zlev), _p(anchors), _p(xs), _p(ys), _p(zs))
    xtol = 1e-10 * abs(float(cfg["x1"]) - float(cfg["x0"]))
    # materials: per element layer, optionally per GLL point
    if material is None:
        lay = np.repeat(np.asarray(cfg["elem_layer"], np.int64), NGLL3)
        rho = np.asarray([m["rho"] for m in cfg["layers"]], np.float32)[lay]
        vp = np.asarray([m["vp"] for m in cfg["layers"]], np.float32)[lay]
        vs = np.asarray([m["vs"] for m in cfg["layers"]], np.float32)[lay]
    else:
        rho, vp, vs = (np.asarray(a, np.float32) for a in material)
    # absorbing faces: xmin, xmax, ymin, ymax, bottom (and top if requested)
    faces = []
    ex = np.arange(nspec) % nx
    ey = (np.arange(nspec) // nx) % ny
    ez = np.arange(nspec) // (nx * ny)
    want = cfg.get("absorbing", ["xmin", "xmax", "ymin", "ymax", "bottom"])
    conds = {"xmin": (1, ex == 0), "xmax": (2, ex == nx - 1), "ymin": (3, ey == 0), "ymax": (4, ey == ny - 1),
             "bottom": (5, ez == 0), "top": (6, ez == nz - 1)}
    for name in ["xmin", "xmax", "ymin", "ymax", "bottom", "top"]:
        if name in want:
            iface, sel = conds[name]
            faces += [(int(e) + 1, iface) for e in np.nonzero(sel)[0]]
    return _database(L, precision, cfg, anchors, xs, ys, zs, xtol, (rho, vp, vs), faces,
                     stacey=bool(cfg.get("stacey", True)))


_FACE_ANCHORS = {1: (0, 3, 7, 4), 2: (1, 2, 6, 5), 3: (0, 1, 5, 4), 4: (3, 2, 6, 7), 5: (0, 1, 2, 3), 6: (4, 5, 6, 7)}
_FACE_FILES = [("xmin", "absorbing_surface_file_xmin"), ("xmax", "absorbing_surface_file_xmax"),
               ("ymin", "absorbing_surface_file_ymin"), ("ymax", "absorbing_surface_file_ymax"),
               ("bottom", "absorbing_surface_file_bottom"), ("top", "free_or_absorbing_surface_file_zmax")]


def element_face_id(an: np.ndarray, corners: np.ndarray, tol: float) -> int:
    """get_element_face_id (get_element_face.f90:28-167) restated: the face of the
    element (anchors an (8,3)) whose four corner points coincide, within tol, with
    the four given corner coordinates (4,3), in any order."""
    for f, ids in _FACE_ANCHORS.items():
        pts = an[list(ids)]
        if all(np.min(np.abs(pts - c).max(axis=1)) <= tol for c in corners):
            return f
    raise ValueError("face corners do not match any face of the element")


def build_database_from_mesh(mesh: dict, cfg: dict, precision: str = "f32") -> dict:
    """The restated set-up chain for a general 8-node hexahedral mesh given as
    nodes (nnod,3), elems (nspec,8) 0-based, mat_id per element, materials {id:
    dict(domain, rho, vp, vs, ...)} and face lists {file name: (nf,5) [element,
    4 nodes] 0-based}, the content of the reference's MESH files.  Absorbing faces
    are found by coordinates like get_element_face_id."""
    L = lib(precision)
    nodes = np.asarray(mesh["nodes"], np.float64)
    elems = np.asarray(mesh["elems"], np.int64)
    nspec = len(elems)
    anchors = np.ascontiguousarray(nodes[elems].reshape(-1))
    npt = NGLL3 * nspec
    xs, ys, zs = np.zeros(npt), np.zeros(npt), np.zeros(npt)
    L.orc_gll_coordinates(nspec, _p(anchors), _p(xs), _p(ys), _p(zs))
    xtol = 1e-10 * abs(float(nodes[:, 0].max() - nodes[:, 0].min()))
    ids = sorted(mesh["materials"])
    mats = [mesh["materials"][i] for i in ids]
    lay = np.array([ids.index(int(m)) for m in mesh["mat_id"]], np.int64)
    per = np.repeat(lay, NGLL3)
    rho = np.array([m["rho"] for m in mats], np.float32)[per]
    vp = np.array([m["vp"] for m in mats], np.float32)[per]
    vs = np.array([0.0 if m["domain"] == 1 else m["vs"] for m in mats], np.float32)[per]
    want = cfg.get("absorbing", ["xmin", "xmax", "ymin", "ymax", "bottom"])
    an3 = anchors.reshape(nspec, 8, 3)
    tol = 1e-6 * (1.0 + float(np.abs(nodes).max()))
    faces = []
    for name, fname in _FACE_FILES:
        if name not in want or fname not in mesh["faces"]:
            continue
        for rec in mesh["faces"][fname]:
            e = int(rec[0])
            faces.append((e + 1, element_face_id(an3[e], nodes[rec[1:5]], tol)))
    cfg2 = dict(cfg, layers=[dict(m) for m in mats], elem_layer=lay)
    db = _database(L, precision, cfg2, anchors, xs, ys, zs, xtol, (rho, vp, vs), faces,
                   stacey=bool(cfg.get("stacey", True)))
    top = mesh["faces"].get("free_or_absorbing_surface_file_zmax", np.zeros((0, 5), np.int64))
    if "top" in want:
        top = np.zeros((0, 5), np.int64)
    db["free_surface_faces"] = [(int(r[0]) + 1, element_face_id(an3[int(r[0])], nodes[r[1:5]], tol))
                                for r in top]
    db["layers"], db["elem_layer"] = cfg2["layers"], lay
    return db


def _database(L, precision, cfg, anchors, xs, ys, zs, xtol, material, faces, stacey):
    """The set-up chain shared by block and general meshes, from the anchors, the
    GLL coordinates, per-point (rho, vp, vs) and the absorbing faces [(ispec, iface)]."""
    rd = real_dtype(precision)
    nspec = len(anchors) // 24
    npt = NGLL3 * nspec
    ibool = np.zeros(npt, np.int32)
    xc, yc, zc = xs.copy(), ys.copy(), zs.copy()
    nglob = L.orc_get_global(npt, _p(xc), _p(yc), _p(zc), _p(ibool), xtol)
    del xc, yc, zc
    metric = [np.zeros(npt, rd) for _ in range(10)]
    mptrs = (ctypes.c_void_p * 10)(*[_p(m) for m in metric])
    irreg = np.zeros(nspec, np.int32)
    xr = (ctypes.c_float if precision == "f32" else ctypes.c_double)(0)
    jr = (ctypes.c_float if precision == "f32" else ctypes.c_double)(0)
    nirr = L.orc_calc_jacobian_all(nspec, _p(anchors), ctypes.addressof(mptrs), _p(irreg),
                                   ctypes.addressof(xr), ctypes.addressof(jr))
    names = ["xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"]
    db = {n: m[: NGLL3 * max(nirr, 1)].copy() for n, m in zip(names, metric)}
    db.update(nspec=nspec, nglob=nglob, nspec_irregular=nirr, ibool=ibool, irregular_element_number=irreg,
              xix_regular=float(xr.value), jacobian_regular=float(jr.value), anchors=anchors,
              xstore=xs, ystore=ys, zstore=zs)
    rho, vp, vs = material
    rho_r, vp_r, vs_r = rho.astype(rd), vp.astype(rd), vs.astype(rd)
    db["rhostore"] = rho_r
    db["kappastore"] = (rho_r * (vp_r * vp_r - rd(4.0 / 3.0) * vs_r * vs_r)).astype(rd)
    db["mustore"] = (rho_r * vs_r * vs_r).astype(rd)
    db["rho_vp"] = (rho_r * vp_r).astype(rd)
    db["rho_vs"] = (rho_r * vs_r).astype(rd)
    db["vp"] = vp
    db["vs"] = vs
    db["ispec_is_acoustic"] = (np.asarray(vs, np.float32).reshape(nspec, NGLL3) == 0).all(axis=1).astype(np.int32)
    nf = len(faces)
    abs_ispec = np.array([f[0] for f in faces], np.int32)
    abs_ijk = np.zeros(3 * 25 * nf, np.int32)
    abs_jw = np.zeros(25 * nf, rd)
    abs_n = np.zeros(3 * 25 * nf, rd)
    for f, (ispec, iface) in enumerate(faces):
        ijk = np.zeros(75, np.int32)
        jw = np.zeros(25, rd)
        nn = np.zeros(75, rd)
        L.orc_face_geometry(_p(anchors[24 * (ispec - 1):]), iface, _p(ijk), _p(jw), _p(nn))
        abs_ijk[75 * f:75 * f + 75] = ijk
        abs_jw[25 * f:25 * f + 25] = jw
        abs_n[75 * f:75 * f + 75] = nn
    db.update(num_abs_boundary_faces=nf, abs_boundary_ispec=abs_ispec, abs_boundary_ijk=abs_ijk,
              abs_boundary_jacobian2Dw=abs_jw, abs_boundary_normal=abs_n)
    # mass matrices
    dt = float(cfg["dt"])
    rmass = np.zeros(nglob, rd)
    _mass_elastic(L, precision, nspec, nglob, db, rmass)
    rmx, rmy, rmz = np.zeros(nglob, rd), np.zeros(nglob, rd), np.zeros(nglob, rd)
    stacey = stacey and nf > 0
    if stacey:
        L.orc_mass_stacey_elastic(nglob, dt, _p(ibool), _p(db["rho_vp"]), _p(db["rho_vs"]), nf, _p(abs_ispec),
                                  _p(abs_ijk), _p(abs_n), _p(abs_jw), _p(rmx), _p(rmy), _p(rmz))
    L.orc_invert_mass(nglob, _p(rmass), _p(rmx), _p(rmy), _p(rmz), int(stacey))
    db.update(rmass=rmass, rmassx=rmx, rmassy=rmy, rmassz=rmz, stacey=int(stacey))
    db.update(derivation_matrices(precision))
    # sources and receivers
    _sources_receivers(L, precision, cfg, db)
    db["stf"], db["t0"] = source_time_functions(cfg, db.get("source_in_fluid"))
    db["attenuation"] = int(bool(cfg.get("attenuation", False)))
    if db["attenuation"]:
        db.update(attenuation_setup(db, cfg, precision))
    return db


def _mass_elastic(L, precision, nspec, nglob, db, rmass):
    fn = L.orc_mass_elastic
    rt = ctypes.c_float if precision == "f32" else ctypes.c_double
    fn.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + [rt, ctypes.c_void_p]
    fn(nspec, nglob, _p(db["ibool"]), _p(db["rhostore"]), _p(db["jacobian"]), _p(db["irregular_element_number"]),
       rt(db["jacobian_regular"]), _p(rmass))


def element_neighbours(ibool: np.ndarray, nspec: int):
    """CSR (xadj, adjncy) of every element's neighbours for the point search:
    elements sharing a corner with it and their own corner neighbours, in element
    order, the element itself excluded (setup_mesh_adjacency.f90 adds neighbours
    of neighbours the same way)."""
    from scipy import sparse
    ib = np.asarray(ibool).reshape(nspec, NGLL3) - 1
    corners = ib[:, [0, 4, 20, 24, 100, 104, 120, 124]].reshape(-1)
    A = sparse.csr_matrix((np.ones(8 * nspec), (np.repeat(np.arange(nspec), 8), corners)),
                          shape=(nspec, int(ib.max()) + 1))
    r1 = (A @ A.T).astype(bool).astype(np.int32)
    r2 = (r1 @ r1).tocsr()
    r2.setdiag(0)
    r2.eliminate_zeros()
    r2.sort_indices()
    return r2.indptr.astype(np.int32), (r2.indices.astype(np.int32) if r2.nnz else np.zeros(1, np.int32))


def surface_points(ibool: np.ndarray, nspec: int) -> np.ndarray:
    """Per element GLL point (125*nspec, uint8): 1 where the point lies on a face
    that only one element has, the mesh's outer surface (iglob_is_surface_external_mesh)."""
    ib = np.asarray(ibool).reshape(nspec, NGLL3) - 1
    count = {}
    faces = []
    for e in range(nspec):
        for f, corners in _FACE_CORNERS.items():
            key = tuple(sorted(int(ib[e][i + 5 * j + 25 * k]) for i, j, k in corners))
            count[key] = count.get(key, 0) + 1
            faces.append((e, f, key))
    on = np.zeros(int(ib.max()) + 1, bool)
    for e, f, key in faces:
        if count[key] == 1:
            c = (f - 1) // 2
            v = 0 if f % 2 == 1 else NGLL - 1
            for a in range(NGLL):
                for b in range(NGLL):
                    ijk = [a, b]
                    ijk.insert(c, v)
                    on[ib[e][ijk[0] + 5 * ijk[1] + 25 * ijk[2]]] = True
    return on[ib].reshape(-1).astype(np.uint8)


def locate(L, db, x, y, z, octant=None):
    """(ispec 1-based, xi, eta, gamma) of a target through orc_locate_point, with
    the element neighbours and outer-surface points of the mesh (computed once)."""
    nspec = db["nspec"]
    if "_nb" not in db:
        db["_nb"] = element_neighbours(db["ibool"], nspec)
        db["_surf"] = surface_points(db["ibool"], nspec)
        db["_isac"] = np.asarray(db.get("ispec_is_acoustic", np.zeros(nspec, np.int32)), np.int32)
    xi, eta, ga = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    xadj, adj = db["_nb"]
    ispec = L.orc_locate_point(nspec, _p(db["anchors"]), _p(db["xstore"]), _p(db["ystore"]), _p(db["zstore"]),
                               _p(xadj), _p(adj), _p(db["_surf"]), _p(db["_isac"]), float(x), float(y), float(z),
                               ctypes.addressof(xi), ctypes.addressof(eta), ctypes.addressof(ga))
    if octant is not None:
        # a target on element boundaries placed in the element on the given side:
        # the first element whose anchor box holds it and whose centre lies on
        # that side, then the location restricted to that element
        an = db["anchors"].reshape(nspec, 8, 3)
        xt = np.array([float(x), float(y), float(z)])
        inside = np.nonzero(((an.min(1) <= xt) & (xt <= an.max(1))).all(1))[0]
        side = (np.sign(an[inside].mean(1) - xt) == np.sign(np.asarray(octant, float))).all(1)
        if side.any():
            e = int(inside[side][0])
            sl = slice(NGLL3 * e, NGLL3 * (e + 1))
            one = [np.ascontiguousarray(db[k][sl]) for k in ("xstore", "ystore", "zstore")]
            L.orc_locate_point(1, _p(np.ascontiguousarray(an[e].reshape(-1))), _p(one[0]), _p(one[1]), _p(one[2]),
                               None, None, None, None, xt[0], xt[1], xt[2], ctypes.addressof(xi),
                               ctypes.addressof(eta), ctypes.addressof(ga))
            ispec = e + 1
    return ispec, xi.value, eta.value, ga.value


def _sources_receivers(L, precision, cfg, db):
    rd = real_dtype(precision)
    nspec = db["nspec"]
    names = ["xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"]
    mptrs = (ctypes.c_void_p * 10)(*[_p(db[n]) for n in names])
    xgl, _ = gll()
    srcs = cfg.get("sources", [])
    ns = len(srcs)
    sa = np.zeros((ns, 3, NGLL3), rd)  # (isrc, c, ijk) -> stored (NSOURCES,3,5,5,5) column-major
    isel = np.zeros(ns, np.int32)
    loc = np.zeros((ns, 3))
    src_fluid = []
    for i, s in enumerate(srcs):
        ispec, xi, eta, ga = locate(L, db, s["x"], s["y"], s["z"], s.get("octant"))
        isel[i] = ispec
        loc[i] = (xi, eta, ga)
        out = np.zeros(3 * NGLL3, rd)
        fluid = bool(np.asarray(db["ispec_is_acoustic"])[ispec - 1]) if "ispec_is_acoustic" in db else False
        src_fluid.append(fluid)
        if s.get("type", "cmt") == "cmt" and fluid:
            # setup_sources_receivers.f90:1187-1212: scalar moment M0 (Dahlen &
            # Tromp 5.91) scaled to the equivalent explosion, on all components
            Mxx, Myy, Mzz, Mxy, Mxz, Myz = (float(v) for v in s["M"])
            m0 = np.sqrt(0.5 * (Mxx * Mxx + Myy * Myy + Mzz * Mzz + 2.0 * (Myz * Myz + Mxz * Mxz + Mxy * Mxy)))
            fac = float(m0 * np.sqrt(2.0 / 3.0))
            L.orc_source_array_force(xi, eta, ga, fac, fac, fac, _p(out))
        elif s.get("type", "cmt") == "cmt":
            Mxx, Myy, Mzz, Mxy, Mxz, Myz = (float(v) for v in s["M"])
            rt = ctypes.c_float if precision == "f32" else ctypes.c_double
            L.orc_source_array_cmt(ispec, _p(db["irregular_element_number"]), ctypes.addressof(mptrs),
                                   rt(db["xix_regular"]), xi, eta, ga,
                                   Mxx, Myy, Mzz, Mxy, Mxz, Myz, _p(out))
        else:
            f = [float(v) for v in s["F"]]
            L.orc_source_array_force(xi, eta, ga, f[0], f[1], f[2], _p(out))
        sa[i] = out.reshape(NGLL3, 3).T
    # Fortran sourcearrays(NSOURCES,NDIM,NGLLX,NGLLY,NGLLZ): isrc fastest
    db["sourcearrays"] = np.ascontiguousarray(sa.transpose(2, 1, 0)).reshape(-1)
    db["ispec_selected_source"] = isel
    db["source_xi_eta_gamma"] = loc
    db["source_in_fluid"] = np.asarray(src_fluid, bool)
    recs = cfg.get("receivers", [])
    nr = len(recs)
    irec = np.zeros(nr, np.int32)
    hx, he, hg = np.zeros((nr, NGLL)), np.zeros((nr, NGLL)), np.zeros((nr, NGLL))
    rloc = np.zeros((nr, 3))
    for r, (x, y, z) in enumerate(recs):
        ispec, xi, eta, ga = locate(L, db, x, y, z)
        irec[r] = ispec
        rloc[r] = (xi, eta, ga)
        hx[r], _ = lagrange_any(xi)
        he[r], _ = lagrange_any(eta)
        hg[r], _ = lagrange_any(ga)
    db.update(ispec_selected_rec=irec, hxir=hx.reshape(-1), hetar=he.reshape(-1), hgammar=hg.reshape(-1),
              receiver_xi_eta_gamma=rloc, nrec=nr, nsources=ns)


def source_time_functions(cfg: dict, in_fluid=None) -> np.ndarray:
    """(NSOURCES, NSTEP) FP64 table following setup_sources_receivers.f90:482-491
    for t0 and get_stf_viscoelastic (compute_add_sources_viscoelastic.F90:837-932).
    Sources in fluid elements: a moment tensor takes the Gaussian instead of the
    Heaviside (get_stf_acoustic), and a Gaussian there sets t0 to at least
    3 (hdur - tshift) (setup_sources_receivers.f90:495-514)."""
    srcs = cfg.get("sources", [])
    dt, nstep = float(cfg["dt"]), int(cfg["nstep"])
    if not srcs:
        return np.zeros((0, nstep)), 0.0
    fl = list(in_fluid) if in_fluid is not None else [False] * len(srcs)
    kinds = []
    for s, f in zip(srcs, fl):
        k = s.get("stf", "ricker")
        if f and s.get("type", "cmt") == "cmt" and k == "heaviside":
            k = "gaussian"
        kinds.append(k)
    params = [float(s["f0"]) if k == "ricker" else float(s["hdur"]) for s, k in zip(srcs, kinds)]
    tsh = np.array([float(s.get("tshift", 0.0)) for s in srcs])
    tsh = tsh - tsh.min() if len(srcs) > 1 else np.zeros(1)
    if all(k == "ricker" for k in kinds):
        t0 = -1.2 * min(ts - 1.0 / p for ts, p in zip(tsh, params))
    else:
        t0 = -2.0 * min(ts - p for ts, p in zip(tsh, params))
    for f, k, ts, p in zip(fl, kinds, tsh, params):
        if f and k == "gaussian" and -3.0 * (ts - p) > t0:
            t0 = -3.0 * (ts - p)
    if "t0" in cfg:
        t0 = float(cfg["t0"])
    return np.stack([stf_table(k, p, ts, t0, dt, nstep) for k, p, ts in zip(kinds, params, tsh)]), t0


ANISO_NAMES = ["c11store", "c12store", "c13store", "c14store", "c15store", "c16store", "c22store", "c23store",
               "c24store", "c25store", "c26store", "c33store", "c34store", "c35store", "c36store", "c44store",
               "c45store", "c46store", "c55store", "c56store", "c66store"]


def make_sim(db: dict, cfg: dict, precision: str = "f32", nthreads: int = 1) -> OracleSim:
    """Oracle forward simulation set up from database arrays (either the ones
    from :func:`build_database` or the product's generator, same names)."""
    rd = real_dtype(precision)
    s = OracleSim(precision)
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    s.seti("nspec", nspec)
    s.seti("nglob", nglob)
    s.seti("nspec_irregular", int(db["nspec_irregular"]))
    s.seti("nthreads", nthreads)
    for n in ["ibool", "irregular_element_number", "abs_boundary_ispec", "abs_boundary_ijk", "ispec_selected_source",
              "ispec_selected_rec"]:
        s.set(n, np.asarray(db[n], np.int32))
    for n in ["xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian", "kappastore",
              "mustore", "rho_vp", "rho_vs", "rmassx", "rmassy", "rmassz", "hprime_xx", "hprimewgll_xx",
              "wgllwgll_xy", "wgllwgll_xz", "wgllwgll_yz", "abs_boundary_normal", "abs_boundary_jacobian2Dw",
              "sourcearrays"]:
        s.set(n, np.asarray(db[n], rd))
    for n in ["hxir", "hetar", "hgammar"]:
        s.set(n, np.asarray(db[n], np.float64))
    if int(db.get("anisotropy", 0)):
        s.set("cstore", np.ascontiguousarray(np.stack([np.asarray(db[n], rd) for n in ANISO_NAMES], axis=1)))
    s.setr("xix_regular", db["xix_regular"])
    s.setr("jacobian_regular", db["jacobian_regular"])
    # C-PML keeps the outer faces for its Dirichlet condition (no Stacey terms)
    s.seti("num_abs_boundary_faces",
           int(db["num_abs_boundary_faces"]) if (db.get("stacey", 1) or db.get("pml", 0)) else 0)
    s.seti("stacey", int(db.get("stacey", 1)))
    dt = float(cfg["dt"])
    dtr = rd(dt)
    s.setr("deltat", dtr)
    s.setr("deltatover2", dtr / rd(2))
    s.setr("deltatsqover2", dtr * dtr / rd(2))
    nstep = int(cfg["nstep"])
    s.seti("nstep", nstep)
    ns = int(db["nsources"])
    s.seti("nsources", ns)
    if ns:
        stf = np.asarray(db["stf"], np.float64).reshape(ns, nstep)
        s.set("stf", np.ascontiguousarray(stf.T).reshape(-1))
    nr = int(db["nrec"])
    s.seti("nrec", nr)
    if nr:
        s.set("seismograms", np.zeros(3 * nr * nstep))
    for n in ["displ", "veloc", "accel"]:
        s.set(n, np.zeros(3 * nglob, rd))
    if int(db.get("pml", 0)):
        _set_pml(s, db, rd)
    att = int(db.get("attenuation", 0))
    s.seti("attenuation", att)
    s.seti("compute_and_store_strain", att)
    if att:
        for n in ["alphaval", "betaval", "gammaval", "factor_common", "factor_common_kappa"]:
            s.set(n, np.asarray(db[n], rd))
        for n in ["R_xx", "R_yy", "R_xy", "R_xz", "R_yz", "R_trace"]:
            s.set(n, np.zeros(N_SLS * NGLL3 * nspec, rd))
        for n in ["epsilondev_xx", "epsilondev_yy", "epsilondev_xy", "epsilondev_xz", "epsilondev_yz",
                  "epsilondev_trace"]:
            s.set(n, np.zeros(NGLL3 * nspec, rd))
    return s


def _set_pml(s, db, rd):
    """C-PML arrays of a database from specfem3d_gb300.pml.setup (layouts of
    prepare_timerun_pml: coefficient index fastest, then GLL point, then CPML element)."""
    from specfem3d_gb300.meshgen import WGLL
    n = len(db["cpml_to_spec"])
    nspec = int(db["nspec"])
    s.seti("nspec_cpml", n)
    s.set("is_cpml", np.asarray(db["is_cpml"], np.int32))
    s.set("cpml_to_spec", np.asarray(db["cpml_to_spec"], np.int32))
    s2c = np.zeros(nspec, np.int32)
    s2c[np.asarray(db["cpml_to_spec"]) - 1] = np.arange(1, n + 1, dtype=np.int32)
    s.set("spec_to_cpml", s2c)
    for k in ("alpha", "beta", "abar", "strain"):
        s.set("pml_coef_" + k, np.ascontiguousarray(np.asarray(db["pml_coef_" + k], rd)).reshape(-1))
    w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1)
    s.set("wgll_cube", w3.astype(rd))
    s.set("rhostore", np.asarray(db["rhostore"], rd))
    s.set("pml_displ_old", np.zeros(3 * 125 * n, rd))
    s.set("pml_displ_new", np.zeros(3 * 125 * n, rd))
    s.set("pml_rmem", np.zeros(48 * 125 * n, rd))


def seismograms(sim: OracleSim) -> np.ndarray:
    """(nrec, 3, nstep) traces recorded so far."""
    nr, nstep = sim.geti("nrec"), sim.geti("nstep")
    return sim.get("seismograms").reshape(nstep, nr, 3).transpose(1, 2, 0)


# ----------------------------------------------------------------------------
# attenuation (shared/get_attenuation_model.f90, specfem3D/prepare_attenuation.f90)
# ----------------------------------------------------------------------------

ATTENUATION_COMP_MAXIMUM = 9000.0
ATTENUATION_F0_REFERENCE = 18.0  # the reference's default Par_file value


def min_resolved_period(db: dict) -> float:
    """check_mesh_resolution.f90:200-280 in single precision: per element
    (max corner edge / (NGLL-1)) / min(vp, vs) * NPTS_PER_WAVELENGTH, maximum over
    elements."""
    f32 = np.float32
    nspec = db["nspec"]
    an = db["anchors"].reshape(nspec, 8, 3).astype(f32)
    edges = [(0, 1), (3, 2), (4, 5), (7, 6), (0, 3), (1, 2), (4, 7), (5, 6), (0, 4), (1, 5), (3, 7), (2, 6)]
    d2 = np.stack([((an[:, a] - an[:, b]) ** 2).sum(axis=1) for a, b in edges], axis=1).astype(f32)
    emax = np.sqrt(d2.max(axis=1)).astype(f32)
    kap = db["kappastore"].reshape(nspec, NGLL3).astype(f32)
    mu = db["mustore"].reshape(nspec, NGLL3).astype(f32)
    rho = db["rhostore"].reshape(nspec, NGLL3).astype(f32)
    vp = np.sqrt((kap + f32(4.0 / 3.0) * mu) / rho).astype(f32)
    vs = np.sqrt(mu / rho).astype(f32)
    vmin = np.minimum(vp.min(axis=1), vs.min(axis=1))
    pmax = (emax / f32(NGLL - 1)) / vmin * f32(5.0)
    return float(pmax.max())


def attenuation_setup(db: dict, cfg: dict, precision: str = "f32") -> dict:
    """Restated attenuation set-up: factor_common(_kappa) (N_SLS,5,5,5,NSPEC),
    unrelaxed-modulus scaling of mustore/kappastore, alpha/beta/gamma values."""
    L = lib(precision)
    rd = real_dtype(precision)
    dp = ctypes.POINTER(ctypes.c_double)
    L.orc_attenuation_constants.argtypes = [ctypes.c_double, dp, dp, dp, dp]
    L.orc_attenuation_factors.argtypes = [ctypes.c_double, dp, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, dp, dp, dp, dp]
    mrp = min_resolved_period(db)
    tau_sigma = (ctypes.c_double * N_SLS)()
    fc, tmin, tmax = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    L.orc_attenuation_constants(mrp, tau_sigma, ctypes.byref(fc), ctypes.byref(tmin), ctypes.byref(tmax))
    ts = np.array(tau_sigma[:])
    tau_f = ts.astype(rd)
    tauinv = (rd(1) / tau_f).astype(rd)
    nspec = db["nspec"]
    lay = np.asarray(cfg["elem_layer"], np.int64)
    cache = {}

    def factors(Q):
        Q = min(max(float(Q), 1.0), ATTENUATION_COMP_MAXIMUM)
        if Q not in cache:
            beta = (ctypes.c_double * N_SLS)()
            omsb, sf = ctypes.c_double(), ctypes.c_double()
            te = (ctypes.c_double * N_SLS)()
            L.orc_attenuation_factors(Q, tau_sigma, tmin.value, tmax.value, fc.value, ATTENUATION_F0_REFERENCE,
                                      beta, ctypes.byref(omsb), ctypes.byref(sf), te)
            cache[Q] = (np.array(beta[:]), omsb.value, sf.value)
        return cache[Q]

    fcm = np.zeros((nspec, NGLL3, N_SLS), rd)
    fck = np.zeros((nspec, NGLL3, N_SLS), rd)
    smu = np.ones((nspec, NGLL3), rd)
    skap = np.ones((nspec, NGLL3), rd)
    for li, m in enumerate(cfg["layers"]):
        sel = lay == li
        if not sel.any():
            continue
        bm, om, sm = factors(np.float32(m["Qmu"]))
        bk, ok_, sk = factors(np.float32(m.get("Qkappa", 9999.0)))
        fcm[sel] = ((2.0 * bm * tauinv.astype(np.float64)) / om).astype(rd)
        fck[sel] = ((bk * tauinv.astype(np.float64)) / ok_).astype(rd)
        smu[sel] = rd(sm)
        skap[sel] = rd(sk)
    out = dict(factor_common=np.ascontiguousarray(fcm).reshape(-1),
               factor_common_kappa=np.ascontiguousarray(fck).reshape(-1),
               mustore=(db["mustore"] * smu.reshape(-1)).astype(rd),
               kappastore=(db["kappastore"] * skap.reshape(-1)).astype(rd),
               tau_sigma=tau_f, f_c_source=fc.value, min_period=tmin.value, max_period=tmax.value,
               min_resolved_period=mrp)
    al, be, ga = (np.zeros(N_SLS, rd) for _ in range(3))
    rt = ctypes.c_float if precision == "f32" else ctypes.c_double
    L.orc_attenuation_memory_values.argtypes = [ctypes.c_void_p, rt, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]
    L.orc_attenuation_memory_values(_p(tau_f), rt(rd(cfg["dt"])), _p(al), _p(be), _p(ga))
    out.update(alphaval=al, betaval=be, gammaval=ga, attenuation=1)
    return out


# ----------------------------------------------------------------------------
# fluid domain set-up (generate_databases/get_coupling_surfaces.f90:240-380,
# shared/define_mass_matrices.f90:100-160, :460-520)
# ----------------------------------------------------------------------------

_FACE_CORNERS = {1: [(0, 0, 0), (0, 4, 0), (0, 4, 4), (0, 0, 4)], 2: [(4, 0, 0), (4, 4, 0), (4, 4, 4), (4, 0, 4)],
                 3: [(0, 0, 0), (4, 0, 0), (4, 0, 4), (0, 0, 4)], 4: [(0, 4, 0), (4, 4, 0), (4, 4, 4), (0, 4, 4)],
                 5: [(0, 0, 0), (4, 0, 0), (4, 4, 0), (0, 4, 0)], 6: [(0, 0, 4), (4, 0, 4), (4, 4, 4), (0, 4, 4)]}
_FACE_MID = {1: (0, 2, 2), 2: (4, 2, 2), 3: (2, 0, 2), 4: (2, 4, 2), 5: (2, 2, 0), 6: (2, 2, 4)}


def fluid_setup(db: dict, cfg: dict, precision: str = "f32") -> dict:
    """Fluid flags, fluid-solid coupling faces (every face of a fluid element whose
    four corners and midpoint are shared with solid elements, first time seen),
    free-surface faces and the fluid mass matrix with its Stacey term."""
    L = lib(precision)
    rd = real_dtype(precision)
    nspec, nglob = db["nspec"], db["nglob"]
    ib = db["ibool"].reshape(nspec, NGLL3) - 1
    vs = np.asarray(db["vs"], np.float32).reshape(nspec, NGLL3)
    isac = (vs == 0).all(axis=1)
    out = {"ispec_is_acoustic": isac.astype(np.int32)}
    elastic_flag = np.zeros(nglob, np.int32)
    for e in np.nonzero(~isac)[0]:
        elastic_flag[ib[e]] = 1
    mask = np.zeros(nglob, bool)
    faces = []
    for e in np.nonzero(isac)[0]:
        for f in range(1, 7):
            corners = [ib[e][i + 5 * j + 25 * k] for i, j, k in _FACE_CORNERS[f]]
            if all(elastic_flag[c] >= 1 for c in corners):
                i, j, k = _FACE_MID[f]
                mid = ib[e][i + 5 * j + 25 * k]
                fijk = np.zeros(75, np.int32)
                jw = np.zeros(25, rd)
                nn = np.zeros(75, rd)
                L.orc_face_geometry(_p(db["anchors"][24 * e:]), f, _p(fijk), _p(jw), _p(nn))
                pts = [ib[e][(fijk[3 * g] - 1) + 5 * (fijk[3 * g + 1] - 1) + 25 * (fijk[3 * g + 2] - 1)] for g in range(25)]
                if not mask[mid] and elastic_flag[mid] >= 1:
                    faces.append((e + 1, fijk, jw, nn))
                mask[pts] = True
    nf = len(faces)
    out["num_coupling_ac_el_faces"] = nf
    out["coupling_ac_el_ispec"] = np.array([f[0] for f in faces], np.int32)
    out["coupling_ac_el_ijk"] = np.concatenate([f[1] for f in faces]) if nf else np.zeros(0, np.int32)
    out["coupling_ac_el_jacobian2Dw"] = np.concatenate([f[2] for f in faces]) if nf else np.zeros(0, rd)
    out["coupling_ac_el_normal"] = np.concatenate([f[3] for f in faces]) if nf else np.zeros(0, rd)
    # free surface: the listed faces of a general mesh, else the top faces of the
    # block (face 6 of the top element row)
    if "free_surface_faces" in db:
        fsf = db["free_surface_faces"]
    else:
        nx, ny = int(cfg["nx"]), int(cfg["ny"])
        nz = len(cfg["zlev"]) - 1
        fsf = [(int(e) + 1, 6) for e in range(nx * ny * (nz - 1), nx * ny * nz)]
    fs = []
    for e1, f in fsf:
        fs_ijk = np.zeros(75, np.int32)
        _jw = np.zeros(25, rd)
        _n = np.zeros(75, rd)
        L.orc_face_geometry(_p(db["anchors"][24 * (e1 - 1):]), f, _p(fs_ijk), _p(_jw), _p(_n))
        fs.append(fs_ijk)
    out["num_free_surface_faces"] = len(fsf)
    out["free_surface_ispec"] = np.array([e1 for e1, _ in fsf], np.int32)
    out["free_surface_ijk"] = np.concatenate(fs) if fs else np.zeros(0, np.int32)
    # fluid mass matrix: sum J w / kappa, plus dt/2 jw / (rho vp) on absorbing faces
    x, w = gll()
    w3 = np.array([w[i] * w[j] * w[k] for k in range(5) for j in range(5) for i in range(5)])
    irr = db["irregular_element_number"]
    rma = np.zeros(nglob, rd)
    kap = db["kappastore"].reshape(nspec, NGLL3)
    for e in np.nonzero(isac)[0]:
        jl = (db["jacobian"].reshape(-1, NGLL3)[irr[e] - 1] if irr[e] else np.full(NGLL3, db["jacobian_regular"]))
        terms = (jl.astype(np.float64) * w3 / kap[e].astype(np.float64)).astype(rd)
        for p in range(NGLL3):
            rma[ib[e][p]] += terms[p]
    if db.get("stacey", 0):
        dt2 = rd(0.5 * float(cfg["dt"]))
        nfa = db["num_abs_boundary_faces"]
        for fidx in range(nfa):
            e = db["abs_boundary_ispec"][fidx] - 1
            if not isac[e]:
                continue
            for g in range(25):
                i, j, k = (db["abs_boundary_ijk"][3 * (g + 25 * fidx) + c] - 1 for c in range(3))
                q = e * NGLL3 + i + 5 * j + 25 * k
                rma[ib[e][i + 5 * j + 25 * k]] += db["abs_boundary_jacobian2Dw"][g + 25 * fidx] * (dt2 / db["rho_vp"][q])
    rma[rma <= 0] = 1
    out["rmass_acoustic"] = (rd(1) / rma).astype(rd)
    # solid mass only over solid elements
    m = np.zeros(nglob, rd)
    for e in np.nonzero(~isac)[0]:
        jl = (db["jacobian"].reshape(-1, NGLL3)[irr[e] - 1] if irr[e] else np.full(NGLL3, db["jacobian_regular"]))
        terms = (jl.astype(np.float64) * w3 * db["rhostore"].reshape(nspec, NGLL3)[e].astype(np.float64)).astype(rd)
        for p in range(NGLL3):
            m[ib[e][p]] += terms[p]
    out["rmass_solid"] = m
    return out


def make_coupled_sim(db: dict, cfg: dict, precision: str = "f32", nthreads: int = 1) -> OracleSim:
    """Oracle coupled fluid-solid simulation on the given database arrays."""
    rd = real_dtype(precision)
    s = make_sim(db, cfg, precision, nthreads)
    isac = np.asarray(db["ispec_is_acoustic"], np.int32)
    s.set("ispec_is_acoustic", isac)
    el = (np.nonzero(isac == 0)[0] + 1).astype(np.int32)
    ac = (np.nonzero(isac)[0] + 1).astype(np.int32)
    s.set("elastic_list", el)
    s.seti("n_elastic", len(el))
    s.set("acoustic_list", ac)
    s.seti("n_acoustic", len(ac))
    s.set("rhostore", np.asarray(db["rhostore"], rd))
    for n in ["potential", "potential_dot", "potential_dot_dot"]:
        s.set(n, np.zeros(int(db["nglob"]), rd))
    s.set("rmass_acoustic", np.asarray(db["rmass_acoustic"], rd))
    s.seti("num_coupling_faces", int(db["num_coupling_ac_el_faces"]))
    s.set("coupling_ispec", np.asarray(db["coupling_ac_el_ispec"], np.int32))
    s.set("coupling_ijk", np.asarray(db["coupling_ac_el_ijk"], np.int32))
    s.set("coupling_normal", np.asarray(db["coupling_ac_el_normal"], rd))
    s.set("coupling_jacobian2Dw", np.asarray(db["coupling_ac_el_jacobian2Dw"], rd))
    s.seti("num_free_surface_faces", int(db["num_free_surface_faces"]))
    s.set("free_surface_ispec", np.asarray(db["free_surface_ispec"], np.int32))
    s.set("free_surface_ijk", np.asarray(db["free_surface_ijk"], np.int32))
    recs = np.asarray(db["ispec_selected_rec"], np.int64) - 1
    s.set("rec_is_acoustic", isac[recs].astype(np.int32) if len(recs) else np.zeros(1, np.int32))
    s.L.orc_run_coupled.argtypes = [ctypes.c_void_p, ctypes.c_int]
    return s


def run_coupled(sim: OracleSim, nsteps: int) -> None:
    sim.L.orc_run_coupled(sim.h, int(nsteps))


# ----------------------------------------------------------------------------
# Gaussian smoothing of kernels (kernels/process_smooth.cu:30-194 and
# normalize_data, smooth_sem.F90:524-559 for the constants)
# ----------------------------------------------------------------------------

def smooth_restated(xyz_me: np.ndarray, xyz_other: np.ndarray, data_other: np.ndarray, integ_other: np.ndarray,
                    sigma_h2: float, sigma_v2: float, sigma_h3: float, sigma_v3: float) -> np.ndarray:
    """Smoothed kernels (nker, nspec_me*125) in FP64 from per-element coordinates
    xyz_me (nspec_me, 125, 3), xyz_other (nspec_other, 125, 3), kernel values
    data_other (nker, nspec_other*125) and J w weights integ_other (nspec_other*125).
    Element o of the other slice takes part for target element e when its centre
    (mean of its first and last GLL point, single precision) lies within sigma_h3
    horizontally and sigma_v3 vertically of GLL point (o mod 125) of e; each pair
    of points weighs exp(-dh/sigma_h2 - dv/sigma_v2) (0 below exp(-86)) times J w."""
    f32 = np.float32
    xo = np.asarray(xyz_other, f32)
    centre = ((xo[:, 0, :] + xo[:, NGLL3 - 1, :]) * f32(0.5)).astype(np.float64)
    no = len(xo)
    dat = np.asarray(data_other, np.float64).reshape(-1, no, NGLL3)
    integ = np.asarray(integ_other, np.float64).reshape(no, NGLL3)
    xo64 = xo.astype(np.float64)
    hcrit, vcrit = float(f32(sigma_h3) * f32(sigma_h3)), float(f32(sigma_v3) * f32(sigma_v3))
    h2inv, v2inv = 1.0 / float(f32(sigma_h2)), 1.0 / float(f32(sigma_v2))
    me = np.asarray(xyz_me, f32).astype(np.float64)
    out = np.zeros((dat.shape[0], len(me), NGLL3))
    pidx = np.arange(no) % NGLL3
    for e in range(len(me)):
        p = me[e][pidx]                                     # the testing point of each candidate
        dh = (p[:, 0] - centre[:, 0]) ** 2 + (p[:, 1] - centre[:, 1]) ** 2
        dv = (p[:, 2] - centre[:, 2]) ** 2
        inc = np.nonzero(~((dh > hcrit) | (dv > vcrit)))[0]
        if not len(inc):
            continue
        q = xo64[inc].reshape(-1, 3)                        # (n_inc*125, 3)
        ddh = (me[e][:, None, 0] - q[None, :, 0]) ** 2 + (me[e][:, None, 1] - q[None, :, 1]) ** 2
        ddv = (me[e][:, None, 2] - q[None, :, 2]) ** 2
        val = -ddh * h2inv - ddv * v2inv
        g = np.where(val < -86.0, 0.0, np.exp(np.maximum(val, -86.0)))
        coef = g * integ[inc].reshape(-1)[None, :]
        norm = coef.sum(axis=1)
        norm = np.where(norm < 1e-24, 1.0, norm)
        out[:, e, :] = np.einsum("pq,kq->kp", coef, dat[:, inc, :].reshape(dat.shape[0], -1)) / norm[None, :]
    return out.reshape(dat.shape[0], -1)


# ------------------------------------------------------------------ misfit post-processing
def adjoint_source(kind: int, syn, dat, dt: float, t0: float, ts: float, te: float, component: int = 0):
    """Adjoint sources of utils/adjoint_sources/*/create_adjsrc_*.f90, one trace at a
    time in sample order (the tools' real*8 loops): syn, dat (nrec, 3, nstep); kind 0
    waveform (create_adjsrc_waveform.f90:222-287), 1 cross-correlation traveltime
    (create_adjsrc_traveltime.f90:131-162), 2 amplitude (create_adjsrc_amplitude.f90:
    130-157).  Returns (adj (nrec, 3, nstep), norms (nrec, 3))."""
    syn = np.asarray(syn, np.float64)
    dat = None if dat is None else np.asarray(dat, np.float64)
    nrec, _, nstep = syn.shape
    pi = 3.1415926                                    # the waveform tool's PI parameter
    eps = 1.0e-17
    istart = int((ts - t0) / dt) + 1
    iend = int((te - t0) / dt) + 1
    if istart < 1 or iend <= istart or iend > nstep:
        raise ValueError("Error in ts, te")
    tw = np.zeros(nstep + 1)                          # 1-based
    if kind == 0:
        taper = int(0.1 * (iend - istart))            # 10 percent taper length
        for j in range(istart, iend + 1):
            if j < istart + taper:
                tw[j] = (1.0 - np.cos(pi * 2.0 * (j - istart) / (taper - 1))) / 2.0
            elif j <= iend - taper:
                tw[j] = 1.0
            else:
                tw[j] = (1.0 - np.cos(pi * 2.0 * (iend - j) / (taper - 1))) / 2.0
    else:
        for j in range(istart, iend + 1):
            tw[j] = 1 - (2 * (float(j) - istart) / (iend - istart) - 1) ** 2
    tw = tw[1:]
    adj = np.zeros_like(syn)
    norms = np.zeros((nrec, 3))
    for r in range(nrec):
        for c in range(3):
            s = syn[r, c]
            if kind == 0:
                out = s - dat[r, c]
            elif kind == 1:
                out = np.zeros(nstep)
                for it in range(1, nstep - 1):
                    out[it] = (s[it + 1] - s[it - 1]) / (2 * dt)
                out[0] = (s[1] - s[0]) / dt
                out[nstep - 1] = (s[nstep - 1] - s[nstep - 2]) / dt
            else:
                out = s.copy()
            norm = dt * np.sum(tw * out * out)
            if component != 0 and component != c + 1:
                norm = 0.0
            if abs(norm) > eps:
                adj[r, c] = out * tw if kind == 0 else (-out * tw / norm if kind == 1 else out * tw / norm)
            norms[r, c] = norm
    return adj, norms


def sum_kernels(kernels, masks=None):
    """Sum of event kernels (src/tomography/sum_kernels.f90:215-315) in FP64: each
    kernel's norm sum(k*k) before masking (:267), masked by its source mask (:289),
    accumulated (:293).  Returns (total, norms)."""
    total = None
    norms = []
    for q, k in enumerate(kernels):
        k = np.asarray(k, np.float64)
        norms.append(float(np.sum(k * k)))
        if masks is not None:
            k = k * np.asarray(masks[q], np.float64)
        total = k.copy() if total is None else total + k
    return total, np.asarray(norms)
