"""Databases of general 8-node hexahedral meshes, and the reference's external mesh files.

The reference turns a CUBIT/Gmsh mesh (``MESH/nodes_coords_file``, ``mesh_file``,
``materials_file``, ``nummaterial_velocity_file``, ``absorbing_surface_file_*``,
``free_or_absorbing_surface_file_zmax``) into solver databases with
xdecompose_mesh + xgenerate_databases.  This module does the same for one
partition, vectorised with numpy, restating:

* GLL point coordinates from the 8 anchor nodes (shape functions of
  shared/get_shape3D.f90 for NGNOD = 8);
* global numbering with a coordinate tolerance (shared/get_global.f90:28-141,
  sort_array_coordinates.f90:30-128), renumbered by first appearance in element
  order (get_global_indirect_addressing);
* Jacobian and metric at every GLL point, and the regular-element rule
  (generate_databases/calc_jacobian.f90:28-360);
* boundary faces from the face files: which element face, its GLL points in the
  order of get_element_face.f90:169-279, outward unit normal and weighted 2-D
  Jacobian (get_jacobian_boundaries.f90:28-297);
* fluid/solid coupling faces between acoustic and elastic elements
  (get_coupling_surfaces.f90) and the free surface of the fluid;
* mass matrices (define_mass_matrices.f90, incl. the Stacey term);
* point location: closest GLL point, then Newton iterations on the local
  coordinates (locate_point.f90:32-416, :422-624).

The result is the same database dict as :func:`meshgen.build_database`, so
:class:`solver.GPUSolver` runs it unchanged.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .meshgen import NGLL, NGLL3, WGLL, XIGLL as GLL, derivation_matrices, lagrange, stf_table

# reference coordinates of the 8 anchors (SPECFEM HEX8 order)
ANCHOR_XI = np.array([-1, 1, 1, -1, -1, 1, 1, -1], np.float64)
ANCHOR_ETA = np.array([-1, -1, 1, 1, -1, -1, 1, 1], np.float64)
ANCHOR_GA = np.array([-1, -1, -1, -1, 1, 1, 1, 1], np.float64)
# corner anchors of faces 1..6 = xi-, xi+, eta-, eta+, gamma-, gamma+
FACE_CORNERS = np.array([[0, 3, 7, 4], [1, 2, 6, 5], [0, 1, 5, 4], [3, 2, 6, 7], [0, 1, 2, 3], [4, 5, 6, 7]])


# ----------------------------------------------------------------------------- reading
def _ints(line):
    return [int(v) for v in line.split()]


def read_external_mesh(mesh_dir: str) -> dict:
    """Nodes (nnod, 3), elements (nspec, 8) 0-based node indices, material id per
    element, material table {id: dict(domain, rho, vp, vs, Qkappa, Qmu)} and the
    face lists {name: (nfaces, 5) [element, 4 nodes] 0-based}."""
    def path(n):
        return os.path.join(mesh_dir, n)
    with open(path("nodes_coords_file")) as f:
        nn = int(f.readline().split()[0])
        raw = np.loadtxt(f, max_rows=nn)
    ids = raw[:, 0].astype(np.int64)
    nodes = np.zeros((int(ids.max()), 3))
    nodes[ids - 1] = raw[:, 1:4]
    with open(path("mesh_file")) as f:
        ne = int(f.readline().split()[0])
        m = np.loadtxt(f, dtype=np.int64, max_rows=ne)
    order = np.argsort(m[:, 0])
    elems = m[order, 1:9] - 1
    mat = np.loadtxt(path("materials_file"), dtype=np.int64)
    mat_id = np.zeros(ne, np.int64)
    mat_id[mat[:, 0] - 1] = mat[:, 1]
    materials = {}
    for line in open(path("nummaterial_velocity_file")):
        t = line.split()
        if len(t) < 7 or t[0].startswith("!") or t[0].startswith("#"):
            continue
        try:
            dom, mid = int(t[0]), int(t[1])
            rho, vp, vs, qk, qmu = (float(v.replace("d", "e")) for v in t[2:7])
        except ValueError:
            continue
        materials[mid] = dict(domain=dom, rho=rho, vp=vp, vs=vs, Qkappa=qk, Qmu=qmu)
    faces = {}
    for name in ("absorbing_surface_file_xmin", "absorbing_surface_file_xmax", "absorbing_surface_file_ymin",
                 "absorbing_surface_file_ymax", "absorbing_surface_file_bottom",
                 "free_or_absorbing_surface_file_zmax"):
        if not os.path.exists(path(name)):
            continue
        with open(path(name)) as f:
            n = int(f.readline().split()[0])
            a = np.loadtxt(f, dtype=np.int64, max_rows=n).reshape(-1, 5) if n else np.zeros((0, 5), np.int64)
        faces[name] = a - 1
    return dict(nodes=nodes, elems=elems, mat_id=mat_id, materials=materials, faces=faces)


def read_par_file(path: str) -> dict:
    """The Par_file keys this path uses (NSTEP, DT, STACEY_ABSORBING_CONDITIONS, ...)."""
    out = {}
    for line in open(path):
        line = line.split("#")[0].strip()
        if "=" not in line:
            continue
        k, v = (s.strip() for s in line.split("=", 1))
        out[k] = v
    def flag(k):
        return out.get(k, ".false.").lower().startswith(".t")
    return dict(NSTEP=int(out["NSTEP"]), DT=float(out["DT"].replace("d", "e")),
                STACEY_ABSORBING_CONDITIONS=flag("STACEY_ABSORBING_CONDITIONS"),
                USE_FORCE_POINT_SOURCE=flag("USE_FORCE_POINT_SOURCE"),
                USE_RICKER_TIME_FUNCTION=flag("USE_RICKER_TIME_FUNCTION"),
                ATTENUATION=flag("ATTENUATION"), NGNOD=int(out.get("NGNOD", "8")),
                SAVE_SEISMOGRAMS_PRESSURE=flag("SAVE_SEISMOGRAMS_PRESSURE"))


def read_cmtsolution(path: str) -> dict:
    """CMTSOLUTION of a Cartesian run: x = longorUTM, y = latorUTM, z = -depth (km -> m);
    moment tensor dyne.cm (r, t, p) -> N.m (x, y, z) (get_cmt.f90:424,
    locate_source.F90:210-223)."""
    v = {}
    for line in open(path).readlines()[1:]:
        if ":" in line:
            k, val = line.split(":", 1)
            try:
                v[k.strip()] = float(val.split()[0].replace("d", "e").replace("D", "e"))
            except (ValueError, IndexError):
                pass
    s = 1e-7
    M = [v["Mpp"] * s, v["Mtt"] * s, v["Mrr"] * s, -v["Mtp"] * s, v["Mrp"] * s, -v["Mrt"] * s]
    return dict(type="cmt", x=v["longorUTM"], y=v["latorUTM"], z=-1000.0 * v["depth"], M=M,
                hdur=v["half duration"], tshift=v["time shift"])


def read_stations(path: str):
    """STATIONS lines "name network lat lon elevation burial": x = lon, y = lat,
    z = -burial (flat top surface at z = 0)."""
    out = []
    for line in open(path):
        t = line.split()
        if len(t) >= 6:
            out.append((t[0], t[1], float(t[3]), float(t[2]), -float(t[5])))
    return out


# ----------------------------------------------------------------------------- geometry
def shape8(xi, eta, ga):
    """Trilinear shape functions of the 8 anchors and their derivatives
    (get_shape3D.f90, NGNOD = 8): sh (..., 8), dsh (..., 3, 8)."""
    xi, eta, ga = (np.asarray(v, np.float64)[..., None] for v in (xi, eta, ga))
    fx, fy, fz = 1.0 + ANCHOR_XI * xi, 1.0 + ANCHOR_ETA * eta, 1.0 + ANCHOR_GA * ga
    sh = 0.125 * fx * fy * fz
    dsh = np.stack([0.125 * ANCHOR_XI * fy * fz, 0.125 * fx * ANCHOR_ETA * fz, 0.125 * fx * fy * ANCHOR_GA], axis=-2)
    return sh, dsh


def _gll_grid():
    """(125,) xi, eta, gamma of the GLL points, i fastest."""
    k, j, i = np.meshgrid(np.arange(NGLL), np.arange(NGLL), np.arange(NGLL), indexing="ij")
    return GLL[i.reshape(-1)], GLL[j.reshape(-1)], GLL[k.reshape(-1)]


_SH, _DSH = shape8(*_gll_grid())          # (125, 8), (125, 3, 8)


def gll_points(anchors: np.ndarray) -> np.ndarray:
    """(nspec, 125, 3) coordinates of every element's GLL points (calc_coords,
    calc_jacobian.f90:148-178) from anchors (nspec, 8, 3)."""
    return np.einsum("pa,ead->epd", _SH, anchors, optimize=True)


def get_global(xyz: np.ndarray, xtol: float):
    """Global numbering of points (npt, 3): sort x, split where consecutive values
    differ by more than xtol, sort y inside each segment, split, then z
    (sort_array_coordinates.f90:30-128); number the final segments, then renumber
    by first appearance (get_global.f90:80-141).  Returns (ibool 1-based int32, nglob)."""
    n = len(xyz)
    order = np.arange(n)
    seg = np.zeros(n, np.int64)                # segment id of each sorted slot
    for d in range(3):
        key = xyz[order, d]
        o = np.lexsort((key, seg))              # by segment, then coordinate
        order, key, seg = order[o], key[o], seg[o]
        brk = np.empty(n, bool)
        brk[0] = True
        brk[1:] = (seg[1:] != seg[:-1]) | (np.abs(np.diff(key)) > xtol)
        seg = np.cumsum(brk) - 1
    glob = np.empty(n, np.int64)
    glob[order] = seg
    nglob = int(seg[-1]) + 1 if n else 0
    first = np.full(nglob, n, np.int64)
    np.minimum.at(first, glob, np.arange(n))
    rank = np.empty(nglob, np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(nglob)
    return (rank[glob] + 1).astype(np.int32), nglob


def jacobian_metric(anchors: np.ndarray, pts=None):
    """Metric terms and Jacobian (calc_jacobian.f90:28-142) at the GLL points of
    anchors (nspec, 8, 3), in float64: dict of xix .. gammaz, jacobian (nspec, 125).
    The Jacobian is re-evaluated as the inverse determinant of the metric, as the
    reference stores it."""
    dsh = _DSH if pts is None else pts
    J = np.einsum("pra,ead->eprd", dsh, anchors, optimize=True)   # J[e,p,r,d] = d x_d / d xi_r
    xxi, yxi, zxi = J[..., 0, 0], J[..., 0, 1], J[..., 0, 2]
    xeta, yeta, zeta = J[..., 1, 0], J[..., 1, 1], J[..., 1, 2]
    xga, yga, zga = J[..., 2, 0], J[..., 2, 1], J[..., 2, 2]
    jac = xxi * (yeta * zga - yga * zeta) - xeta * (yxi * zga - yga * zxi) + xga * (yxi * zeta - yeta * zxi)
    m = dict(xix=(yeta * zga - yga * zeta) / jac, xiy=(xga * zeta - xeta * zga) / jac,
             xiz=(xeta * yga - xga * yeta) / jac, etax=(yga * zxi - yxi * zga) / jac,
             etay=(xxi * zga - xga * zxi) / jac, etaz=(xga * yxi - xxi * yga) / jac,
             gammax=(yxi * zeta - yeta * zxi) / jac, gammay=(xeta * zxi - xxi * zeta) / jac,
             gammaz=(xxi * yeta - xeta * yxi) / jac)
    m["jacobian"] = 1.0 / (m["xix"] * (m["etay"] * m["gammaz"] - m["etaz"] * m["gammay"])
                           - m["xiy"] * (m["etax"] * m["gammaz"] - m["etaz"] * m["gammax"])
                           + m["xiz"] * (m["etax"] * m["gammay"] - m["etay"] * m["gammax"]))
    return m


METRIC_NAMES = ["xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"]


def regularity(anchors: np.ndarray):
    """Regular-element rule of check_element_regularity (calc_jacobian.f90:184-360):
    an element is regular when its single-precision anchors form an axis-aligned
    cube (x, y, z of the corner groups equal to within 2^-23, edges 1-2, 1-4, 1-5 of
    equal length to 1e-5) whose metric at the first GLL point is diagonal with
    xix = etay = gammaz, and its edge matches the first regular element's cube.
    Returns (irregular_element_number (nspec,) int32 1-based or 0, xix_regular,
    jacobian_regular)."""
    nspec = len(anchors)
    a32 = anchors.astype(np.float32)
    x, y, z = a32[..., 0], a32[..., 1], a32[..., 2]

    def eq(u, v):
        return np.abs(u - v) <= np.float32(1.1920929e-7)

    box = (eq(x[:, 0], x[:, 3]) & eq(x[:, 0], x[:, 4]) & eq(x[:, 0], x[:, 7]) & eq(x[:, 1], x[:, 2])
           & eq(x[:, 1], x[:, 5]) & eq(x[:, 1], x[:, 6]) & eq(y[:, 0], y[:, 1]) & eq(y[:, 0], y[:, 4])
           & eq(y[:, 0], y[:, 5]) & eq(y[:, 2], y[:, 3]) & eq(y[:, 2], y[:, 6]) & eq(y[:, 2], y[:, 7])
           & eq(z[:, 0], z[:, 1]) & eq(z[:, 0], z[:, 2]) & eq(z[:, 0], z[:, 3]) & eq(z[:, 4], z[:, 5])
           & eq(z[:, 4], z[:, 6]) & eq(z[:, 4], z[:, 7]))

    def edge2(b):
        d = (a32[:, b] - a32[:, 0]).astype(np.float64)
        return (d * d).sum(axis=1)

    d1, d2, d3 = edge2(1), edge2(4), edge2(3)
    cand = box & (np.abs(d2 - d1) < 1e-5 * d1) & (np.abs(d3 - d1) < 1e-5 * d1)
    idx = np.nonzero(cand)[0]
    if len(idx):
        m0 = jacobian_metric(a32[idx].astype(np.float64), _DSH[:1])
        g = {k: v[:, 0].astype(np.float32).astype(np.float64) for k, v in m0.items()}
        tz = 1e-25
        diag = ((np.abs(g["xix"] - g["etay"]) < tz) & (np.abs(g["xix"] - g["gammaz"]) < tz)
                & (np.abs(g["xiy"]) < tz) & (np.abs(g["xiz"]) < tz) & (np.abs(g["etax"]) < tz)
                & (np.abs(g["etaz"]) < tz) & (np.abs(g["gammax"]) < tz) & (np.abs(g["gammay"]) < tz))
        cand[idx] = diag
    regular = np.zeros(nspec, bool)
    xr = jr = 0.0
    idx = np.nonzero(cand)[0]
    if len(idx):
        first = idx[0]
        cube = d1[first]
        regular = cand & (np.abs(d1 - cube) <= 1e-5 * cube)
        regular[:first] = False
        m = jacobian_metric(anchors[first:first + 1], _DSH[:1])
        xr = float(np.float32(m["xix"][0, 0]))
        jr = float(np.float32(m["jacobian"][0, 0]))
    irr = np.where(regular, 0, np.cumsum(~regular)).astype(np.int32)
    return irr, xr, jr


# ----------------------------------------------------------------------------- faces
def face_gll_ijk(iface: int) -> np.ndarray:
    """(25, 3) 0-based (i, j, k) of face iface (1..6) in face GLL order, first face
    index fastest (get_element_face_gll_indices, get_element_face.f90:169-279)."""
    a = np.arange(NGLL)
    A, Bb = np.meshgrid(a, a, indexing="xy")
    A, Bb = A.reshape(-1), Bb.reshape(-1)
    lo_hi = 0 if iface % 2 == 1 else NGLL - 1
    c = np.full(25, lo_hi)
    if iface in (1, 2):
        return np.stack([c, A, Bb], axis=-1)
    if iface in (3, 4):
        return np.stack([A, c, Bb], axis=-1)
    return np.stack([A, Bb, c], axis=-1)


FACE_IJK = np.stack([face_gll_ijk(f) for f in range(1, 7)])           # (6, 25, 3)
FACE_PT = FACE_IJK[..., 0] + NGLL * FACE_IJK[..., 1] + NGLL * NGLL * FACE_IJK[..., 2]  # (6, 25)


def face_ids(elems: np.ndarray, recs: np.ndarray) -> np.ndarray:
    """Face number 1..6 of each face record (nf, 5) = [element, 4 nodes] (0-based):
    the element face whose four corner anchors are those nodes (get_element_face_id,
    which matches the corners by coordinates; node ids are the same test on a
    conforming mesh).  Raises if a record names no face of its element."""
    if not len(recs):
        return np.zeros(0, np.int64)
    corners = np.sort(elems[recs[:, 0]][:, FACE_CORNERS], axis=-1)     # (nf, 6, 4)
    want = np.sort(recs[:, 1:5], axis=-1)[:, None, :]
    hit = (corners == want).all(axis=-1)
    if not hit.any(axis=1).all():
        bad = int(np.nonzero(~hit.any(axis=1))[0][0])
        raise ValueError(f"face record {bad} (element {int(recs[bad, 0]) + 1}) matches no face of its element")
    return np.argmax(hit, axis=1) + 1


def face_geometry(anchors: np.ndarray, iface: np.ndarray):
    """Weighted 2-D Jacobian (nf, 25) and outward unit normal (nf, 25, 3) of faces
    iface (nf,) of elements with anchors (nf, 8, 3): bilinear map of the four face
    corners, normal e_a x e_b oriented away from the element centre
    (get_jacobian_boundary_face, get_element_face_normal)."""
    nf = len(iface)
    if nf == 0:
        return np.zeros((0, 25)), np.zeros((0, 25, 3))
    cx = anchors[np.arange(nf)[:, None], FACE_CORNERS[iface - 1]]     # (nf, 4, 3)
    a = np.arange(NGLL)
    A, Bb = np.meshgrid(a, a, indexing="xy")
    s, t = GLL[A.reshape(-1)], GLL[Bb.reshape(-1)]                     # (25,)
    dsa = np.stack([-0.25 * (1 - t), 0.25 * (1 - t), 0.25 * (1 + t), -0.25 * (1 + t)], axis=-1)
    dsb = np.stack([-0.25 * (1 - s), -0.25 * (1 + s), 0.25 * (1 + s), 0.25 * (1 - s)], axis=-1)
    sh = np.stack([0.25 * (1 - s) * (1 - t), 0.25 * (1 + s) * (1 - t), 0.25 * (1 + s) * (1 + t),
                   0.25 * (1 - s) * (1 + t)], axis=-1)
    e1 = np.einsum("gc,fcd->fgd", dsa, cx)
    e2 = np.einsum("gc,fcd->fgd", dsb, cx)
    px = np.einsum("gc,fcd->fgd", sh, cx)
    n = np.cross(e1, e2)
    jac2 = np.sqrt((n * n).sum(axis=-1))
    n = n / jac2[..., None]
    ctr = anchors.mean(axis=1)[:, None, :]
    flip = ((n * (px - ctr)).sum(axis=-1) < 0)
    n = np.where(flip[..., None], -n, n)
    w = (WGLL[A.reshape(-1)] * WGLL[Bb.reshape(-1)])[None, :]
    return jac2 * w, n


def _face_block(ispec0: np.ndarray, iface: np.ndarray, anchors: np.ndarray, dtype):
    """Reference face arrays for faces (0-based elements): ispec (1-based), ijk
    (1-based, flat), jacobian2Dw (flat), normal (flat)."""
    jw, n = face_geometry(anchors[ispec0], iface)
    ijk = FACE_IJK[iface - 1] + 1 if len(iface) else np.zeros((0, 25, 3), np.int64)
    return ((ispec0 + 1).astype(np.int32), ijk.astype(np.int32).reshape(-1), jw.astype(dtype).reshape(-1),
            n.astype(dtype).reshape(-1))


def coupling_faces(elems_ib: np.ndarray, is_acoustic: np.ndarray, nglob: int):
    """Fluid-solid coupling faces seen from the fluid side (get_coupling_surfaces.f90:
    270-380): a face of an acoustic element whose four corners and centre point are
    points of elastic elements, each face once (first occurrence in element, face
    order).  elems_ib: (nspec, 125) 0-based global numbers.  Returns (ispec0, iface)."""
    isac = np.asarray(is_acoustic, bool)
    if not isac.any() or isac.all():
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    on_solid = np.zeros(nglob, bool)
    on_solid[elems_ib[~isac].reshape(-1)] = True
    # corners by face, in the element's own point numbering i + 5 j + 25 k
    corner_pt = np.array([FACE_PT[f][[0, 4, 24, 20]] for f in range(6)])
    mid_pt = FACE_PT[:, 12]
    ac = np.nonzero(isac)[0]
    ib = elems_ib[ac]
    ok = on_solid[ib[:, corner_pt]].all(axis=-1) & on_solid[ib[:, mid_pt]]      # (nac, 6)
    e_idx, f_idx = np.nonzero(ok)
    mids = ib[e_idx, mid_pt[f_idx]]
    _, first = np.unique(mids, return_index=True)
    keep = np.sort(first)
    return ac[e_idx[keep]], f_idx[keep] + 1


# ----------------------------------------------------------------------------- location
def element_neighbours(ibool: np.ndarray, nspec: int):
    """CSR (indptr, indices) of the elements searched around an element when a
    point falls on its boundary or outside it: elements sharing a corner with it
    and their corner neighbours, in element order, itself excluded
    (setup_mesh_adjacency.f90 also adds neighbours of neighbours)."""
    from scipy import sparse
    ib = np.asarray(ibool).reshape(nspec, NGLL3) - 1
    c = ib[:, [0, 4, 20, 24, 100, 104, 120, 124]].reshape(-1)
    A = sparse.csr_matrix((np.ones(8 * nspec, np.int32), (np.repeat(np.arange(nspec), 8), c)),
                          shape=(nspec, int(ib.max()) + 1))
    r1 = (A @ A.T).astype(bool).astype(np.int32)
    r2 = (r1 @ r1).tocsr()
    r2.setdiag(0)
    r2.eliminate_zeros()
    r2.sort_indices()
    return r2.indptr, r2.indices


def outer_surface_points(ibool: np.ndarray, nspec: int) -> np.ndarray:
    """(nspec, 125) bool: GLL points on a face that belongs to one element only,
    the outer surface of the mesh (iglob_is_surface_external_mesh)."""
    ib = np.asarray(ibool).reshape(nspec, NGLL3).astype(np.int64) - 1
    corners = np.sort(ib[:, FACE_PT[:, [0, 4, 24, 20]]], axis=-1).reshape(-1, 4)      # (nspec*6, 4)
    _, inv, cnt = np.unique(corners, axis=0, return_inverse=True, return_counts=True)
    single = (cnt[inv.reshape(-1)] == 1).reshape(nspec, 6)
    on = np.zeros(int(ib.max()) + 1, bool)
    e, f = np.nonzero(single)
    on[ib[e[:, None], FACE_PT[f]]] = True
    return on[ib]


class Locator:
    """Point location in a general hexahedral mesh (locate_point_in_mesh,
    locate_point.f90:32-416): the closest GLL point over all elements
    (single-precision coordinates; the first strictly closer point in element,
    k, j, i order wins), Newton iterations on (xi, eta, gamma) in that element
    (find_local_coordinates, :422-624); unless the result lies strictly inside the
    element (or above the top of an outer-surface point), up to 3 rounds of
    find_best_neighbor (:630-804) over the element's neighbours: a neighbour is
    taken when its location is closer by more than 1e-15 (the reference's tie
    threshold), when it puts an outside point inside, or when it moves a point
    from a fluid to a solid element at their interface."""

    def __init__(self, anchors: np.ndarray, gll_xyz: np.ndarray, ibool=None, is_acoustic=None):
        self.anchors = anchors
        self.g32 = gll_xyz.astype(np.float32).astype(np.float64)         # (nspec, 125, 3)
        self.lo = anchors.min(axis=1)
        self.hi = anchors.max(axis=1)
        self.ibool = ibool
        self.isac = None if is_acoustic is None else np.asarray(is_acoustic, bool)
        self._nb = self._surf = None

    def closest(self, xt):
        # elements that can hold the closest point: bounding-box distance below the
        # distance to the nearest anchor (anchors are GLL points)
        da = ((self.g32[:, [0, 4, 20, 24, 100, 104, 120, 124]] - xt) ** 2).sum(-1).min()
        gap = np.maximum(0.0, np.maximum(self.lo - xt, xt - self.hi))
        slack = 1e-6 * (1.0 + np.abs(xt).max()) ** 2
        cand = np.nonzero((gap * gap).sum(-1) <= da * (1 + 1e-6) + slack)[0]
        d = ((self.g32[cand] - xt) ** 2).sum(-1)
        flat = int(np.argmin(d.reshape(-1)))
        return int(cand[flat // NGLL3]), flat % NGLL3

    def newton(self, e, xt, p0):
        """(xi, eta, gamma, squared distance) after find_local_coordinates."""
        an = self.anchors[e]
        xi, eta, ga = GLL[p0 % 5], GLL[(p0 // 5) % 5], GLL[p0 // 25]
        dmin2 = 1e30
        for _ in range(5):
            sh, dsh = shape8(xi, eta, ga)
            dx = xt - sh @ an
            d2 = float(dx @ dx)
            if not d2 < dmin2:
                break
            dmin2 = d2
            step = np.linalg.solve((dsh @ an).T, dx)          # (dsh @ an)[r, d] = d x_d / d xi_r
            if float(step @ step) > 1.0:
                step = step * 0.33333333333
            xi, eta, ga = (float(np.clip(v + s, -1.01, 1.01)) for v, s in zip((xi, eta, ga), step))
        sh, _ = shape8(xi, eta, ga)
        dx = xt - sh @ an
        return xi, eta, ga, float(dx @ dx)

    def _neighbours(self, e):
        if self._nb is None:
            self._nb = element_neighbours(self.ibool, len(self.anchors))
        ptr, idx = self._nb
        return idx[ptr[e]:ptr[e + 1]]

    def _on_surface(self, e, p):
        if self.ibool is None:
            return False
        if self._surf is None:
            self._surf = outer_surface_points(self.ibool, len(self.anchors))
        return bool(self._surf[e, p])

    def __call__(self, x, y, z, octant=None):
        """(ispec 1-based, xi, eta, gamma) of target (x, y, z).  ``octant`` (3 signs)
        places a target on element boundaries in the first element (bounding box
        holding it) whose centre lies on that side of it along every axis."""
        xt = np.array([x, y, z], np.float64)
        if octant is not None:
            inside = np.nonzero(((self.lo <= xt) & (xt <= self.hi)).all(axis=1))[0]
            ctr = self.anchors[inside].mean(axis=1)
            ok = inside[(np.sign(ctr - xt) == np.sign(np.asarray(octant, np.float64))).all(axis=1)]
            if len(ok):
                e = int(ok[0])
                d = ((self.g32[e] - xt) ** 2).sum(-1)
                xi, eta, ga, _ = self.newton(e, xt, int(np.argmin(d)))
                return e + 1, xi, eta, ga
        e, p = self.closest(xt)
        xi, eta, ga, d2 = self.newton(e, xt, p)

        def out(a, b, c):
            return abs(a) > 1.0 or abs(b) > 1.0 or abs(c) > 1.0

        search = not (abs(xi) < 1.0 and abs(eta) < 1.0 and abs(ga) < 1.0)
        if search and ga > 1.0 and self._on_surface(e, p):
            search = False
        if search and self.ibool is not None:
            for _ in range(3):
                e0 = e
                for n in self._neighbours(e0):
                    dg = ((self.g32[n] - xt) ** 2).sum(-1)
                    nxi, neta, nga, nd2 = self.newton(int(n), xt, int(np.argmin(dg)))
                    better = False
                    if nd2 < 1e-10 and not out(nxi, neta, nga):
                        if out(xi, eta, ga):
                            better = True
                        if self.isac is not None and self.isac[e] and not self.isac[n]:
                            better = True
                    # improvements below the reference's 1e-15 tie threshold count as
                    # ties (the earlier element stays): a point on an element boundary
                    # does not move with rounding noise
                    if nd2 < d2 - 1e-15:
                        better = True
                    if better:
                        e, xi, eta, ga, d2 = int(n), nxi, neta, nga, nd2
                if e == e0 or not out(xi, eta, ga):
                    break
        return e + 1, xi, eta, ga


# ----------------------------------------------------------------------------- database
ABSORBING_FILES = [("xmin", "absorbing_surface_file_xmin"), ("xmax", "absorbing_surface_file_xmax"),
                   ("ymin", "absorbing_surface_file_ymin"), ("ymax", "absorbing_surface_file_ymax"),
                   ("bottom", "absorbing_surface_file_bottom"), ("top", "free_or_absorbing_surface_file_zmax")]
_EDGES = np.array([[0, 4], [20, 24], [100, 104], [120, 124], [0, 20], [4, 24], [100, 120], [104, 124],
                   [0, 100], [4, 104], [20, 120], [24, 124]])


def element_size_max(xyz: np.ndarray) -> np.ndarray:
    """Longest of the 12 edges of every element, from single-precision corner GLL
    points (get_elem_minmaxsize, check_mesh_resolution.f90:1474-1575)."""
    c = xyz.astype(np.float32)
    d = c[:, _EDGES[:, 0]] - c[:, _EDGES[:, 1]]
    return np.sqrt((d * d).sum(axis=-1, dtype=np.float32).max(axis=1)).astype(np.float32)


def material_table(mesh: dict):
    """(layers, elem_layer): the material list in id order and each element's index
    into it, the form the attenuation set-up takes."""
    ids = sorted(mesh["materials"])
    pos = {m: i for i, m in enumerate(ids)}
    layers = [dict(mesh["materials"][m]) for m in ids]
    elem_layer = np.array([pos[int(m)] for m in mesh["mat_id"]], np.int32)
    return layers, elem_layer


def build_database(mesh: dict, cfg: dict, dtype=np.float32, chunk: int = 1 << 15) -> dict:
    """Solver arrays (reference layouts, 1-based indices) of a general hexahedral
    mesh as read by :func:`read_external_mesh` (or built by :func:`block_mesh`).
    cfg: dt, nstep, sources, receivers, stacey (bool), absorbing (names of the
    face lists that absorb; "top" = STACEY_INSTEAD_OF_FREE_SURFACE), attenuation."""
    from . import meshgen
    anchors = mesh["nodes"][mesh["elems"]]
    nspec = len(anchors)
    xyz = gll_points(anchors)
    span = float(mesh["nodes"][:, 0].max() - mesh["nodes"][:, 0].min())
    ibool, nglob = get_global(xyz.reshape(-1, 3), 1e-10 * abs(span))
    db = dict(nspec=nspec, nglob=nglob, ibool=ibool)
    irr, xr, jr = regularity(anchors)
    nirr = int(irr.max()) if nspec else 0
    db.update(irregular_element_number=irr, nspec_irregular=nirr, xix_regular=xr, jacobian_regular=jr)
    ne = max(nirr, 1)
    for n in METRIC_NAMES:
        db[n] = np.zeros((ne, NGLL3), dtype)
    el = np.nonzero(irr)[0]
    for s in range(0, len(el), chunk):
        e = el[s:s + chunk]
        m = jacobian_metric(anchors[e])
        for n in METRIC_NAMES:
            db[n][irr[e] - 1] = m[n].astype(dtype)
    for n in METRIC_NAMES:
        db[n] = db[n].reshape(-1)
    # materials (get_model.F90: domain 1 acoustic, 2 elastic)
    layers, elem_layer = material_table(mesh)
    rho_l = np.array([m["rho"] for m in layers], np.float32)
    vp_l = np.array([m["vp"] for m in layers], np.float32)
    vs_l = np.array([0.0 if m["domain"] == 1 else m["vs"] for m in layers], np.float32)
    r, p, s_ = (np.repeat(a[elem_layer], NGLL3).astype(dtype) for a in (rho_l, vp_l, vs_l))
    db["ispec_is_acoustic"] = np.array([layers[i]["domain"] == 1 for i in elem_layer], np.int32)
    db["rhostore"] = r
    db["kappastore"] = r * (p * p - dtype(4.0 / 3.0) * s_ * s_)
    db["mustore"] = r * s_ * s_
    db["rho_vp"] = r * p
    db["rho_vs"] = r * s_
    db["elem_size_max"] = element_size_max(xyz)
    # absorbing faces in the order xmin, xmax, ymin, ymax, bottom[, top]
    want = cfg.get("absorbing", ["xmin", "xmax", "ymin", "ymax", "bottom"]) if cfg.get("stacey", True) else []
    ispec0, iface = [], []
    for name, fname in ABSORBING_FILES:
        recs = mesh["faces"].get(fname)
        if name in want and recs is not None and len(recs):
            ispec0.append(recs[:, 0])
            iface.append(face_ids(mesh["elems"], recs))
    i0 = np.concatenate(ispec0) if ispec0 else np.zeros(0, np.int64)
    fi = np.concatenate(iface) if iface else np.zeros(0, np.int64)
    (db["abs_boundary_ispec"], db["abs_boundary_ijk"], db["abs_boundary_jacobian2Dw"],
     db["abs_boundary_normal"]) = _face_block(i0, fi, anchors, dtype)
    db["num_abs_boundary_faces"] = len(i0)
    db["stacey"] = int(len(i0) > 0)
    # fluid-solid coupling and free surface
    ib0 = ibool.reshape(nspec, NGLL3).astype(np.int64) - 1
    ce, cf = coupling_faces(ib0, db["ispec_is_acoustic"], nglob)
    (db["coupling_ac_el_ispec"], db["coupling_ac_el_ijk"], db["coupling_ac_el_jacobian2Dw"],
     db["coupling_ac_el_normal"]) = _face_block(ce, cf, anchors, dtype)
    db["num_coupling_ac_el_faces"] = len(ce)
    top = mesh["faces"].get("free_or_absorbing_surface_file_zmax")
    if top is None or "top" in want:
        top = np.zeros((0, 5), np.int64)
    ft = face_ids(mesh["elems"], top)
    db["num_free_surface_faces"] = len(top)
    db["free_surface_ispec"] = (top[:, 0] + 1).astype(np.int32)
    db["free_surface_ijk"] = ((FACE_IJK[ft - 1] + 1).reshape(-1) if len(top) else np.zeros(0)).astype(np.int32)
    meshgen._mass(cfg, None, db, dtype)
    db.update(derivation_matrices())
    meshgen._sources_receivers(cfg, None, db, dtype,
                               locator=Locator(anchors, xyz, ibool, db["ispec_is_acoustic"]))
    db["attenuation"] = int(bool(cfg.get("attenuation", False)))
    if db["attenuation"]:
        from . import attenuation
        db.update(attenuation.setup(dict(cfg, layers=layers, elem_layer=elem_layer), db))
    return db


def block_mesh(cfg: dict) -> dict:
    """The layered block of a block configuration as an external mesh: nodes on
    the (x, y, zlev) grid, elements x fastest then y then z from the bottom, one
    material per layer, and the five absorbing face lists plus the top surface."""
    nx, ny = int(cfg["nx"]), int(cfg["ny"])
    zl = np.asarray(cfg["zlev"], np.float64)
    nz = len(zl) - 1
    xl = np.array([cfg["x0"] + (cfg["x1"] - cfg["x0"]) * e / nx for e in range(nx + 1)])
    yl = np.array([cfg["y0"] + (cfg["y1"] - cfg["y0"]) * e / ny for e in range(ny + 1)])
    Z, Y, X = np.meshgrid(zl, yl, xl, indexing="ij")
    nodes = np.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], axis=-1)

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    e = np.arange(nx * ny * nz)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    elems = np.stack([nid(ex + (ANCHOR_XI[a] > 0), ey + (ANCHOR_ETA[a] > 0), ez + (ANCHOR_GA[a] > 0))
                      for a in range(8)], axis=-1).astype(np.int64)
    layers = cfg["layers"]
    materials = {i + 1: dict(domain=1 if float(m["vs"]) == 0.0 else 2, rho=float(m["rho"]), vp=float(m["vp"]),
                             vs=float(m["vs"]), Qkappa=float(m.get("Qkappa", 9999.0)), Qmu=float(m.get("Qmu", 9999.0)))
                 for i, m in enumerate(layers)}
    mat_id = np.asarray(cfg["elem_layer"], np.int64) + 1
    sel = {"absorbing_surface_file_xmin": (ex == 0, 1), "absorbing_surface_file_xmax": (ex == nx - 1, 2),
           "absorbing_surface_file_ymin": (ey == 0, 3), "absorbing_surface_file_ymax": (ey == ny - 1, 4),
           "absorbing_surface_file_bottom": (ez == 0, 5), "free_or_absorbing_surface_file_zmax": (ez == nz - 1, 6)}
    faces = {}
    for name, (m, f) in sel.items():
        el = np.nonzero(m)[0]
        faces[name] = np.concatenate([el[:, None], elems[el][:, FACE_CORNERS[f - 1]]], axis=1)
    return dict(nodes=nodes, elems=elems, mat_id=mat_id, materials=materials, faces=faces)
