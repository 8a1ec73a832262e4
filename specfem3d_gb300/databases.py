"""The solver databases of xgenerate_databases: ``proc%06d_external_mesh.bin`` and
``proc%06d_attenuation.bin``, read and written.

Both are Fortran unformatted sequential files: every ``write(IOUT) x`` is one
record framed by its byte length as a 4-byte integer before and after (gfortran;
a record longer than 2^31 - 9 bytes is split into subrecords whose leading
marker is negative while more follow).  Records hold the arrays in Fortran
(column-major) order, which for the per-element arrays (5,5,5,NSPEC) is the
element-major, i-fastest order the solver here uses.  The record sequence is the
one of save_arrays_solver_mesh (generate_databases/save_arrays_solver.F90:100-
405), which read_mesh_databases (specfem3D/read_mesh_databases.F90:146-1200)
reads back, for acoustic and elastic domains (no poroelastic elements, C-PML,
ocean load or anisotropy); attenuation.bin follows prepare_attenuation.f90:95-
110.  ``CUSTOM_REAL`` is 4 bytes unless ``real_bytes=8`` (a reference built with
``--enable-double-precision``).
"""
from __future__ import annotations

import os
import struct

import numpy as np

NGLL3 = 125
N_SLS = 3
_MAX_SUB = 2 ** 31 - 9          # gfortran's largest subrecord


# ----------------------------------------------------------------------------- records
class RecordWriter:
    """Fortran unformatted sequential records."""

    def __init__(self, path: str):
        self.f = open(path, "wb")
        self.names = []     # the reference's variable names of the records written

    def write(self, *items, name: str = ""):
        """One record holding the given scalars / arrays back to back (name: the
        variable(s) the reference writes there)."""
        self.names.append(name)
        data = b"".join(np.ascontiguousarray(a).tobytes(order="C") if isinstance(a, np.ndarray) else a
                        for a in items)
        n, off = len(data), 0
        while True:
            chunk = data[off:off + _MAX_SUB]
            more = off + len(chunk) < n
            # gfortran subrecords: the leading marker is negative when another
            # subrecord follows, the trailing one when a subrecord preceded
            lead = -len(chunk) if more else len(chunk)
            tail = -len(chunk) if off > 0 else len(chunk)
            self.f.write(struct.pack("<i", lead) + chunk + struct.pack("<i", tail))
            off += len(chunk)
            if not more:
                break

    def close(self):
        self.f.close()


class RecordReader:
    def __init__(self, path: str):
        self.f = open(path, "rb")

    def raw(self) -> bytes:
        parts = []
        while True:
            head = self.f.read(4)
            if len(head) < 4:
                raise EOFError("unexpected end of the database file")
            lead = struct.unpack("<i", head)[0]
            n = abs(lead)
            parts.append(self.f.read(n))
            tail = struct.unpack("<i", self.f.read(4))[0]
            if abs(tail) != n:
                raise ValueError("corrupt record markers in the database file")
            if lead >= 0:
                return b"".join(parts)

    def array(self, dtype) -> np.ndarray:
        return np.frombuffer(self.raw(), dtype=dtype).copy()

    def ints(self, count=None):
        a = self.array(np.int32)
        if count is not None and len(a) != count:
            raise ValueError(f"expected {count} integers, the record holds {len(a)}")
        return a

    def int(self) -> int:
        return int(self.ints(1)[0])

    def check(self, marker: int):
        v = self.int()
        if v != marker:
            raise ValueError(f"database check value {v} where {marker} was expected")

    def close(self):
        self.f.close()


# ----------------------------------------------------------------------------- helpers
def global_coordinates(ibool: np.ndarray, xyz_elem: np.ndarray, nglob: int) -> np.ndarray:
    """(nglob, 3) coordinates of the global points from per-element GLL points
    (nspec, 125, 3) and ibool (1-based)."""
    out = np.zeros((nglob, 3))
    out[np.asarray(ibool, np.int64).reshape(-1) - 1] = xyz_elem.reshape(-1, 3)
    return out


def _face_of_ijk(ijk25: np.ndarray) -> int:
    """Face number 1..6 of a face given its 25 (i, j, k), 1-based."""
    for axis in range(3):
        v = np.unique(ijk25[:, axis])
        if len(v) == 1:
            return 2 * axis + (1 if v[0] == 1 else 2)
    raise ValueError("face points do not share a constant index")


def _logical(a) -> np.ndarray:
    return np.asarray(a, bool).astype(np.int32)


def _surface_and_neighbours(db):
    from .hexmesh import FACE_PT, element_neighbours
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    ib = np.asarray(db["ibool"]).reshape(nspec, NGLL3).astype(np.int64) - 1
    corners = np.sort(ib[:, FACE_PT[:, [0, 4, 24, 20]]], axis=-1).reshape(-1, 4)
    _, inv, cnt = np.unique(corners, axis=0, return_inverse=True, return_counts=True)
    single = (cnt[inv.reshape(-1)] == 1).reshape(nspec, 6)
    on = np.zeros(nglob, bool)
    e, f = np.nonzero(single)
    on[ib[e[:, None], FACE_PT[f]]] = True
    ptr, idx = element_neighbours(db["ibool"], nspec)
    return int(single.sum()), single.any(axis=1), on, ptr.astype(np.int32), (idx + 1).astype(np.int32)


# ----------------------------------------------------------------------------- writing
def write_external_mesh(path: str, db: dict, xyz_global: np.ndarray, stacey: bool | None = None,
                        real_bytes: int = 4, colors=None):
    """proc######_external_mesh.bin of one slice, in the record order of
    save_arrays_solver_mesh (save_arrays_solver.F90:100-405).  ``db`` is a
    database of this package (meshgen / hexmesh); with attenuation its relaxed
    moduli are written (the unrelaxed scaling goes to attenuation.bin).  Returns the
    reference's variable names of the records written, in order."""
    rt = np.float32 if real_bytes == 4 else np.float64
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    nirr = int(db["nspec_irregular"])
    isac = np.asarray(db.get("ispec_is_acoustic", np.zeros(nspec)), bool)
    acoustic, elastic = bool(isac.any()), bool((~isac).any())
    stacey = bool(db.get("stacey", 0)) if stacey is None else bool(stacey)
    R = lambda a: np.asarray(a, rt)                                  # noqa: E731
    I = lambda a: np.asarray(a, np.int32)                            # noqa: E731
    w = RecordWriter(path)
    for v, n in ((nspec, "nspec"), (nglob, "nglob"), (nirr, "nspec_irregular")):
        w.write(I([v]), name=n)
    w.write(I(db["ibool"]), name="ibool")
    for d in range(3):
        w.write(R(xyz_global[:, d]), name="xyz"[d] + "store_unique")
    w.write(I(db["irregular_element_number"]), name="irregular_element_number")
    w.write(R([db["xix_regular"]]), name="xix_regular")
    w.write(R([db["jacobian_regular"]]), name="jacobian_regular")
    for n in ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"):
        w.write(R(np.asarray(db[n])[:NGLL3 * nirr]), name=n + "store")
    w.write(R(db.get("kappastore_relaxed", db["kappastore"])), name="kappastore")
    w.write(R(db.get("mustore_relaxed", db["mustore"])), name="mustore")
    w.write(_logical(isac), name="ispec_is_acoustic")
    w.write(_logical(~isac), name="ispec_is_elastic")
    w.write(_logical(np.zeros(nspec, bool)), name="ispec_is_poroelastic")
    w.write(I([9999]), name="itest")
    if acoustic:
        w.write(R(db["rmass_acoustic_volume"]), name="rmass_acoustic")
    w.write(R(db["rhostore"]), name="rhostore")
    if elastic:
        w.write(R(db["rmass"]), name="rmass")
        w.write(R(db["rho_vp"]), name="rho_vp")
        w.write(R(db["rho_vs"]), name="rho_vs")
    nf = int(db["num_abs_boundary_faces"])
    w.write(I([nf]), name="num_abs_boundary_faces")
    if nf:
        w.write(I(db["abs_boundary_ispec"]), name="abs_boundary_ispec")
        w.write(I(db["abs_boundary_ijk"]), name="abs_boundary_ijk")
        w.write(R(db["abs_boundary_jacobian2Dw"]), name="abs_boundary_jacobian2Dw")
        w.write(R(db["abs_boundary_normal"]), name="abs_boundary_normal")
        if stacey:
            if elastic:
                for c in "xyz":
                    w.write(R(db["rmass" + c + "_stacey"]), name="rmass" + c)
            if acoustic:
                w.write(R(db.get("rmassz_acoustic", np.zeros(nglob))), name="rmassz_acoustic")
    w.write(I([9998]), name="itest")
    for n in ("nspec2D_xmin", "nspec2D_xmax", "nspec2D_ymin", "nspec2D_ymax", "NSPEC2D_BOTTOM", "NSPEC2D_TOP"):
        w.write(I([0]), name=n)              # the boundary element lists are not kept here
    nfs = int(db.get("num_free_surface_faces", 0))
    w.write(I([nfs]), name="num_free_surface_faces")
    if nfs:
        from .hexmesh import face_geometry
        ijk = I(db["free_surface_ijk"]).reshape(nfs, 25, 3)
        ispec = I(db["free_surface_ispec"])
        iface = np.array([_face_of_ijk(q) for q in ijk])
        ib = np.asarray(db["ibool"]).reshape(nspec, NGLL3).astype(np.int64) - 1
        corner = [0, 4, 24, 20, 100, 104, 124, 120]
        anchors = xyz_global[ib[ispec - 1][:, corner]]
        jw, nrm = face_geometry(anchors, iface)
        w.write(ispec, name="free_surface_ispec")
        w.write(ijk.reshape(-1), name="free_surface_ijk")
        w.write(R(jw.reshape(-1)), name="free_surface_jacobian2Dw")
        w.write(R(nrm.reshape(-1)), name="free_surface_normal")
    ncp = int(db.get("num_coupling_ac_el_faces", 0))
    w.write(I([ncp]), name="num_coupling_ac_el_faces")
    if ncp:
        w.write(I(db["coupling_ac_el_ispec"]), name="coupling_ac_el_ispec")
        w.write(I(db["coupling_ac_el_ijk"]), name="coupling_ac_el_ijk")
        w.write(R(db["coupling_ac_el_jacobian2Dw"]), name="coupling_ac_el_jacobian2Dw")
        w.write(R(db["coupling_ac_el_normal"]), name="coupling_ac_el_normal")
    w.write(I([0]), name="num_coupling_ac_po_faces")
    w.write(I([0]), name="num_coupling_el_po_faces")
    w.write(I([9997]), name="itest")
    nif = int(db.get("num_interfaces", 0))
    mxn = int(db.get("max_nibool_interfaces", 0)) if nif else 0
    w.write(I([nif]), name="num_interfaces_ext_mesh")
    w.write(I([mxn]), name="max_nibool_interfaces_ext_mesh")
    if nif:
        w.write(I(db.get("my_neighbors", db.get("neighbours", np.arange(nif)))), name="my_neighbors_ext_mesh")
        w.write(I(db["nibool_interfaces"]), name="nibool_interfaces_ext_mesh")
        w.write(I(db["ibool_interfaces"]), name="ibool_interfaces_ext_mesh_dummy")
    w.write(I([9996]), name="itest")
    outer = I(db.get("phase_outer", np.zeros(0)))
    inner_flag = np.ones(nspec, bool)
    inner_flag[outer - 1] = False
    w.write(_logical(inner_flag), name="ispec_is_inner")
    for flag, sel, dom in ((acoustic, isac, "acoustic"), (elastic, ~isac, "elastic")):
        if not flag:
            continue
        members = np.nonzero(sel)[0] + 1
        out_l = members[~inner_flag[members - 1]]
        in_l = members[inner_flag[members - 1]]
        w.write(I([len(in_l), len(out_l)]), name=f"nspec_inner_{dom},nspec_outer_{dom}")
        nph = max(len(in_l), len(out_l))
        w.write(I([nph]), name="num_phase_ispec_" + dom)
        if nph:
            ph = np.zeros((nph, 2), np.int32)
            ph[:len(out_l), 0] = out_l
            ph[:len(in_l), 1] = in_l
            w.write(ph.reshape(-1, order="F"), name="phase_ispec_inner_" + dom)
    if colors is not None:
        # USE_MESH_COLORING_GPU: colours of the outer, then the inner elements
        col = np.asarray(colors)
        for flag, sel, dom in ((acoustic, isac, "acoustic"), (elastic, ~isac, "elastic")):
            if not flag:
                continue
            co = np.unique(col[sel & ~inner_flag], return_counts=True)[1]
            ci = np.unique(col[sel & inner_flag], return_counts=True)[1]
            w.write(I([len(co), len(ci)]), name=f"num_colors_outer_{dom},num_colors_inner_{dom}")
            w.write(I(np.concatenate([co, ci])), name="num_elem_colors_" + dom)
    nsurf, isurf, gsurf, xadj, adj = _surface_and_neighbours(db)
    w.write(I([nsurf]), name="nfaces_surface")
    w.write(_logical(isurf), name="ispec_is_surface_external_mesh")
    w.write(_logical(gsurf), name="iglob_is_surface_external_mesh")
    w.write(I([len(adj)]), name="num_neighbors_all")
    w.write(xadj, name="neighbors_xadj")
    w.write(adj, name="neighbors_adjncy")
    w.write(I([9995]), name="itest")
    w.close()
    return w.names


def write_attenuation(path: str, db: dict, real_bytes: int = 4):
    """proc######_attenuation.bin: NSPEC, factor_common (N_SLS,5,5,5,NSPEC),
    scale_factor (5,5,5,NSPEC), factor_common_kappa, scale_factor_kappa
    (read by prepare_attenuation.f90:95-110)."""
    rt = np.float32 if real_bytes == 4 else np.float64
    nspec = int(db["nspec"])
    w = RecordWriter(path)
    w.write(np.asarray([nspec], np.int32))
    w.write(np.asarray(db["factor_common"], rt))
    w.write(np.asarray(db["scale_factor"], rt))
    w.write(np.asarray(db["factor_common_kappa"], rt))
    w.write(np.asarray(db["scale_factor_kappa"], rt))
    w.close()


# ----------------------------------------------------------------------------- reading
def read_external_mesh(path: str, stacey: bool, coloring: bool = False, real_bytes: int = 4) -> dict:
    """The records of proc######_external_mesh.bin as read_mesh_databases reads
    them (read_mesh_databases.F90:146-1200; the Par_file switches it needs:
    STACEY_ABSORBING_CONDITIONS, USE_MESH_COLORING_GPU).  Returns the raw arrays
    under the reference's names (1-based indices, masses not yet inverted)."""
    rt = np.float32 if real_bytes == 4 else np.float64
    r = RecordReader(path)
    d = {}
    d["nspec"], d["nglob"], d["nspec_irregular"] = r.int(), r.int(), r.int()
    nspec, nglob, nirr = d["nspec"], d["nglob"], d["nspec_irregular"]
    d["ibool"] = r.ints(NGLL3 * nspec)
    for n in ("xstore", "ystore", "zstore"):
        d[n] = r.array(rt)
    d["irregular_element_number"] = r.ints(nspec)
    d["xix_regular"] = float(r.array(rt)[0])
    d["jacobian_regular"] = float(r.array(rt)[0])
    for n in ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"):
        d[n] = r.array(rt)
        if len(d[n]) != NGLL3 * nirr:
            raise ValueError(f"{n}: {len(d[n])} values for {nirr} irregular elements")
    d["kappastore"], d["mustore"] = r.array(rt), r.array(rt)
    d["ispec_is_acoustic"] = r.ints(nspec) != 0
    d["ispec_is_elastic"] = r.ints(nspec) != 0
    d["ispec_is_poroelastic"] = r.ints(nspec) != 0
    if d["ispec_is_poroelastic"].any():
        raise ValueError("poroelastic elements are not supported")
    acoustic, elastic = bool(d["ispec_is_acoustic"].any()), bool(d["ispec_is_elastic"].any())
    r.check(9999)
    if acoustic:
        d["rmass_acoustic"] = r.array(rt)
    d["rhostore"] = r.array(rt)
    if elastic:
        d["rmass"], d["rho_vp"], d["rho_vs"] = r.array(rt), r.array(rt), r.array(rt)
    nf = r.int()
    d["num_abs_boundary_faces"] = nf
    if nf:
        d["abs_boundary_ispec"] = r.ints(nf)
        d["abs_boundary_ijk"] = r.ints(75 * nf)
        d["abs_boundary_jacobian2Dw"] = r.array(rt)
        d["abs_boundary_normal"] = r.array(rt)
        if stacey:
            if elastic:
                d["rmassx"], d["rmassy"], d["rmassz"] = r.array(rt), r.array(rt), r.array(rt)
            if acoustic:
                d["rmassz_acoustic"] = r.array(rt)
    r.check(9998)
    counts = [r.int() for _ in range(6)]
    for name, n in zip(("xmin", "xmax", "ymin", "ymax", "bottom", "top"), counts):
        d["ibelm_" + name] = r.ints(n) if n else np.zeros(0, np.int32)
    nfs = r.int()
    d["num_free_surface_faces"] = nfs
    if nfs:
        d["free_surface_ispec"] = r.ints(nfs)
        d["free_surface_ijk"] = r.ints(75 * nfs)
        d["free_surface_jacobian2Dw"] = r.array(rt)
        d["free_surface_normal"] = r.array(rt)
    ncp = r.int()
    d["num_coupling_ac_el_faces"] = ncp
    if ncp:
        d["coupling_ac_el_ispec"] = r.ints(ncp)
        d["coupling_ac_el_ijk"] = r.ints(75 * ncp)
        d["coupling_ac_el_jacobian2Dw"] = r.array(rt)
        d["coupling_ac_el_normal"] = r.array(rt)
    for _ in range(2):                      # acoustic-poroelastic, elastic-poroelastic faces
        if r.int():
            raise ValueError("poroelastic coupling faces are not supported")
    r.check(9997)
    nif, mxn = r.int(), r.int()
    d["num_interfaces"], d["max_nibool_interfaces"] = nif, mxn
    if nif:
        d["my_neighbors"] = r.ints(nif)
        d["nibool_interfaces"] = r.ints(nif)
        d["ibool_interfaces"] = r.ints(mxn * nif)
    r.check(9996)
    d["ispec_is_inner"] = r.ints(nspec) != 0
    for tag, flag in (("acoustic", acoustic), ("elastic", elastic)):
        if not flag:
            continue
        nin, nout = r.ints(2)
        nph = r.int()
        d[f"nspec_inner_{tag}"], d[f"nspec_outer_{tag}"] = int(nin), int(nout)
        d[f"phase_ispec_inner_{tag}"] = (r.ints(2 * nph).reshape(2, nph).T if nph
                                         else np.zeros((0, 2), np.int32))
    if coloring:
        for tag, flag in (("acoustic", acoustic), ("elastic", elastic)):
            if flag:
                d[f"num_colors_outer_{tag}"], d[f"num_colors_inner_{tag}"] = (int(v) for v in r.ints(2))
                d[f"num_elem_colors_{tag}"] = r.ints()
    d["nfaces_surface"] = r.int()
    d["ispec_is_surface_external_mesh"] = r.ints(nspec) != 0
    d["iglob_is_surface_external_mesh"] = r.ints(nglob) != 0
    nn = r.int()
    d["neighbors_xadj"] = r.ints(nspec + 1)
    d["neighbors_adjncy"] = r.ints(nn)
    r.check(9995)
    r.close()
    return d


def read_attenuation(path: str, nspec: int, real_bytes: int = 4) -> dict:
    rt = np.float32 if real_bytes == 4 else np.float64
    r = RecordReader(path)
    n = r.int()
    if n != nspec:
        raise ValueError(f"attenuation file array {n} should be {nspec}")
    out = {"factor_common": r.array(rt), "scale_factor": r.array(rt),
           "factor_common_kappa": r.array(rt), "scale_factor_kappa": r.array(rt)}
    r.close()
    for k, per in (("factor_common", N_SLS * NGLL3), ("scale_factor", NGLL3), ("factor_common_kappa", N_SLS * NGLL3),
                   ("scale_factor_kappa", NGLL3)):
        if len(out[k]) != per * nspec:
            raise ValueError(f"{k}: {len(out[k])} values, expected {per * nspec}")
    return out


# ----------------------------------------------------------------------------- to the solver
def solver_database(raw: dict, cfg: dict, attenuation_arrays: dict | None = None, dtype=np.float32) -> dict:
    """The arrays the time loop takes (this package's database dict) from what the
    files hold, finishing the set-up the way the solver does: the Stacey mass
    terms added and the masses inverted (prepare_timerun.F90:246-330), the
    moduli scaled to unrelaxed and the memory-variable constants computed
    (prepare_attenuation.f90:95-160), sources and receivers located from cfg
    (setup_sources_receivers.f90).  cfg: dt, nstep, sources, receivers, stacey."""
    from . import meshgen
    from .hexmesh import Locator, element_size_max
    nspec, nglob, nirr = int(raw["nspec"]), int(raw["nglob"]), int(raw["nspec_irregular"])
    db = dict(nspec=nspec, nglob=nglob, nspec_irregular=nirr)
    db["ibool"] = np.asarray(raw["ibool"], np.int32)
    db["irregular_element_number"] = np.asarray(raw["irregular_element_number"], np.int32)
    db["xix_regular"], db["jacobian_regular"] = raw["xix_regular"], raw["jacobian_regular"]
    ne = max(nirr, 1)
    for n in ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"):
        a = np.zeros(ne * NGLL3, dtype)
        a[:NGLL3 * nirr] = raw[n]
        db[n] = a
    isac = np.asarray(raw["ispec_is_acoustic"], bool)
    db["ispec_is_acoustic"] = isac.astype(np.int32)
    for n in ("rhostore", "kappastore", "mustore"):
        db[n] = np.asarray(raw[n], dtype)
    npt = NGLL3 * nspec
    db["rho_vp"] = np.asarray(raw.get("rho_vp", np.zeros(npt)), dtype)
    db["rho_vs"] = np.asarray(raw.get("rho_vs", np.zeros(npt)), dtype)
    stacey = bool(cfg.get("stacey", True)) and int(raw["num_abs_boundary_faces"]) > 0
    db["stacey"] = int(stacey)
    nf = int(raw["num_abs_boundary_faces"]) if stacey else 0
    db["num_abs_boundary_faces"] = nf
    for n, t in (("abs_boundary_ispec", np.int32), ("abs_boundary_ijk", np.int32),
                 ("abs_boundary_jacobian2Dw", dtype), ("abs_boundary_normal", dtype)):
        db[n] = np.asarray(raw[n], t) if nf else np.zeros(0, t)
    one = dtype(1)
    if "rmass" in raw:
        rm = np.asarray(raw["rmass"], dtype)
        db["rmass"] = rm
        for c in "xyz":
            m = rm + np.asarray(raw["rmass" + c], dtype) if stacey else rm.copy()
            m[m <= 0] = one
            db["rmass" + c] = (one / m).astype(dtype)
    if isac.any():
        m = np.asarray(raw["rmass_acoustic"], dtype)
        if stacey and "rmassz_acoustic" in raw:
            m = m + np.asarray(raw["rmassz_acoustic"], dtype)
        m = m.copy()
        m[m <= 0] = one
        db["rmass_acoustic"] = (one / m).astype(dtype)
    for n in ("free_surface", "coupling_ac_el"):
        k = "num_" + n + "_faces"
        db[k] = int(raw.get(k, 0))
    db["free_surface_ispec"] = np.asarray(raw.get("free_surface_ispec", np.zeros(0)), np.int32)
    db["free_surface_ijk"] = np.asarray(raw.get("free_surface_ijk", np.zeros(0)), np.int32)
    for n, t in (("ispec", np.int32), ("ijk", np.int32), ("jacobian2Dw", dtype), ("normal", dtype)):
        db["coupling_ac_el_" + n] = np.asarray(raw.get("coupling_ac_el_" + n, np.zeros(0)), t)
    if int(raw.get("num_interfaces", 0)):
        for n in ("num_interfaces", "max_nibool_interfaces", "nibool_interfaces", "ibool_interfaces", "my_neighbors"):
            db[n] = raw[n]
    ph = raw.get("phase_ispec_inner_elastic")
    if ph is not None and int(raw.get("nspec_outer_elastic", 0)):
        db["phase_outer"] = np.asarray(ph[:int(raw["nspec_outer_elastic"]), 0], np.int32)
    db.update(meshgen.derivation_matrices())
    # geometry of the element points, for the resolution and the point location
    xyz = np.stack([np.asarray(raw[n], np.float64) for n in ("xstore", "ystore", "zstore")], axis=1)
    ib0 = db["ibool"].reshape(nspec, NGLL3).astype(np.int64) - 1
    xyz_elem = xyz[ib0]
    db["elem_size_max"] = element_size_max(xyz_elem)
    db["attenuation"] = int(attenuation_arrays is not None)
    if attenuation_arrays is not None:
        from . import attenuation as ATT
        tau_sigma, f_c, minp, maxp = ATT.band(ATT.min_resolved_period(cfg, db))
        tau_f = tau_sigma.astype(np.float32)
        solid = np.repeat(~isac, NGLL3)
        db["mustore_relaxed"], db["kappastore_relaxed"] = db["mustore"], db["kappastore"]
        sf, sk = (np.asarray(attenuation_arrays[k], dtype) for k in ("scale_factor", "scale_factor_kappa"))
        db["mustore"] = np.where(solid, db["mustore"] * sf, db["mustore"]).astype(dtype)
        db["kappastore"] = np.where(solid, db["kappastore"] * sk, db["kappastore"]).astype(dtype)
        db["factor_common"] = np.asarray(attenuation_arrays["factor_common"], dtype)
        db["factor_common_kappa"] = np.asarray(attenuation_arrays["factor_common_kappa"], dtype)
        db["scale_factor"], db["scale_factor_kappa"] = sf, sk
        al, be, ga = ATT.memory_values(tau_f, cfg["dt"])
        db.update(alphaval=al, betaval=be, gammaval=ga, tau_sigma=tau_f, f_c_source=f_c)
    corner = [0, 4, 24, 20, 100, 104, 124, 120]
    loc = Locator(xyz_elem[:, corner], xyz_elem, db["ibool"], isac)
    meshgen._sources_receivers(cfg, None, db, dtype, locator=loc)
    return db
