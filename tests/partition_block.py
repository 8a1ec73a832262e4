"""Split a block database into slices along x with MPI interface lists (test
infrastructure: it plays the part of xdecompose_mesh + xgenerate_databases for
a structured block).

Each slice gets the elements whose x index falls in its range, a local point
numbering, the assembled (global) mass matrices restricted to its points, its
Stacey faces, sources and receivers, and, per neighbouring slice, the shared
points sorted by global index (so both sides of an interface order their
buffers the same way).  Elements touching an interface are the outer elements
(phase 1), the others inner (phase 2), as in the reference's
phase_ispec_inner_elastic.
"""
import numpy as np

NGLL3 = 125


def split_x(db: dict, cfg: dict, nparts: int):
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    nx = int(cfg["nx"])
    e = np.arange(nspec)
    part_of = ((e % nx) * nparts) // nx
    ib = db["ibool"].reshape(nspec, NGLL3)
    points = [np.unique(ib[part_of == p]) for p in range(nparts)]  # 1-based, sorted
    parts = []
    for p in range(nparts):
        el = np.nonzero(part_of == p)[0]
        gl = points[p]
        loc = np.zeros(nglob + 1, np.int64)
        loc[gl] = np.arange(1, len(gl) + 1)
        d = {k: v for k, v in db.items()}
        d["nspec"], d["nglob"] = len(el), len(gl)
        d["ibool"] = loc[ib[el]].astype(np.int32).reshape(-1)
        d["global_points"] = gl
        d["global_elements"] = el
        # irregular elements and their metric rows
        irr = db["irregular_element_number"][el]
        rows = irr[irr > 0] - 1
        newirr = np.zeros(len(el), np.int32)
        newirr[irr > 0] = np.arange(1, len(rows) + 1)
        d["irregular_element_number"] = newirr
        d["nspec_irregular"] = int(len(rows))
        for n in ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian"):
            a = db[n].reshape(-1, NGLL3)
            d[n] = (a[rows] if len(rows) else np.zeros((1, NGLL3), a.dtype)).reshape(-1)
        for n in ("kappastore", "mustore", "rhostore", "rho_vp", "rho_vs"):
            d[n] = db[n].reshape(nspec, NGLL3)[el].reshape(-1)
        d["ispec_is_acoustic"] = db["ispec_is_acoustic"][el]
        for n in ("factor_common", "factor_common_kappa"):
            if n in db:
                d[n] = db[n].reshape(nspec, -1)[el].reshape(-1)
        for n in ("rmass", "rmassx", "rmassy", "rmassz"):
            d[n] = db[n][gl - 1]
        # Stacey faces of the slice
        eloc = np.zeros(nspec + 1, np.int32)
        eloc[el + 1] = np.arange(1, len(el) + 1)
        f = np.nonzero(np.isin(db["abs_boundary_ispec"] - 1, el))[0]
        d["abs_boundary_ispec"] = eloc[db["abs_boundary_ispec"][f]]
        d["abs_boundary_ijk"] = db["abs_boundary_ijk"].reshape(-1, 75)[f].reshape(-1)
        d["abs_boundary_normal"] = db["abs_boundary_normal"].reshape(-1, 75)[f].reshape(-1)
        d["abs_boundary_jacobian2Dw"] = db["abs_boundary_jacobian2Dw"].reshape(-1, 25)[f].reshape(-1)
        d["num_abs_boundary_faces"] = len(f)
        # sources (sourcearrays(NSOURCES,3,5,5,5): source index fastest)
        ns = int(db["nsources"])
        s = np.nonzero(np.isin(db["ispec_selected_source"] - 1, el))[0]
        d["nsources"] = len(s)
        d["ispec_selected_source"] = eloc[db["ispec_selected_source"][s]]
        d["sourcearrays"] = db["sourcearrays"].reshape(-1, ns)[:, s].reshape(-1) if ns else db["sourcearrays"]
        d["stf"] = np.asarray(db["stf"]).reshape(ns, -1)[s]
        # receivers
        nr = int(db["nrec"])
        r = np.nonzero(np.isin(db["ispec_selected_rec"] - 1, el))[0]
        d["nrec"] = len(r)
        d["receiver_index"] = r
        d["ispec_selected_rec"] = eloc[db["ispec_selected_rec"][r]]
        for n in ("hxir", "hetar", "hgammar"):
            d[n] = db[n].reshape(nr, 5)[r].reshape(-1)
        # interfaces with the other slices
        nb, lists = [], []
        for q in range(nparts):
            if q == p:
                continue
            shared = np.intersect1d(gl, points[q])
            if len(shared):
                nb.append(q)
                lists.append(loc[shared])
        d["neighbours"] = nb
        d["num_interfaces"] = len(nb)
        mx = max((len(x) for x in lists), default=0)
        d["max_nibool_interfaces"] = mx
        d["nibool_interfaces"] = np.asarray([len(x) for x in lists], np.int32)
        ibi = np.zeros((max(len(nb), 1), max(mx, 1)), np.int32)
        for i, x in enumerate(lists):
            ibi[i, :len(x)] = x
        d["ibool_interfaces"] = ibi.reshape(-1)  # Fortran (max_nibool, num_interfaces)
        on_iface = np.zeros(len(gl) + 1, bool)
        for x in lists:
            on_iface[x] = True
        outer = np.nonzero(on_iface[d["ibool"].reshape(-1, NGLL3)].any(axis=1))[0] + 1
        d["phase_outer"] = outer.astype(np.int32)
        parts.append(d)
    return parts


def receive_buffers(parts, sent):
    """The receive buffer of every slice: for interface i of slice p (neighbour q),
    the section of q's send buffer for its interface with p."""
    out = []
    for p, d in enumerate(parts):
        buf = np.zeros_like(sent[p])
        for i, q in enumerate(d["neighbours"]):
            j = parts[q]["neighbours"].index(p)
            buf[i] = sent[q][j]
        out.append(buf)
    return out
