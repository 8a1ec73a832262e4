"""General hexahedral meshes: the product's numpy set-up chain (specfem3d_gb300.hexmesh)
against the block builder and against the oracle's C restatement of
xgenerate_databases + the solver's point location, on a structured block, a block
with randomly moved interior nodes, a rotated block, and the reference's own CUBIT
mesh files when the reference tree is present (its root in the environment variable
SPECFEM3D_REFERENCE).

Bars: integer arrays (ibool, nglob, irregular numbering, face ijk, selected
elements) bit-exact; metric terms and face geometry within 2 float32 ulps of the
oracle's (both evaluate the same double-precision formulas, summed in another
order); mass matrices within 1e-6 relative (float32 sums in another order); local
coordinates of sources and receivers within 1e-9."""
import os

import numpy as np
import pytest

from conftest import ROOT
import hexmesh_cases as C

# root of a SPECFEM3D source tree (read-only); the two tests on its CUBIT meshes skip without it
REF_EXAMPLES = os.path.join(os.environ.get("SPECFEM3D_REFERENCE", ""), "EXAMPLES", "applications")

INT_KEYS = ["ibool", "irregular_element_number", "abs_boundary_ispec", "abs_boundary_ijk", "ispec_selected_source",
            "ispec_selected_rec", "coupling_ac_el_ispec", "coupling_ac_el_ijk", "free_surface_ispec",
            "free_surface_ijk", "ispec_is_acoustic"]
F32_KEYS = ["xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian",
            "abs_boundary_jacobian2Dw", "abs_boundary_normal", "coupling_ac_el_jacobian2Dw", "coupling_ac_el_normal",
            "rhostore", "kappastore", "mustore", "rho_vp", "rho_vs"]
SUM_KEYS = ["rmass", "rmassx", "rmassy", "rmassz", "rmass_acoustic", "sourcearrays", "hxir", "hetar", "hgammar",
            "factor_common", "factor_common_kappa"]


def _compare(a, b, ulps=2, rel=1e-6):
    assert a["nspec"] == b["nspec"] and a["nglob"] == b["nglob"]
    assert a["nspec_irregular"] == b["nspec_irregular"]
    assert np.float32(a["xix_regular"]) == np.float32(b["xix_regular"])
    assert np.float32(a["jacobian_regular"]) == np.float32(b["jacobian_regular"])
    for k in INT_KEYS:
        if k in a and k in b:
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    metric_scale = max(float(np.abs(np.asarray(b[k])).max()) for k in F32_KEYS[:9])
    for k in F32_KEYS:
        if k in a and k in b and np.asarray(a[k]).size:
            x, y = np.asarray(a[k], np.float32), np.asarray(b[k], np.float32)
            # values far below their array's scale (off-diagonal metric terms of
            # axis-aligned elements: exact zeros on one side, rounding residue of
            # the general formulas on the other) are held to the scale's ulps
            scale = np.float32(metric_scale if k in F32_KEYS[:9] else np.abs(y).max())
            tol = ulps * np.spacing(np.maximum(np.abs(y), scale * np.float32(1e-6)))
            assert (np.abs(x - y) <= tol).all(), (k, float(np.abs(x - y).max()))
    for k in SUM_KEYS:
        if k in a and k in b and np.asarray(a[k]).size:
            x, y = np.asarray(a[k], np.float64), np.asarray(b[k], np.float64)
            assert np.abs(x - y).max() <= rel * np.abs(y).max(), (k, float(np.abs(x - y).max() / np.abs(y).max()))
    for k in ("source_xi_eta_gamma", "receiver_xi_eta_gamma"):
        assert np.abs(np.asarray(a[k]) - np.asarray(b[k])).max() <= 1e-9, k


def _cfg_layered():
    from specfem3d_gb300 import configs
    return configs.small_layered(nstep=10, attenuation=True)


def _cfg_coupled():
    from specfem3d_gb300 import configs
    cfg = configs.small_coupled(nstep=10)
    cfg.pop("perturbation", None)       # one material per element row
    return cfg


@pytest.mark.parametrize("which", ["layered", "coupled"])
def test_block_mesh_matches_block_builder(which):
    """The general path on a structured block reproduces the block builder's
    database (which the GPU parity tests already hold to the oracle)."""
    from specfem3d_gb300 import hexmesh, meshgen
    cfg = _cfg_layered() if which == "layered" else _cfg_coupled()
    a = hexmesh.build_database(hexmesh.block_mesh(cfg), cfg)
    b = meshgen.build_database(cfg)
    _compare(a, b)


@pytest.mark.parametrize("case", ["distorted", "rotated", "rotated_distorted", "coupled_distorted"])
def test_general_mesh_matches_oracle(case):
    """Moved interior nodes and a rotation give full, varying metric tensors:
    every array of the general path matches the oracle's restatement."""
    from specfem3d_gb300 import hexmesh
    from oracle import oracle as O
    cfg = _cfg_coupled() if case.startswith("coupled") else _cfg_layered()
    R = C.rotation()
    if case == "distorted" or case == "coupled_distorted":
        mesh, c = C.distorted(cfg), cfg
    elif case == "rotated":
        mesh, c = C.rotated(cfg, R)
    else:
        mesh, c = C.rotated(cfg, R, C.distorted(cfg))
    a = hexmesh.build_database(mesh, c)
    b = O.build_database_from_mesh(mesh, c)
    if case.startswith("coupled"):
        b.update(O.fluid_setup(b, c))
        assert a["num_coupling_ac_el_faces"] > 0
        assert a["num_coupling_ac_el_faces"] == b["num_coupling_ac_el_faces"]
        assert np.abs(a["rmass"] - b["rmass_solid"]).max() <= 1e-6 * np.abs(b["rmass_solid"]).max()
        # the oracle's elastic set-up sums the mass over every element; its fluid
        # set-up gives the solid-only mass compared above
        b = {k: v for k, v in b.items() if k not in ("rmass", "rmassx", "rmassy", "rmassz")}
    assert a["nspec_irregular"] == a["nspec"]
    _compare(a, b)


def test_global_numbering_tolerance():
    """Points closer than the tolerance merge; the numbering follows first
    appearance whatever the input order of coordinates."""
    from specfem3d_gb300 import hexmesh
    rng = np.random.default_rng(3)
    base = rng.integers(0, 6, size=(400, 3)).astype(np.float64) * 10.0
    jitter = rng.uniform(-1e-9, 1e-9, size=base.shape)
    ib, n = hexmesh.get_global(base + jitter, 1e-7)
    _, first, inv = np.unique(base, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)
    rank = np.empty(len(first), np.int64)
    rank[order] = np.arange(len(first))
    assert n == len(first)
    assert np.array_equal(ib, rank[inv.reshape(-1)] + 1)
    from oracle import oracle as O
    xs, ys, zs = (np.ascontiguousarray((base + jitter)[:, d]) for d in range(3))
    ib2 = np.zeros(400, np.int32)
    n2 = O.lib().orc_get_global(400, xs.ctypes.data, ys.ctypes.data, zs.ctypes.data, ib2.ctypes.data, 1e-7)
    assert n2 == n and np.array_equal(ib2, ib)


def test_face_records_must_match_an_element_face():
    from specfem3d_gb300 import hexmesh
    cfg = _cfg_layered()
    mesh = hexmesh.block_mesh(cfg)
    recs = mesh["faces"]["absorbing_surface_file_xmin"].copy()
    assert (hexmesh.face_ids(mesh["elems"], recs) == 1).all()
    recs[3, 1] = recs[3, 0] * 0 + mesh["elems"][recs[3, 0], 6]   # a node of the opposite face
    with pytest.raises(ValueError, match="matches no face"):
        hexmesh.face_ids(mesh["elems"], recs)


def test_source_octant_choice_agrees_between_block_and_general_paths():
    """A source on a vertex of 8 elements goes into the element on the requested
    side, in the block builder, the general path and the oracle alike."""
    from specfem3d_gb300 import configs, hexmesh, meshgen
    from oracle import oracle as O
    cfg = configs.refex_no_absorbing(10)
    a = meshgen.build_database(cfg)
    b = hexmesh.build_database(hexmesh.block_mesh(cfg), cfg)
    o = O.build_database(cfg)
    e = int(a["ispec_selected_source"][0]) - 1
    assert (e % 36, (e // 36) % 36, e // 1296) == (17, 18, 7)
    for d in (b, o):
        assert d["ispec_selected_source"][0] == a["ispec_selected_source"][0]
        assert np.allclose(d["source_xi_eta_gamma"], a["source_xi_eta_gamma"], atol=1e-12)
        assert np.abs(d["sourcearrays"] - a["sourcearrays"]).max() <= 1e-6 * np.abs(a["sourcearrays"]).max()


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="SPECFEM3D_REFERENCE does not name a reference tree")
def test_reference_cubit_mesh_files():
    """The reference example's own MESH-default (a CUBIT mesh of the same block with
    its elements in another order and orientation): the database has the block's
    point count and mass, the source lands where the reference's log puts it
    (element with local coordinates (-1, -1, 1)), and every receiver's located
    position reproduces its target."""
    from specfem3d_gb300 import configs, hexmesh, meshgen
    d = os.path.join(REF_EXAMPLES, "homogeneous_halfspace_HEX8_elastic_no_absorbing")
    mesh = hexmesh.read_external_mesh(os.path.join(d, "MESH-default"))
    assert mesh["elems"].shape == (20736, 8) and len(mesh["materials"]) == 1
    src = hexmesh.read_cmtsolution(os.path.join(d, "DATA", "CMTSOLUTION"))
    cfg = configs.refex_no_absorbing(10)
    assert np.allclose(src["M"], cfg["sources"][0]["M"], rtol=1e-12)
    assert (src["x"], src["y"], src["z"]) == (67000.0, 67000.0, -30000.0)
    st = hexmesh.read_stations(os.path.join(d, "DATA", "STATIONS"))
    assert [s[0] for s in st] == ["X20", "X30", "X40", "X50"]
    par = hexmesh.read_par_file(os.path.join(d, "DATA", "Par_file"))
    assert par["NSTEP"] == 5000 and par["DT"] == 0.05 and not par["STACEY_ABSORBING_CONDITIONS"]
    db = hexmesh.build_database(mesh, cfg)
    blk = meshgen.build_database(cfg)
    assert db["nglob"] == blk["nglob"]
    assert abs(db["rmass"].astype(np.float64).sum() / blk["rmass"].astype(np.float64).sum() - 1) < 1e-6
    assert np.allclose(db["source_xi_eta_gamma"][0], [-1.0, -1.0, 1.0])
    xyz = hexmesh.gll_points(mesh["nodes"][mesh["elems"]])
    for r, (x, y, z) in enumerate(cfg["receivers"]):
        e = int(db["ispec_selected_rec"][r]) - 1
        h = [db[k].reshape(-1, 5)[r] for k in ("hxir", "hetar", "hgammar")]
        w = (h[2][:, None, None] * h[1][None, :, None] * h[0][None, None, :]).reshape(-1)
        assert np.allclose(w @ xyz[e], [x, y, z], atol=1e-6 * 134000.0)


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="SPECFEM3D_REFERENCE does not name a reference tree")
def test_reference_cubit_waterlayered_mesh():
    """waterlayered_halfspace's own CUBIT mesh, Par_file, CMTSOLUTION and STATIONS
    read and set up by the general path give the database of the block
    configuration the GPU golden test runs (configs.waterlayered): same point count,
    coupling, absorbing and free-surface faces, masses, source time function, and
    the same fluid/solid side for every station."""
    from specfem3d_gb300 import configs, hexmesh, meshgen
    d = os.path.join(REF_EXAMPLES, "waterlayered_halfspace")
    mesh = hexmesh.read_external_mesh(os.path.join(d, "MESH-default"))
    assert mesh["elems"].shape == (40500, 8) and len(mesh["materials"]) == 3
    par = hexmesh.read_par_file(os.path.join(d, "DATA", "Par_file"))
    assert par["NSTEP"] == 4500 and par["DT"] == 0.005 and par["STACEY_ABSORBING_CONDITIONS"]
    src = hexmesh.read_cmtsolution(os.path.join(d, "DATA", "CMTSOLUTION"))
    src["stf"] = "heaviside"
    st = hexmesh.read_stations(os.path.join(d, "DATA", "STATIONS"))
    ref_cfg = configs.waterlayered(20)
    assert [s[0] for s in st] == ref_cfg["station_names"]
    cfg = dict(dt=par["DT"], nstep=20, stacey=True, sources=[src], receivers=[(x, y, z) for _, _, x, y, z in st])
    assert np.allclose(cfg["receivers"], ref_cfg["receivers"])
    a = hexmesh.build_database(mesh, cfg)
    b = meshgen.build_database(ref_cfg)
    for k in ("nglob", "num_coupling_ac_el_faces", "num_abs_boundary_faces", "num_free_surface_faces"):
        assert a[k] == b[k], k
    for k in ("rmass", "rmass_acoustic", "rmassx", "rmassy", "rmassz"):
        assert abs(a[k].astype(np.float64).sum() / b[k].astype(np.float64).sum() - 1) < 1e-6, k
    assert a["t0"] == b["t0"] == 6.0 and np.allclose(a["stf"], b["stf"])
    fa, fb = a["ispec_is_acoustic"].astype(bool), b["ispec_is_acoustic"].astype(bool)
    assert fa.sum() == fb.sum() == 2025
    assert np.array_equal(fa[a["ispec_selected_rec"] - 1], fb[b["ispec_selected_rec"] - 1])
    assert fa[a["ispec_selected_source"][0] - 1]
