"""The product's database generator against the oracle's restatement of the
reference's setup (CPU): integer arrays bit-exact, floating arrays to rounding."""
import numpy as np
import pytest

INT_KEYS = ["ibool", "irregular_element_number", "abs_boundary_ispec", "abs_boundary_ijk",
            "ispec_selected_source", "ispec_selected_rec"]
FLOAT_KEYS = ["xix", "etay", "gammaz", "jacobian", "kappastore", "mustore", "rho_vp", "rho_vs", "rmassx",
              "rmassy", "rmassz", "abs_boundary_normal", "abs_boundary_jacobian2Dw", "sourcearrays", "hxir",
              "hetar", "hgammar", "hprime_xx", "hprimewgll_xx", "wgllwgll_xy", "wgllwgll_xz", "wgllwgll_yz"]


def _cfgs():
    from specfem3d_gb300 import configs
    return {"homogeneous_block": configs.homogeneous_block(nstep=20), "small_layered": configs.small_layered(nstep=20),
            "small_noatt": configs.small_layered(nstep=20, attenuation=False, nx=3, ny=4, counts=(1, 2, 2)),
            "refex": configs.refex(20)}


@pytest.mark.parametrize("name", ["homogeneous_block", "small_layered", "small_noatt", "refex"])
def test_database_parity(name):
    from oracle import oracle as O
    from specfem3d_gb300 import meshgen
    cfg = _cfgs()[name]
    a = meshgen.build_database(cfg)
    b = O.build_database(cfg, "f32")
    assert a["nglob"] == b["nglob"] and a["nspec"] == b["nspec"]
    assert a["nspec_irregular"] == b["nspec_irregular"]
    for k in INT_KEYS:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    assert np.float32(a["xix_regular"]) == np.float32(b["xix_regular"])
    assert np.float32(a["jacobian_regular"]) == np.float32(b["jacobian_regular"])
    for k in FLOAT_KEYS:
        x = np.asarray(a[k], np.float64)
        y = np.asarray(b[k], np.float64)
        assert x.shape == y.shape, k
        assert np.abs(x - y).max() <= 1e-6 * max(np.abs(y).max(), 1e-30), k
    # off-diagonal metric terms vanish for axis-aligned boxes
    for k in ["xiy", "xiz", "etax", "etaz", "gammax", "gammay"]:
        assert np.abs(b[k]).max() <= 1e-12 * max(np.abs(b["xix"]).max(), 1e-30)
        assert not np.any(a[k])
    assert np.allclose(a["stf"], b["stf"], rtol=0, atol=1e-12)
    if cfg.get("attenuation"):
        for k in ["factor_common", "factor_common_kappa", "alphaval", "betaval", "gammaval"]:
            assert np.array_equal(np.asarray(a[k], np.float32), np.asarray(b[k], np.float32)), k


def test_ibool_invariants():
    from specfem3d_gb300 import configs, meshgen
    cfg = configs.small_layered(nstep=5, nx=4, ny=3, counts=(1, 2, 1))
    db = meshgen.build_database(cfg)
    ib = db["ibool"].reshape(-1, 125)
    # every global point used, numbered by first appearance in element order
    flat = ib.reshape(-1)
    assert flat.min() == 1 and flat.max() == db["nglob"]
    first = np.unique(flat, return_index=True)[1]
    assert np.all(np.diff(flat[np.sort(first)]) == 1)
    # multiplicity: corners of interior nodes shared by 8 elements
    counts = np.bincount(flat)
    assert counts.max() == 8


def test_regular_mesh_split_follows_single_precision_rule():
    """The cube test of check_element_regularity runs on single-precision corner
    coordinates, so rounding makes most homogeneous_block cubes 'irregular'; both sides agree."""
    from specfem3d_gb300 import configs, meshgen
    db = meshgen.build_database(configs.homogeneous_block(nstep=5))
    irr = db["irregular_element_number"]
    assert 0 < (irr == 0).sum() < len(irr)
    assert np.array_equal(irr[irr > 0], np.arange(1, (irr > 0).sum() + 1))


def test_fluid_setup_parity():
    """Fluid flags, coupling faces (reference algorithm: corners and midpoint shared
    with solid elements), free surface and fluid mass matrix."""
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen, models
    cfg = configs.small_coupled(nstep=10)
    a = meshgen.build_database(cfg)
    mat = models.perturbed_material(cfg, **cfg["perturbation"])
    b = O.build_database(cfg, "f32", material=mat)
    f = O.fluid_setup(b, cfg)
    for k in ["ispec_is_acoustic", "coupling_ac_el_ispec", "coupling_ac_el_ijk", "free_surface_ispec",
              "free_surface_ijk"]:
        assert np.array_equal(np.asarray(a[k]), np.asarray(f[k])), k
    assert a["num_coupling_ac_el_faces"] == f["num_coupling_ac_el_faces"] > 0
    for k in ["coupling_ac_el_jacobian2Dw", "coupling_ac_el_normal", "rmass_acoustic"]:
        x, y = np.asarray(a[k], np.float64), np.asarray(f[k], np.float64)
        assert np.abs(x - y).max() <= 1e-6 * np.abs(y).max(), k
    assert np.abs(f["rmass_solid"] - a["rmass"]).max() <= 1e-6 * np.abs(a["rmass"]).max()
    assert np.array_equal(a["kappastore"], b["kappastore"]) and np.array_equal(a["mustore"], b["mustore"])


def test_perturbation_model_bounds():
    from specfem3d_gb300 import configs, models
    cfg = configs.small_coupled(nstep=5)
    f, _ = models.gaussian_field(cfg, seed=3)
    assert abs(f).max() <= 0.05 + 1e-12 and 0.015 < f.std() < 0.03
    rho, vp, vs = models.perturbed_material(cfg, **cfg["perturbation"])
    solid = vs > 0
    assert np.all(np.abs(vp[solid] / 3000.0 - 1) <= 0.0500001)
    assert np.all(vp[~solid] == 1500.0)


@pytest.mark.parametrize("kind", ["block", "greedy"])
def test_element_colouring_is_conflict_free(kind):
    """No two elements of one colour share a GLL point (the condition for the
    atomic-free assembly of USE_MESH_COLORING_GPU)."""
    from specfem3d_gb300 import configs, meshgen
    cfg = configs.small_layered(nx=6, ny=5, counts=(2, 2, 3), nstep=4)
    db = meshgen.build_database(cfg)
    n = db["nspec"]
    col = meshgen.block_colors(cfg) if kind == "block" else meshgen.greedy_colors(db["ibool"], n, db["nglob"])
    ib = db["ibool"].reshape(n, 125)
    for c in np.unique(col):
        pts = ib[col == c].reshape(-1)
        assert len(np.unique(pts)) == len(pts), c
    assert col.max() + 1 <= (8 if kind == "block" else 27)
