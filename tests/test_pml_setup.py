"""C-PML set-up (specfem3d_gb300.pml): regions, damping profiles, parameter
separation, recursive-convolution coefficients and the PML mass matrix of a
block, against the formulas of the reference's set-up
(pml_set_local_dampingcoeff.f90, prepare_timerun.F90 prepare_timerun_pml,
pml_compute_accel_contribution.f90, pml_compute_memory_variables.f90,
define_mass_matrices.f90), and a short oracle run with the layers."""
import numpy as np
import pytest

import pml_cases as C


@pytest.fixture(scope="module")
def setup():
    from specfem3d_gb300 import meshgen, pml
    cfg = C.block(12, 6, 0.0, 40)
    db = meshgen.build_database(cfg)
    return cfg, db, pml.setup(db, cfg, nel=2)


def test_regions(setup):
    from specfem3d_gb300 import pml
    cfg, db, p = setup
    r = p["cpml_regions"]
    counts = np.bincount(r, minlength=8)
    # 12 x 12 x 6 cubes, two layers on xmin xmax ymin ymax and the bottom
    assert counts[0] == 8 * 8 * 4
    assert counts[pml.X_ONLY] == counts[pml.Y_ONLY] == 2 * 2 * 8 * 4
    assert counts[pml.Z_ONLY] == 8 * 8 * 2
    assert counts[pml.XY_ONLY] == 4 * 4 * 4
    assert counts[pml.XZ_ONLY] == counts[pml.YZ_ONLY] == 2 * 2 * 8 * 2
    assert counts[pml.XYZ] == 4 * 4 * 2
    assert len(p["cpml_to_spec"]) == (r > 0).sum()


def test_damping_profiles(setup):
    from specfem3d_gb300 import pml
    cfg, db, p = setup
    K, d, al = p["pml_K"], p["pml_d"], p["pml_alpha"]
    assert (K == 1).all() and (d >= 0).all() and (al >= 0).all()
    assert np.allclose(p["pml_width"], 2 * C.H)
    f0 = 2.0
    amax = np.pi * f0 * np.array([0.9, 1.0, 1.1])
    # a face element: d grows as dist^1.2 (NPOWER = 1) to d0 at the outer face
    reg = p["cpml_regions"][p["cpml_to_spec"] - 1]
    d0 = -(1.0 + 1.0) * 3000.0 * np.log(0.001) / (2.0 * 2 * C.H)
    assert np.isclose(d[0][reg == pml.X_ONLY].max(), d0, rtol=1e-5)
    assert (al[0][reg == pml.X_ONLY] <= amax[0] * (1 + 1e-6)).all()
    assert not d[1][reg == pml.X_ONLY].any() and not d[2][reg == pml.X_ONLY].any()
    # the separation the recursive convolution needs on edges and corners
    mind = p["pml_min_distance"]
    for rr, (a0, a1) in ((pml.XY_ONLY, (0, 1)), (pml.XZ_ONLY, (0, 2)), (pml.YZ_ONLY, (1, 2))):
        sel = reg == rr
        ax, ay = al[a0][sel], al[a1][sel]
        bx, by = ax + d[a0][sel] / K[a0][sel], ay + d[a1][sel] / K[a1][sel]
        assert (np.abs(ax - ay) >= mind * (1 - 1e-5)).all()
        assert (np.abs(bx - ay) >= mind * (1 - 1e-5)).all() and (np.abs(by - ax) >= mind * (1 - 1e-5)).all()
    sel = reg == pml.XYZ
    a = al[:, sel]
    for i, j in ((0, 1), (0, 2), (1, 2)):
        assert (np.abs(a[i] - a[j]) >= mind * (1 - 1e-5)).all()


def test_convolution_coefficients():
    from specfem3d_gb300 import pml
    dt, mind = 0.008, 0.05
    for b in (0.3, 5.0, 40.0):
        c0, c1, c2 = pml.convolution_coef(b, dt, mind)
        e = np.exp(-0.5 * b * dt)
        # CUSTOM_REAL arithmetic as the reference: 1 - exp(-b dt / 2) cancels in float32
        assert np.isclose(c0, e * e, rtol=1e-6) and np.isclose(c1, (1 - e) / b, rtol=1e-3)
        assert np.isclose(c2, (1 - e) / b * e, rtol=1e-3)
    # below the threshold: the third-order Taylor expansion, continuous at b -> 0
    c0, c1, c2 = pml.convolution_coef(1e-4, dt, mind)
    assert np.isclose(c1, dt / 2, rtol=1e-3) and np.isclose(c2, dt / 2, rtol=1e-3) and np.isclose(c0, 1.0)


def test_coefficients_and_mass(setup):
    from specfem3d_gb300 import pml
    cfg, db, p = setup
    for k in ("alpha", "beta", "abar", "strain"):
        assert np.isfinite(p["pml_coef_" + k]).all()
    reg = p["cpml_regions"][p["cpml_to_spec"] - 1]
    # X_ONLY A-bar: kappa_x (beta - alpha), -kappa_x alpha (beta - alpha), kappa_x alpha^2 (beta - alpha), 0, 0
    e = int(np.nonzero(reg == pml.X_ONLY)[0][0])
    K, d, al = p["pml_K"][0, e], p["pml_d"][0, e], p["pml_alpha"][0, e]
    be = al + d / K
    ab = p["pml_coef_abar"][e]
    assert np.allclose(ab[:, 0], K * (be - al), rtol=1e-5, atol=1e-6)
    assert np.allclose(ab[:, 1], -K * al * (be - al), rtol=1e-5, atol=1e-4)
    assert not ab[:, 3:].any()
    # the PML mass is the regular mass plus rho J w dt/2 sum d inside the layers
    m0 = db["rmass"].astype(np.float64)
    m1 = p["rmass"].astype(np.float64)
    assert (m1 >= m0 * (1 - 1e-6)).all() and m1.sum() > m0.sum()
    assert np.allclose(1.0 / p["rmassx"].astype(np.float64), m1, rtol=1e-6)


def test_oracle_runs_with_layers(setup):
    from oracle import oracle as O
    cfg, db, p = setup
    sim = O.make_sim(p, cfg, "f32", nthreads=2)
    sim.step(40)
    s = O.seismograms(sim)
    assert np.isfinite(s).all() and np.abs(s).max() > 0
    assert np.abs(sim.get("pml_displ_new")).max() > 0


def test_vectorized_coefficients_equal_the_per_point_routines(setup):
    """The set-up applies the per-point restatements of the reference routines to
    whole regions at once; on every point of the block they agree with the scalar
    routines to float32 rounding (exp may differ by one ulp between numpy's vector
    and scalar paths)."""
    from specfem3d_gb300 import pml
    cfg, db, p = setup
    K, d, al = p["pml_K"], p["pml_d"], p["pml_alpha"]
    reg = p["cpml_regions"][p["cpml_to_spec"] - 1]
    dt, mind = float(cfg["dt"]), p["pml_min_distance"]
    rng = np.random.default_rng(0)
    for e in rng.choice(len(reg), 60, replace=False):
        for q in rng.choice(125, 5, replace=False):
            kx, ky, kz = K[:, e, q]
            dx, dy, dz = d[:, e, q]
            ax, ay, az = al[:, e, q]
            ref = []
            for a_ in (ax, ay, az):
                ref += list(pml.convolution_coef(a_, dt, mind))
            assert np.allclose(p["pml_coef_alpha"][e, q], ref, rtol=1e-6, atol=1e-12)
            r = int(reg[e])
            lp = pml.l_parameters(kx, dx, ax, ky, dy, ay, kz, dz, az, r)[1:]
            assert np.allclose(p["pml_coef_abar"][e, q], lp, rtol=1e-6, atol=1e-9)
            st = (list(pml.lijk_parameters(kz, dz, az, ky, dy, ay, kx, dx, ax, r, 231)) +
                  list(pml.lijk_parameters(kx, dx, ax, kz, dz, az, ky, dy, ay, r, 132)) +
                  list(pml.lijk_parameters(kx, dx, ax, ky, dy, ay, kz, dz, az, r, 123)) +
                  list(pml.lq_parameters(kx, dx, ax, r, 0)) + list(pml.lq_parameters(ky, dy, ay, r, 1)) +
                  list(pml.lq_parameters(kz, dz, az, r, 2)))
            assert np.allclose(p["pml_coef_strain"][e, q], st, rtol=1e-6, atol=1e-9)
