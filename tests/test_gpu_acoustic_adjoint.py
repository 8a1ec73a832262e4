"""SIMULATION_TYPE = 3 on a fluid-solid mesh through the reference-named entry
points (FORWARD_OR_ADJOINT = 3 on the acoustic entry points, the acoustic
boundary record b_absorb_potential, compute_add_sources_ac_s3_cuda,
prepare_fields_acoustic_adj_dev, compute_kernels_acoustic_cuda):

* the backward potentials reconstructed in reverse time (Stacey records of both
  domains replayed) follow the forward run's potentials;
* rho_ac_kl and kappa_ac_kl equal the reference's accumulation
  (compute_kernels.f90:257-330: dt grad(chi_adj).grad(b_chi) and
  dt chi_adj b_chi_dd) restated on the host from the device's fields;
* the solid kappa kernel of the coupled run gives the derivative of the misfit of
  solid receivers (central differences of the FP64 oracle, eps = 3e-5);
* in the fluid, the derivative of the misfit along a kappa perturbation is the
  pairing of chi_adj_dd (not chi_adj) with b_chi_dd: the reference's adjoint
  potential is the second time integral of the discrete adjoint variable of the
  fluid (its coupling terms are u.n and chi_dd n with flipped signs), so its
  kappa kernel is the continuous-adjoint formula, not the discrete gradient.
  The test prints the reference formula's value beside the finite difference.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 3e-5


def _setup():
    from specfem3d_gb300 import configs, gradient as G
    cfg = configs.small_coupled(nstep=300)
    h = 20000.0 / 96
    z = cfg["zlev"][0] + 2.5 * h  # in the solid, below the fluid layers
    cfg["receivers"] = [(cfg["x1"] * fx, cfg["y1"] * fy, z) for fx, fy in ((0.3, 0.4), (0.7, 0.6), (0.45, 0.55))]
    # a moment tensor in the solid and the force of the configuration in the fluid
    # (amplitudes that keep every field well inside FP32's normal range)
    src = dict(cfg["sources"][0])
    src["F"] = [1e10 * f for f in src["F"]]
    cmt = dict(type="cmt", x=cfg["x1"] * 0.55, y=cfg["y1"] * 0.45, z=cfg["zlev"][0] + 1.5 * h,
               M=[1e10 * m for m in (0.3, -0.5, 0.2, 0.4, -0.1, 0.25)], stf="ricker", f0=3.0)
    cfg["sources"] = [cmt, src]
    cfg["record"] = ("displ",)
    mat = tuple(np.asarray(m, np.float64) for m in G.background_material(cfg))
    return cfg, mat


def _db(cfg, mat, dtype=np.float32):
    from specfem3d_gb300 import meshgen
    return meshgen.build_database(cfg, material=tuple(np.asarray(m, dtype) for m in mat), dtype=dtype)


def _misfit64(cfg, mat):
    from oracle import oracle as O
    db = _db(cfg, mat, np.float64)
    sim = O.make_coupled_sim(db, cfg, "f64", nthreads=os.cpu_count() or 1)
    O.run_coupled(sim, cfg["nstep"])
    s = O.seismograms(sim)
    return 0.5 * float(cfg["dt"]) * float(np.sum(s * s))


def _volume(db):
    from specfem3d_gb300.meshgen import NGLL3, WGLL
    n = int(db["nspec"])
    irr = np.asarray(db["irregular_element_number"])
    jac = np.empty((n, NGLL3))
    reg = irr == 0
    jac[reg] = float(np.float32(db["jacobian_regular"]))
    if (~reg).any():
        jac[~reg] = np.asarray(db["jacobian"], np.float64).reshape(-1, NGLL3)[irr[~reg] - 1]
    w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1)
    return jac * w3[None, :]


def _run(stacey, fluid_source, discrete=False, hessian=False):
    from specfem3d_gb300 import adjoint as ADJ
    from specfem3d_gb300.solver import GPUSolver
    cfg, mat = _setup()
    cfg["stacey"] = bool(stacey)
    if not fluid_source:
        cfg["sources"] = cfg["sources"][:1]
    db = _db(cfg, mat)
    assert int(db["num_coupling_ac_el_faces"]) > 0
    seis, fin_el, fin_ac, rec_el, rec_ac = ADJ.forward_with_boundary_record_coupled(db, cfg)
    g = GPUSolver(db, cfg, nlength=cfg["nstep"])
    H = {}
    for s in range(1, cfg["nstep"] + 1):
        g.run_per_call(1)
        H[s] = g.potentials()[0]
    g.close()
    hist = []
    kl = ADJ.kernel_run_coupled(db, cfg, seis.astype(np.float64), fin_el, fin_ac, rec_el, rec_ac, history=hist,
                                discrete_fluid_kernels=discrete, hessian=hessian)
    return cfg, mat, db, seis, H, hist, kl


@pytest.fixture(scope="module")
def run_stacey(gpulib):
    """Stacey faces on the sides and bottom, a source in each domain."""
    return _run(True, True, hessian=True)


@pytest.fixture(scope="module")
def run_plain(gpulib):
    """No absorbing faces (the Stacey coefficients rho vp, rho vs depend on the model
    and the volume kernels leave that out), the moment tensor only."""
    return _run(False, False)


@pytest.fixture(scope="module")
def run_discrete(gpulib):
    """As run_plain, with the fluid kernels pairing chi_adj_dd (sf3d_set_acoustic_kernel_pairing)."""
    return _run(False, False, discrete=True)


def _gradient(db, f):
    """Physical gradient of a global scalar field at every element point, the
    way the kernels take it: d/dxi_l = sum_m hprime_xx(l, m) f_m, then the metric."""
    n = int(db["nspec"])
    ib = np.asarray(db["ibool"]).reshape(n, 5, 5, 5) - 1          # [e][k][j][i]
    X = np.asarray(f, np.float64)[ib]
    HP = np.asarray(db["hprime_xx"], np.float64).reshape(5, 5).T  # HP[i, l] = hprime_xx(i, l)
    d0 = np.einsum("ekjl,il->ekji", X, HP)
    d1 = np.einsum("eklx,jl->ekjx", X, HP)
    d2 = np.einsum("eljx,kl->ekjx", X, HP)
    irr = np.asarray(db["irregular_element_number"]) - 1
    g = np.empty((3, n, 5, 5, 5))
    xr = float(np.float32(db["xix_regular"]))
    for c in range(3):
        g[c] = xr * (d0, d1, d2)[c]
    if (irr >= 0).any():
        names = ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz")
        M = [np.asarray(db[q], np.float64).reshape(-1, 5, 5, 5) for q in names]
        e = np.nonzero(irr >= 0)[0]
        r = irr[e]
        for c in range(3):
            g[c][e] = M[c][r] * d0[e] + M[3 + c][r] * d1[e] + M[6 + c][r] * d2[e]
    return g.reshape(3, n, 125)


def test_backward_potentials_follow_the_forward_run(run_stacey):
    """b_potential at adjoint step it is the forward potential of step NSTEP - it + 1
    (the first step is replaced by the saved final state); measured 4.0e-7."""
    cfg, mat, db, seis, H, hist, kl = run_stacey
    nstep = cfg["nstep"]
    assert int(db["num_abs_boundary_faces"]) > 0
    scale = max(np.linalg.norm(h) for h in H.values())
    worst = max(np.linalg.norm(h["b_chi"].astype(np.float64) - H[nstep - h["it"] + 1]) for h in hist) / scale
    print(f"backward potentials vs forward run: worst {worst:.2e} of the largest potential")
    assert np.abs(seis).max() > 0
    assert worst < 1e-5


def test_fluid_kernels_equal_the_reference_accumulation(run_stacey):
    """Both accumulators against the host restatement of compute_kernels.f90:257-330
    from the fields of every step (FP64 sums of FP32 fields); measured 1.7e-8."""
    cfg, mat, db, seis, H, hist, kl = run_stacey
    n, dt = int(db["nspec"]), float(cfg["dt"])
    fluid = np.repeat(np.asarray(db["ispec_is_acoustic"]) > 0, 125).reshape(n, 125)
    ib = np.asarray(db["ibool"]).reshape(n, 125) - 1
    kap, rho = np.zeros((n, 125)), np.zeros((n, 125))
    for h in hist:
        kap += dt * h["chi"].astype(np.float64)[ib] * h["b_chi_dd"].astype(np.float64)[ib]
        ga, gb = _gradient(db, h["chi"]), _gradient(db, h["b_chi"])
        rho += dt * np.sum(ga * gb, axis=0)
    ek = np.linalg.norm((kl["kappa_ac"] - kap)[fluid]) / np.linalg.norm(kap[fluid])
    er = np.linalg.norm((kl["rho_ac"] - rho)[fluid]) / np.linalg.norm(rho[fluid])
    print(f"fluid kernels vs host restatement: kappa {ek:.2e}, rho {er:.2e}")
    assert np.abs(kap[fluid]).max() > 0 and np.abs(rho[fluid]).max() > 0
    assert not kl["kappa_ac"][~fluid].any() and not kl["rho_ac"][~fluid].any()
    assert ek < 1e-6 and er < 1e-5


def test_solid_kernels_of_the_coupled_run_match_finite_differences(run_plain):
    """The solid's kappa kernel (K = -kappa kappa_kl) along a smooth perturbation of
    the solid's kappa (mu fixed); measured 1.5e-7."""
    from specfem3d_gb300 import gradient as G
    cfg, mat, db, seis, H, hist, kl = run_plain
    n = int(db["nspec"])
    solid = np.repeat(np.asarray(db["ispec_is_acoustic"]) == 0, 125).reshape(n, 125)
    rho, vp, vs = mat
    kappa = np.asarray(db["kappastore"], np.float64).reshape(n, 125)
    d = G.smooth_direction(cfg, 33, corr_len=600.0).reshape(n, 125) * solid
    mu = rho * vs * vs
    k0 = rho * vp * vp - 4.0 / 3.0 * mu
    js = []
    for sgn in (1.0, -1.0):
        k = k0 * (1.0 + sgn * EPS * d.reshape(-1))
        js.append(_misfit64(cfg, (rho, np.sqrt((k + 4.0 / 3.0 * mu) / rho), vs)))
    fd = (js[0] - js[1]) / (2 * EPS)
    pred = float(np.sum(-kappa * kl["kappa"] * d * _volume(db)))
    e = abs(pred - fd) / abs(fd)
    print(f"solid kappa: finite difference {fd:.6e}, kernels {pred:.6e}, relative {e:.2e}")
    assert e < 1e-4


def test_fluid_kappa_derivative_is_the_second_derivative_pairing(run_plain):
    """sum dt chi_adj_dd b_chi_dd / kappa (J w) delta over fluid element points against
    central differences along a smooth relative perturbation of the fluid's kappa
    (rho fixed); measured 2.4e-5.  The reference formula (chi_adj in place of
    chi_adj_dd) is printed beside it."""
    from specfem3d_gb300 import gradient as G
    cfg, mat, db, seis, H, hist, kl = run_plain
    n, dt = int(db["nspec"]), float(cfg["dt"])
    fluid = np.repeat(np.asarray(db["ispec_is_acoustic"]) > 0, 125).reshape(n, 125)
    ib = np.asarray(db["ibool"]).reshape(n, 125) - 1
    acc = np.zeros((n, 125))
    for h in hist:
        acc += dt * h["chi_dd"].astype(np.float64)[ib] * h["b_chi_dd"].astype(np.float64)[ib]
    kap = np.asarray(db["kappastore"], np.float64).reshape(n, 125)
    rho, vp, vs = mat
    vol = _volume(db)
    d = G.smooth_direction(cfg, 11, corr_len=600.0).reshape(n, 125) * fluid
    js = [_misfit64(cfg, (rho, vp * np.sqrt((1.0 + s * EPS * d).reshape(-1)), vs)) for s in (1.0, -1.0)]
    fd = (js[0] - js[1]) / (2 * EPS)
    pred = float(np.sum(acc / kap * d * vol))
    ref_formula = float(np.sum(kl["kappa_ac"] / kap * d * vol))
    e = abs(pred - fd) / abs(fd)
    print(f"fluid kappa: finite difference {fd:.6e}, chi_adj_dd pairing {pred:.6e} (relative {e:.2e}), "
          f"reference formula {ref_formula:.6e}")
    assert abs(fd) > 0 and e < 1e-3


@pytest.mark.parametrize("param", ["kappa", "rho"])
def test_discrete_fluid_kernels_match_finite_differences(run_discrete, param):
    """With the chi_adj_dd pairing the library's fluid kernels, scaled as the
    reference scales its own (K = kl / kappa, kl / rho), give the derivative of the
    misfit along smooth relative perturbations of the fluid's kappa (rho fixed) or
    rho (kappa fixed): central differences of the FP64 oracle, eps = 3e-5."""
    from specfem3d_gb300 import gradient as G
    cfg, mat, db, seis, H, hist, kl = run_discrete
    n = int(db["nspec"])
    fluid = np.repeat(np.asarray(db["ispec_is_acoustic"]) > 0, 125).reshape(n, 125)
    rho, vp, vs = mat
    store = np.asarray(db["kappastore" if param == "kappa" else "rhostore"], np.float64).reshape(n, 125)
    K = kl[param + "_ac"] / store
    d = G.smooth_direction(cfg, 11 if param == "kappa" else 22, corr_len=600.0).reshape(n, 125) * fluid
    js = []
    for sgn in (1.0, -1.0):
        f = (1.0 + sgn * EPS * d).reshape(-1)
        m = (rho, vp * np.sqrt(f), vs) if param == "kappa" else (rho * f, vp / np.sqrt(f), vs)
        js.append(_misfit64(cfg, m))
    fd = (js[0] - js[1]) / (2 * EPS)
    pred = float(np.sum(K * d * _volume(db)))
    e = abs(pred - fd) / abs(fd)
    print(f"discrete fluid {param}: finite difference {fd:.6e}, kernels {pred:.6e}, relative {e:.2e}")
    assert abs(fd) > 0 and e < 1e-3


def test_fluid_hessian_kernels_equal_the_reference_accumulation(run_stacey):
    """hess_ac_kl, hess_rho_ac_kl, hess_kappa_ac_kl (compute_kernels.f90:459-510:
    gradients carry 1/rho) against the host restatement from the fields of every
    step; the device returns them in FP32 like transfer_kernels_hess_ac_tohost."""
    cfg, mat, db, seis, H, hist, kl = run_stacey
    n, dt = int(db["nspec"]), float(cfg["dt"])
    fluid = np.repeat(np.asarray(db["ispec_is_acoustic"]) > 0, 125).reshape(n, 125)
    ib = np.asarray(db["ibool"]).reshape(n, 125) - 1
    rho = np.asarray(db["rhostore"], np.float64).reshape(n, 125)
    kap = np.asarray(db["kappastore"], np.float64).reshape(n, 125)
    hs, hr, hk = (np.zeros((n, 125)) for _ in range(3))
    for h in hist:
        ga, gb, gv = (_gradient(db, h[k]) / rho for k in ("chi_dd", "b_chi_dd", "b_chi_dot"))
        hs += dt * np.sum(ga * gb, axis=0)
        hr += dt * rho * np.sum(gv * gv, axis=0)
        hk += dt * h["b_chi_dot"].astype(np.float64)[ib] ** 2 / kap
    errs = {}
    for name, ref in (("hess_ac", hs), ("hess_rho_ac", hr), ("hess_kappa_ac", hk)):
        errs[name] = np.linalg.norm((kl[name] - ref)[fluid]) / np.linalg.norm(ref[fluid])
        assert np.abs(ref[fluid]).max() > 0
        assert not kl[name][~fluid].any()
    print("fluid Hessian kernels vs host restatement: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert all(v < 1e-5 for v in errs.values())
