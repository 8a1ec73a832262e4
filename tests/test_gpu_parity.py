"""GPU parity: the sm_103a CUDA path, called through the C ABI, against the oracle.

Tolerances (FP32 fields on both sides; the device sums with FMA and atomics in
a different order, and recomputes J from the metric as the reference GPU does):
* one stiffness pass on random fields: relative L2 <= 2e-6 on accel;
* time-stepped seismograms: relative L2 <= 5e-5 over all receivers after two
  thousand steps; final wavefields <= 1e-4 (the field left in the block after
  the waves exit through the Stacey faces is small, so FP32 rounding of two
  differently ordered sums shows more in it);
* accuracy against the FP64 oracle (the reference built with double
  CUSTOM_REAL): the device's FP32 error is at most 1.5x the FP32 CPU oracle's;
* the fused graph-captured loop against the per-call ABI loop: seismograms
  <= 2e-5 (atomic accumulation order differs from run to run), and the same
  FP64-relative bound;
* the reference's golden seismograms: relative L2 <= 1e-3, correlation >= 0.999.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu


def _oracle_sim(db, cfg, precision="f32"):
    from oracle import oracle as O
    return O.make_sim(db, cfg, precision, nthreads=os.cpu_count() or 1)


def _solver(db, cfg, **kw):
    from specfem3d_gb300 import solver
    return solver.GPUSolver(db, cfg, **kw)


@pytest.mark.parametrize("att,variant", [(False, None), (True, None), (False, 15), (False, 16)])
def test_stiffness_pass_random_fields(gpulib, att, variant):
    """One stiffness pass on random fields against the FP32 oracle: the default
    build with and without attenuation, and the register-blocked pencil kernel
    (variants 15, 16: five elements a CTA at 8 and 7 CTAs/SM; every element of
    the layered mesh is irregular, so the metric path runs)."""
    from specfem3d_gb300 import configs, meshgen
    cfg = configs.small_layered(nstep=4, attenuation=att)
    db = meshgen.build_database(cfg)
    rng = np.random.default_rng(11)
    n3 = 3 * db["nglob"]
    d = rng.standard_normal(n3).astype(np.float32) * 1e-3
    v = rng.standard_normal(n3).astype(np.float32) * 1e-2
    a = np.zeros(n3, np.float32)
    g = _solver(db, cfg)
    if variant is not None:
        g.set_stiffness_variant(variant)
    g.set_fields(d, v, a)
    g.forces_only()
    _, _, acc_gpu = g.fields()
    sim = _oracle_sim(db, cfg)
    sim.get("displ")[:] = d
    sim.get("veloc")[:] = v
    sim.forces()
    acc_cpu = sim.get("accel")
    assert rel_l2(acc_gpu, acc_cpu) < 2e-6
    if att:
        R, E = g.memory_variables()
        for c, name in enumerate(["R_xx", "R_yy", "R_xy", "R_xz", "R_yz", "R_trace"]):
            assert rel_l2(R[c], sim.get(name)) < 2e-5, name
        for c, name in enumerate(["epsilondev_xx", "epsilondev_yy", "epsilondev_xy", "epsilondev_xz",
                                  "epsilondev_yz", "epsilondev_trace"]):
            assert rel_l2(E[c], sim.get(name)) < 2e-5, name
    g.close()


@pytest.mark.parametrize("att,mesh", [(False, "layered"), (True, "layered"), (False, "regular")])
def test_stiffness_variants_agree(gpulib, att, mesh):
    """All stiffness variants (one CTA per element at 4-7 CTAs/SM, the pipelined
    persistent kernel, the cp.async-staged builds at 6-8 CTAs/SM, the builds with
    evict-first hints, three threads per point, the bulk-copy-staged builds at
    8-10 CTAs/SM, without attenuation the register-blocked pencil kernel) do the same
    arithmetic in the same order; the scatter-added acceleration differs
    only by the order of the atomic additions, the memory variables and strains
    at most by FMA contraction choices of the compiler.  Meshes: the layered block
    (every element irregular) and a perturbed block of cubes (every element
    regular, moduli varying per point; 324 elements, so the pencil kernel's last
    CTA holds 4 of its 5 elements)."""
    from specfem3d_gb300 import configs, gradient as G, meshgen
    if mesh == "layered":
        cfg = configs.small_layered(nx=9, ny=7, counts=(3, 3, 4), nstep=4, attenuation=att)
        db = meshgen.build_database(cfg)
    else:
        cfg = configs.small_adjoint(nstep=4, nshots=1, n=9)
        db = meshgen.build_database(cfg, material=G.background_material(cfg))
        assert db["nspec"] == 324 and db["nspec_irregular"] == 0
    rng = np.random.default_rng(5)
    n3 = 3 * db["nglob"]
    d = rng.standard_normal(n3).astype(np.float32) * 1e-3
    v = rng.standard_normal(n3).astype(np.float32) * 1e-2
    out = []
    from specfem3d_gb300.solver import NUM_STIFFNESS_VARIANTS
    for variant in range(NUM_STIFFNESS_VARIANTS):
        g = _solver(db, cfg)
        g.set_stiffness_variant(variant)
        g.set_fields(d, v, np.zeros(n3, np.float32))
        g.forces_only()
        g.forces_only()
        acc = g.fields()[2]
        mem = g.memory_variables() if att else None
        out.append((acc, mem))
        g.close()
    for v in range(1, NUM_STIFFNESS_VARIANTS):
        assert rel_l2(out[v][0], out[0][0]) < 1e-6, v
        if att:
            same = []
            for a, b in zip(out[0][1][0] + out[0][1][1], out[v][1][0] + out[v][1][1]):
                assert rel_l2(b, a) < 1e-6, v
                same.append(float(np.mean(a == b)))
            print(f"variant {v}: fraction of bit-identical memory-variable/strain values:", min(same))


@pytest.fixture(scope="module")
def homog_runs(gpulib):
    from specfem3d_gb300 import configs, meshgen
    from oracle import oracle as O
    cfg = configs.homogeneous_block(nstep=2000)
    db = meshgen.build_database(cfg)
    sim = _oracle_sim(db, cfg)
    sim.step(cfg["nstep"])
    so = O.seismograms(sim)
    db64 = meshgen.build_database(cfg, dtype=np.float64)
    sim64 = _oracle_sim(db64, cfg, "f64")
    sim64.step(cfg["nstep"])
    so64 = O.seismograms(sim64)
    g = _solver(db, cfg)
    g.run_per_call(cfg["nstep"])
    sp = g.seismograms()
    fp = g.fields()
    g.close()
    g2 = _solver(db, cfg)
    g2.run(cfg["nstep"], steps_per_graph=100)
    sf = g2.seismograms()
    ff = g2.fields()
    g2.close()
    return dict(cfg=cfg, db=db, so=so, sim=sim, sp=sp, fp=fp, sf=sf, ff=ff, so64=so64, sim64=sim64)


def test_homogeneous_seismograms_vs_oracle(homog_runs):
    r = homog_runs
    err = rel_l2(r["sp"], r["so"])
    assert err < 5e-5, err
    per_rec = [rel_l2(r["sp"][i], r["so"][i]) for i in range(len(r["so"]))]
    assert max(per_rec) < 1e-4
    ed = rel_l2(r["fp"][0], r["sim"].get("displ"))
    ev = rel_l2(r["fp"][1], r["sim"].get("veloc"))
    print(f"homogeneous_block 2000 steps: seismograms {err:.2e} (max receiver {max(per_rec):.2e}), displ {ed:.2e}, veloc {ev:.2e}")
    assert ed < 3e-4 and ev < 3e-4


def test_homogeneous_accuracy_against_fp64_oracle(homog_runs):
    """The device's FP32 error against the FP64 oracle is no larger than the FP32
    CPU oracle's own (seismograms and final wavefields)."""
    r = homog_runs
    e_gpu = rel_l2(r["sp"], r["so64"])
    e_cpu = rel_l2(r["so"], r["so64"])
    print(f"seismograms vs FP64: device {e_gpu:.2e}, FP32 oracle {e_cpu:.2e}")
    assert e_gpu < 1.5 * e_cpu + 1e-7, (e_gpu, e_cpu)
    assert e_gpu < 1e-4
    for k, name in ((0, "displ"), (1, "veloc")):
        eg = rel_l2(r["fp"][k], r["sim64"].get(name))
        ec = rel_l2(r["sim"].get(name), r["sim64"].get(name))
        print(f"{name} vs FP64: device {eg:.2e}, FP32 oracle {ec:.2e}")
        assert eg < 1.5 * ec + 1e-7, (name, eg, ec)


def test_fused_loop_equals_per_call_abi(homog_runs):
    """The graph-captured fused loop and the per-call ABI loop give the same
    seismograms, and the fused loop's FP32 error against the FP64 oracle is no
    larger than the FP32 CPU oracle's (the wavefields left after the waves
    exit are a tiny residual, so they are compared through that accuracy bound
    rather than against each other)."""
    r = homog_runs
    assert rel_l2(r["sf"], r["sp"]) < 2e-5
    e_cpu = rel_l2(r["so"], r["so64"])
    assert rel_l2(r["sf"], r["so64"]) < 1.5 * e_cpu + 1e-7
    for k, name in ((0, "displ"), (1, "veloc")):
        eg = rel_l2(r["ff"][k], r["sim64"].get(name))
        ec = rel_l2(r["sim"].get(name), r["sim64"].get(name))
        print(f"fused {name} vs FP64: device {eg:.2e}, FP32 oracle {ec:.2e}")
        assert eg < 1.5 * ec + 1e-7, (name, eg, ec)


def test_attenuation_time_stepping_vs_oracle(gpulib):
    from specfem3d_gb300 import configs, meshgen
    from oracle import oracle as O
    cfg = configs.small_layered(nstep=400, attenuation=True)
    db = meshgen.build_database(cfg)
    sim = _oracle_sim(db, cfg)
    sim.step(cfg["nstep"])
    g = _solver(db, cfg)
    g.run(cfg["nstep"], steps_per_graph=50)
    assert rel_l2(g.seismograms(), O.seismograms(sim)) < 5e-5
    d, v, a = g.fields()
    assert rel_l2(d, sim.get("displ")) < 5e-5
    R, E = g.memory_variables()
    for c, name in enumerate(["R_xx", "R_yy", "R_xy", "R_xz", "R_yz", "R_trace"]):
        assert rel_l2(R[c], sim.get(name)) < 1e-4, name
    g.close()


@pytest.mark.parametrize("example", ["refex_stacey5sides", "refex_no_absorbing"])
def test_reference_golden_seismograms_on_gpu(gpulib, example):
    """Full 5000-step reference examples on the GPU against the reference's REF_SEIS:
    relative L2 <= 1e-3 and correlation >= 0.999 per trace.  The source of both
    examples is a vertex of 8 elements; each configuration places it in the element
    its REF_SEIS run chose (logged in that run's output_solver.txt).  The
    no-absorbing run is also held to the FP64 oracle's traces
    (tests/golden/make_oracle_fixture.py) at <= 2e-4 (FP32 after 5000 steps)."""
    from specfem3d_gb300 import configs, meshgen
    stacey = example == "refex_stacey5sides"
    cfg = configs.refex(5000) if stacey else configs.refex_no_absorbing(5000)
    db = meshgen.build_database(cfg)
    g = _solver(db, cfg)
    g.run(cfg["nstep"], steps_per_graph=100)
    seis = g.seismograms()
    g.close()
    ref = np.load(os.path.join(ROOT, "tests", "golden", example + ".npz"))["displ"]
    errs = [rel_l2(seis[r, c], ref[r, c]) for r in range(4) for c in range(3)]
    print(f"{example}: all traces {rel_l2(seis, ref):.2e}, worst trace {max(errs):.2e}")
    for r in range(4):
        for c in range(3):
            assert rel_l2(seis[r, c], ref[r, c]) < 1e-3, (r, c)
            assert np.corrcoef(seis[r, c], ref[r, c])[0, 1] > 0.999
    if not stacey:
        o64 = np.load(os.path.join(ROOT, "tests", "golden", "refex_no_absorbing_oracle_f64.npz"))["displ"]
        e = rel_l2(seis, o64)
        print(f"no-absorbing example vs FP64 oracle: {e:.2e}")
        assert e < 2e-4


def test_attenuation_benchmark_golden_seismograms(gpulib):
    """The reference's viscoelastic attenuation benchmark (80^3 regular elements,
    Q_kappa 10, Q_mu 20, N_SLS = 3, 1300 steps) against its REF_SEIS displacement:
    relative L2 <= 1e-5 per component (measured 1.0e-6: FP32 rounding level),
    correlation >= 0.99999.
    The same run without attenuation differs from REF_SEIS by far more, so the
    match pins the memory-variable path itself."""
    from specfem3d_gb300 import configs, meshgen
    ref = np.load(os.path.join(ROOT, "tests", "golden", "attenuation_benchmark.npz"))["displ"]
    out = {}
    for att in (True, False):
        cfg = configs.attenuation_benchmark(1300)
        cfg["attenuation"] = att
        db = meshgen.build_database(cfg)
        g = _solver(db, cfg)
        g.run(cfg["nstep"], steps_per_graph=100)
        out[att] = g.seismograms()
        g.close()
    for c in range(3):
        e, e0 = rel_l2(out[True][0, c], ref[0, c]), rel_l2(out[False][0, c], ref[0, c])
        cc = np.corrcoef(out[True][0, c], ref[0, c])[0, 1]
        print(f"attenuation benchmark component {'XYZ'[c]}: rel L2 {e:.2e} (elastic run {e0:.2e}), corr {cc:.7f}")
        assert e < 1e-5 and cc > 0.99999
        assert e0 > 1e3 * e


def test_stability_check_and_errors(gpulib):
    from specfem3d_gb300 import abi, configs, meshgen
    cfg = configs.small_layered(nstep=4, attenuation=False)
    db = meshgen.build_database(cfg)
    g = _solver(db, cfg)
    rc, m = g.check_stability()
    assert rc == 0 and m == 0.0
    d = np.zeros(3 * db["nglob"], np.float32)
    d[17] = np.nan
    g.set_fields(d, d * 0, d * 0)
    rc, m = g.check_stability()
    assert rc == 4 and np.isnan(m)
    with pytest.raises(abi.SF3DError, match="unstable"):
        abi.check()
    g.close()
    bad = dict(db)
    bad["ibool"] = db["ibool"].copy()
    bad["ibool"][5] = db["nglob"] + 7
    with pytest.raises(abi.SF3DError, match="ibool"):
        _solver(bad, cfg)


def test_adjoint_kernel_accumulation(gpulib):
    """compute_kernels_elastic_cuda against compute_kernels.f90:151-186 in FP64."""
    import ctypes
    from specfem3d_gb300 import abi, configs, meshgen
    cfg = configs.small_layered(nstep=4, attenuation=False)
    db = meshgen.build_database(cfg)
    g = _solver(db, cfg, simulation_type=3)
    L, A = g.L, abi.Args()
    n3 = 3 * db["nglob"]
    L.prepare_fields_elastic_adj_dev_(g.mp, A.i(n3), *([A.af(None)] * 7), A.i(1), *([A.af(None)] * 10), A.i(0),
                                      A.i(0))
    abi.check()
    rng = np.random.default_rng(5)
    b = rng.standard_normal(n3).astype(np.float32)
    f = rng.standard_normal(n3).astype(np.float32)
    g.set_fields(f, f * 0.5, f * 0.1)                       # adjoint field
    L.transfer_b_fields_to_device_(A.i(n3), A.af(b), A.af(b * 0), A.af(b * 0), g.mp)
    L.compute_strain_cuda_(g.mp, A.i(1))
    L.compute_strain_cuda_(g.mp, A.i(3))
    dt = np.float32(cfg["dt"])
    L.compute_kernels_elastic_cuda_(g.mp, A.f(dt))
    L.compute_kernels_elastic_cuda_(g.mp, A.f(dt))
    abi.check()
    nk = 125 * db["nspec"]
    rho, mu, kap = (np.zeros(nk) for _ in range(3))
    L.sf3d_get_kernels_f64(g.mp, rho.ctypes.data, mu.ctypes.data, kap.ctypes.data)
    abi.check()
    g.close()
    # host evaluation of the same formulas on the oracle's strains of both fields
    from oracle import oracle as O
    sim = O.make_sim(db, cfg, "f64")
    sim.seti("compute_and_store_strain", 1)
    names = ["epsilondev_xx", "epsilondev_yy", "epsilondev_xy", "epsilondev_xz", "epsilondev_yz"]
    strains = {}
    for tag, fld in (("adj", f), ("b", b)):
        for nm in names + ["epsilon_trace_over_3"]:
            sim.set(nm, np.zeros(nk))
        sim.get("displ")[:] = fld.astype(np.float64)
        sim.forces()
        strains[tag] = [sim.get(nm).copy() for nm in names] + [sim.get("epsilon_trace_over_3").copy()]
    e, eb = strains["adj"], strains["b"]
    ib = db["ibool"] - 1
    acc = (f * np.float32(0.1)).astype(np.float64).reshape(-1, 3)
    rho_ref = 2 * float(dt) * (acc[ib] * b.astype(np.float64).reshape(-1, 3)[ib]).sum(1)
    mu_ref = 2 * float(dt) * (e[0] * eb[0] + e[1] * eb[1] + (e[0] + e[1]) * (eb[0] + eb[1])
                              + 2 * (e[2] * eb[2] + e[3] * eb[3] + e[4] * eb[4]))
    kap_ref = 2 * float(dt) * 9 * e[5] * eb[5]
    assert rel_l2(rho, rho_ref) < 1e-6
    assert rel_l2(mu, mu_ref) < 1e-5
    assert rel_l2(kap, kap_ref) < 1e-5


def test_analytic_elastic_golden_seismograms(gpulib):
    """The reference's analytic_solution_elastic benchmark (16^3 elements, Stacey on
    all six faces, double couple at a vertex, 14000 steps) against its REF_SEIS
    (every 10th sample): relative L2 <= 1e-3 and correlation >= 0.9999 per trace
    (measured: worst trace 2.1e-4).  The Aki & Richards solution it ships is printed for scale only (it is the
    continuous problem, not the discrete one)."""
    from specfem3d_gb300 import configs, meshgen
    cfg = configs.analytic_elastic(14000)
    db = meshgen.build_database(cfg)
    g = _solver(db, cfg)
    g.run(cfg["nstep"], steps_per_graph=100)
    seis = g.seismograms()[:, :, ::10]
    g.close()
    gold = np.load(os.path.join(ROOT, "tests", "golden", "analytic_elastic.npz"))
    ref, ana = gold["displ"], gold["analytic"]
    errs = []
    for r in range(6):
        for c in range(3):
            if np.abs(ref[r, c]).max() < 1e-3 * np.abs(ref).max():
                continue                     # a nodal component of the double couple
            e = rel_l2(seis[r, c], ref[r, c])
            cc = np.corrcoef(seis[r, c], ref[r, c])[0, 1]
            errs.append(e)
            assert e < 1e-3 and cc > 0.9999, (r, c, e, cc)
    print(f"analytic benchmark vs REF_SEIS: worst trace {max(errs):.2e}; vs the analytic solution "
          f"{rel_l2(seis, ana):.2e} (REF_SEIS itself {rel_l2(ref, ana):.2e})")


def test_anisotropic_and_hessian_kernel_accumulation(gpulib):
    """ANISOTROPIC_KL (21 strain products, compute_kernels.f90:566-618) and
    APPROXIMATE_HESS_KL (hess, hess_rho, hess_kappa, hess_mu, :513-545) against the
    formulas evaluated in FP64 on the oracle's strains of both fields."""
    from specfem3d_gb300 import abi, configs, meshgen
    from oracle import oracle as O
    cfg = configs.small_layered(nstep=4, attenuation=False)
    db = meshgen.build_database(cfg)
    g = _solver(db, cfg, simulation_type=3)
    L, A = g.L, abi.Args()
    n3 = 3 * db["nglob"]
    L.prepare_fields_elastic_adj_dev_(g.mp, A.i(n3), *([A.af(None)] * 7), A.i(1), *([A.af(None)] * 10), A.i(1),
                                      A.i(1))
    abi.check()
    rng = np.random.default_rng(8)
    f = rng.standard_normal(n3).astype(np.float32)
    b = rng.standard_normal(n3).astype(np.float32)
    bv = rng.standard_normal(n3).astype(np.float32)
    ba = rng.standard_normal(n3).astype(np.float32)
    g.set_fields(f, f * 0.5, f * 0.1)
    L.transfer_b_fields_to_device_(A.i(n3), A.af(b), A.af(bv), A.af(ba), g.mp)
    L.compute_strain_cuda_(g.mp, A.i(1))
    L.compute_strain_cuda_(g.mp, A.i(3))
    dt = np.float32(cfg["dt"])
    L.compute_kernels_elastic_cuda_(g.mp, A.f(dt))
    L.compute_kernels_hess_cuda_(g.mp, A.f(dt), A.i(1), A.i(0))
    abi.check()
    nspec = db["nspec"]
    nk = 125 * nspec
    cij = np.zeros(21 * nk)
    hess = np.zeros(4 * nk)
    assert L.sf3d_get_extra_kernels_f64(g.mp, cij.ctypes.data, hess.ctypes.data) == 0
    h32 = [np.zeros(nk, np.float32) for _ in range(4)]
    L.transfer_kernels_hess_el_tohost_(g.mp, *(h.ctypes.data for h in h32), A.i(nspec))
    abi.check()
    for q in range(4):
        assert np.allclose(h32[q], hess[q * nk:(q + 1) * nk].astype(np.float32))
    g.close()
    sim = O.make_sim(db, cfg, "f64")
    sim.seti("compute_and_store_strain", 1)
    names = ["epsilondev_xx", "epsilondev_yy", "epsilondev_xy", "epsilondev_xz", "epsilondev_yz"]
    strains = {}
    for tag, fld in (("adj", f), ("b", b)):
        for nm in names + ["epsilon_trace_over_3"]:
            sim.set(nm, np.zeros(nk))
        sim.get("displ")[:] = fld.astype(np.float64)
        sim.forces()
        strains[tag] = [sim.get(nm).copy() for nm in names] + [sim.get("epsilon_trace_over_3").copy()]

    def voigt(s):
        e11, e22 = s[0] + s[5], s[1] + s[5]
        return [e11, e22, -(e11 + e22) + 3 * s[5], s[4], s[3], s[2]]

    ea, eb = voigt(strains["adj"]), voigt(strains["b"])
    ref = []
    for i in range(6):
        for j in range(i, 6):
            v = ea[i] * eb[j]
            if j > i:
                v = v + ea[j] * eb[i]
                if j > 2 and i < 3:
                    v = v * 2
            if i > 2:
                v = v * 4
            ref.append(float(dt) * v)
    ref = np.stack(ref, axis=1).reshape(-1)
    assert rel_l2(cij, ref) < 1e-5
    ib = db["ibool"] - 1
    acc = (f * np.float32(0.1)).astype(np.float64).reshape(-1, 3)[ib]
    e = strains["b"]
    href = [float(dt) * (acc * ba.astype(np.float64).reshape(-1, 3)[ib]).sum(1),
            float(dt) * (bv.astype(np.float64).reshape(-1, 3)[ib] ** 2).sum(1),
            float(dt) * 9 * e[5] * e[5],
            float(dt) * (e[0] * e[0] + e[1] * e[1] + (e[0] + e[1]) ** 2 + 2 * (e[2] ** 2 + e[3] ** 2 + e[4] ** 2))]
    for q in range(4):
        assert rel_l2(hess[q * nk:(q + 1) * nk], href[q]) < 1e-5, q
