"""GPU parity of the fluid-solid path: fluid stiffness, Sommerfeld faces,
coupling terms, pressure source and hydrophones, through the per-call C ABI in
the reference's call order, against the oracle's coupled step (FP32 both)."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_coupled_fluid_solid_vs_oracle(gpulib):
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.small_coupled(nstep=300)
    db = meshgen.build_database(cfg)
    assert db["num_coupling_ac_el_faces"] > 0 and db["ispec_is_acoustic"].sum() > 0
    sim = O.make_coupled_sim(db, cfg, "f32", nthreads=os.cpu_count() or 1)
    O.run_coupled(sim, cfg["nstep"])
    ref = O.seismograms(sim)
    g = solver.GPUSolver(db, cfg)
    g.run_per_call(cfg["nstep"])
    seis = g.seismograms()
    p, pd, pdd = g.potentials()
    d, v, a = g.fields()
    g.close()
    e_p = rel_l2(seis[:, 0], ref[:, 0])
    e_chi = rel_l2(p, sim.get("potential"))
    e_u = rel_l2(d, sim.get("displ"))
    print(f"coupled 300 steps: pressure {e_p:.2e}, potential {e_chi:.2e}, solid displacement {e_u:.2e}")
    assert np.abs(ref[:, 0]).max() > 0 and np.abs(sim.get("displ")).max() > 0
    assert e_p < 5e-5 and e_chi < 5e-5 and e_u < 1e-4


def test_coupled_fused_loop_equals_per_call(gpulib):
    """sf3d_iterate_time with the fluid domain fused into the graph-captured step
    gives the per-call path's hydrophone traces and fields within the tolerance
    the per-call path itself meets against the oracle (5e-5; measured 1.2e-5:
    atomics reorder sums and the fused corrector/predictor rounds differently)."""
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.small_coupled(nstep=300)
    db = meshgen.build_database(cfg)
    g = solver.GPUSolver(db, cfg)
    g.run_per_call(cfg["nstep"])
    s1, p1, d1 = g.seismograms(), g.potentials()[0], g.fields()[0]
    g.close()
    g = solver.GPUSolver(db, cfg)
    g.run(cfg["nstep"], steps_per_graph=50)
    s2, p2, d2 = g.seismograms(), g.potentials()[0], g.fields()[0]
    g.close()
    assert np.abs(s1[:, 0]).max() > 0
    assert rel_l2(s2[:, 0], s1[:, 0]) < 5e-5
    assert rel_l2(p2, p1) < 5e-5 and rel_l2(d2, d1) < 5e-5
    # the fused loop advances the solid fields over the solid elements' span of
    # points and the potentials over the fluid elements' span: outside its own
    # elements each field stays exactly zero, as in the per-call path
    ib = np.asarray(db["ibool"]).reshape(db["nspec"], -1) - 1
    isac = np.asarray(db["ispec_is_acoustic"]).astype(bool)
    fluid_only = np.setdiff1d(np.unique(ib[isac]), np.unique(ib[~isac]))
    solid_only = np.setdiff1d(np.unique(ib[~isac]), np.unique(ib[isac]))
    assert len(fluid_only) > 0 and len(solid_only) > 0
    assert not np.any(p1[solid_only]) and not np.any(p2[solid_only])
    d1p, d2p = d1.reshape(-1, 3), d2.reshape(-1, 3)
    assert not np.any(d1p[fluid_only]) and not np.any(d2p[fluid_only])


def test_fluid_receiver_vector_seismograms_vs_oracle(gpulib):
    """Receivers in fluid elements record (1/rho) grad of chi, chi_dot and
    chi_dot_dot as displacement, velocity and acceleration (the reference's
    compute_gradient_in_acoustic path), solid receivers their fields: per-call
    GPU traces against the oracle's, 300 steps, <= 5e-5 relative L2 per kind."""
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.small_coupled(nstep=300)
    cfg["record"] = ("displ", "veloc", "accel")
    zf = cfg["zlev"][len(cfg["zlev"]) - 3]
    cfg["receivers"] = cfg["receivers"] + [(cfg["x1"] * 0.45, cfg["y1"] * 0.55, zf - 120.0)]   # one in the solid
    db = meshgen.build_database(cfg)
    isac = db["ispec_is_acoustic"].astype(bool)
    in_fluid = isac[db["ispec_selected_rec"] - 1]
    assert in_fluid[:3].all() and not in_fluid[3]
    g = solver.GPUSolver(db, cfg)
    g.run_per_call(cfg["nstep"])
    got = {k: g.seismograms(k) for k in ("displ", "veloc", "accel")}
    g.close()
    for code, k in ((1, "displ"), (2, "veloc"), (3, "accel")):
        sim = O.make_coupled_sim(db, cfg, "f32", nthreads=os.cpu_count() or 1)
        sim.seti("fluid_vector", 1)
        sim.seti("record_what", code)
        O.run_coupled(sim, cfg["nstep"])
        ref = O.seismograms(sim)
        e = rel_l2(got[k], ref)
        ef = rel_l2(got[k][:3], ref[:3])
        print(f"{k}: all receivers {e:.2e}, fluid receivers {ef:.2e}")
        assert np.abs(ref[:3]).max() > 0 and np.abs(ref[3]).max() > 0
        assert e < 5e-5 and ef < 5e-5


def test_waterlayered_reference_golden_seismograms(gpulib):
    """The reference example waterlayered_halfspace (4500 steps, 40500 elements,
    explosion in the water) against its REF_SEIS vertical traces: displacement at
    the 9 X10..X90 stations (in the water, 100 m deep) and velocity at all 22
    (water, solid, and 0.1-0.2 m either side of the sea floor).  Per trace:
    relative L2 <= 1e-3 and correlation >= 0.99999 (measured: <= 2.5e-4, the
    worst at the stations 0.1 m above the sea floor)."""
    from conftest import ROOT
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.waterlayered(4500)
    db = meshgen.build_database(cfg)
    g = solver.GPUSolver(db, cfg)
    g.run_per_call(cfg["nstep"])
    got = {k: g.seismograms(k) for k in ("displ", "veloc")}
    g.close()
    ref = np.load(os.path.join(ROOT, "tests", "golden", "waterlayered.npz"))
    names = list(cfg["station_names"])
    worst = {}
    for k in ("displ", "veloc"):
        for n, tr in zip(ref[k + "_stations"], ref[k]):
            r = names.index(str(n))
            e = rel_l2(got[k][r, 2], tr)
            c = np.corrcoef(got[k][r, 2], tr)[0, 1]
            worst[(k, str(n))] = (e, c)
    for (k, n), (e, c) in sorted(worst.items(), key=lambda t: -t[1][0])[:8]:
        print(f"waterlayered {k} {n}: rel L2 {e:.2e}, correlation {c:.6f}")
    for (k, n), (e, c) in worst.items():
        assert e < 1e-3 and c > 0.99999, (k, n, e, c)


@pytest.mark.parametrize("per_call", [False, True])
def test_acoustic_reference_golden_pressure(gpulib, per_call):
    """The reference's homogeneous_acoustic example (its 36x36x16 block filled with
    one fluid, Stacey faces on five sides, free surface, an explosion with a
    Gaussian time function, four hydrophones 50 m deep, 1000 steps) against its
    REF_SEIS pressure traces (tests/golden/refex_acoustic.npz): relative L2 <= 1e-2
    per trace, the tolerance of the reference's own comparison
    (utils/scripts/compare_seismogram_correlations.py: TOL_ERR = 0.01), and
    correlation >= 0.9999.  Measured 5.7e-3, correlation 0.999996: the device and
    the oracle both differ from that 2016 run by one constant amplitude factor of
    1.005 on every trace (the fluid source, its Gaussian width and the waterlayered
    example's traces agree with the reference to 2.5e-4 and better)."""
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.refex_acoustic(1000)
    db = meshgen.build_database(cfg)
    assert int(db["ispec_is_acoustic"].sum()) == db["nspec"]
    g = solver.GPUSolver(db, cfg)
    if per_call:
        g.run_per_call(cfg["nstep"])
    else:
        g.run(cfg["nstep"], steps_per_graph=100)
    p = g.seismograms()[:, 0]
    g.close()
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "refex_acoustic.npz"))["pressure"]
    errs = [rel_l2(p[r], ref[r]) for r in range(4)]
    print(f"acoustic example: pressure traces {rel_l2(p, ref):.2e}, worst {max(errs):.2e}")
    for r in range(4):
        assert errs[r] < 1e-2, (r, errs[r])
        assert np.corrcoef(p[r], ref[r])[0, 1] > 0.9999
