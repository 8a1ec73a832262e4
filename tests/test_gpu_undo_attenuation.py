"""SIMULATION_TYPE = 3 under UNDO_ATTENUATION_AND_OR_PML (iterate_time_undoatt.F90)
on the GPU, through the reference-named entry points: snapshots of the forward
run every nt_dump steps, the backward field recomputed forward in time from each
snapshot (transfer_b_fields_to_device, transfer_b_rmemory_to_device,
compute_strain_cuda, compute_stacey_viscoelastic_undoatt_cuda, the backward
sources at forward time), buffered and replayed in reverse beside the adjoint
field, with the strain of the replayed b_displ recomputed in
compute_kernels_elastic_cuda.

* the recomputed backward displacement equals the forward run's displacement at
  every step (the restart from a snapshot of displ, veloc, accel and the memory
  variables continues the forward trajectory);
* the kernels equal those accumulated against the forward run's own stored
  displacement history;
* without attenuation they equal the kernels of the time-reversed
  reconstruction (SAVE_FORWARD boundary record), which match the discrete
  adjoint of the Newmark step.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

NT_DUMP = 70


def _history(db, cfg):
    """Displacement after every step of a plain forward run, keyed by step number."""
    from specfem3d_gb300.solver import GPUSolver
    g = GPUSolver(db, cfg, nlength=cfg["nstep"])
    H = {}
    for s in range(1, cfg["nstep"] + 1):
        g.run_per_call(1)
        H[s] = g.fields()[0]
    g.close()
    return H


def _kernels_from_history(db, cfg, adj, H):
    """The adjoint field of the kernel run paired with the stored forward
    displacement of step NSTEP - it + 1 at adjoint step it."""
    from specfem3d_gb300 import abi, adjoint as ADJ
    from specfem3d_gb300.solver import GPUSolver
    nstep = cfg["nstep"]
    g = GPUSolver(db, cfg, nlength=nstep, simulation_type=3, undo_attenuation=True)
    ADJ._prepare_adjoint(g, db, nstep)
    L, n3 = g.L, 3 * g.nglob
    src = np.ascontiguousarray(np.asarray(adj, np.float32).transpose(2, 0, 1))
    dt = np.float32(cfg["dt"])
    dt2, dtsq2 = np.float32(dt / np.float32(2)), np.float32(dt * dt / np.float32(2))
    for it in range(1, nstep + 1):
        S = abi.Args()
        one = S.i(1)
        L.transfer_b_displ_to_device_(S.i(n3), S.af(H[nstep - it + 1]), g.mp)
        L.update_displacement_cuda_(g.mp, S.f(dt), S.f(dt2), S.f(dtsq2), one)
        for iphase in (1, 2):
            L.compute_forces_viscoelastic_cuda_(g.mp, S.i(iphase), S.f(dt), S.i(g.nspec_outer),
                                                S.i(g.nspec_elastic), one, S.i(g.attenuation), one)
            if iphase == 1:
                L.compute_stacey_viscoelastic_cuda_(g.mp, one, None, one)
                if it < nstep:
                    L.add_sources_el_sim_type_2_or_3_(g.mp, S.af(src), S.i(g.nrec), S.i(g.nrec), S.i(nstep),
                                                      S.i(it))
        L.kernel_3_a_cuda_(g.mp, S.f(dt2), S.f(dt2), S.i(0), one)
        L.compute_kernels_elastic_cuda_(g.mp, S.f(dt))
    abi.check()
    return ADJ._kernels_f64(g)


@pytest.mark.parametrize("att", [False, True])
def test_undo_attenuation_kernels(gpulib, att):
    from specfem3d_gb300 import adjoint as ADJ, configs, meshgen
    cfg = configs.small_layered(nstep=300, attenuation=att)
    db = meshgen.build_database(cfg)
    assert int(db.get("stacey", 1)) and int(db["num_abs_boundary_faces"]) > 0
    seis, snaps = ADJ.undo_attenuation_forward(db, cfg, NT_DUMP)
    assert len(snaps) == 5  # 4 x 70 + 20 steps
    H = _history(db, cfg)
    assert seis.shape[2] == cfg["nstep"] and np.abs(seis).max() > 0
    # adjoint source: the L2 misfit against zero data (the synthetics themselves)
    adj = seis.astype(np.float64)
    hist = []
    kl = ADJ.undo_attenuation_kernel_run(db, cfg, adj, snaps, NT_DUMP, history=hist)
    assert sorted(s for s, _ in hist) == list(range(1, cfg["nstep"] + 1))
    # relative to the largest displacement of the run (the first steps are near zero)
    scale = max(np.linalg.norm(h) for h in H.values())
    worst = max(np.linalg.norm(d.astype(np.float64) - H[s]) for s, d in hist) / scale
    ref = _kernels_from_history(db, cfg, adj, H)
    errs = {k: rel_l2(kl[k], ref[k]) for k in ("rho", "mu", "kappa")}
    print(f"undo attenuation (att={att}): recomputed b_displ vs forward worst {worst:.2e}; kernels vs stored "
          f"history " + ", ".join(f"{k} {e:.2e}" for k, e in errs.items()))
    # atomics reorder the assembly sums from run to run, and with attenuation the
    # restart recomputes the strain of the snapshot (the forward run kept it from
    # the stiffness pass): measured b_displ 3.7e-7 (elastic) and 5.3e-6
    # (attenuation); kernels 1e-7 to 4.4e-6 and 1.2e-5 to 3.0e-5
    assert worst < (2e-5 if att else 2e-6)
    for k in ("rho", "mu", "kappa"):
        assert np.abs(ref[k]).max() > 0
        assert errs[k] < (1e-4 if att else 2e-5), k
    if not att:
        s1, final, rec = ADJ.forward_with_boundary_record(db, cfg)
        tr = ADJ.kernel_run(db, cfg, adj, final, rec)
        e = {k: rel_l2(kl[k], tr[k]) for k in ("rho", "mu", "kappa")}
        print("undo attenuation vs time-reversed reconstruction: " + ", ".join(f"{k} {v:.2e}" for k, v in e.items()))
        # measured: rho 9.1e-6, mu 2.1e-7, kappa 3.2e-7
        assert all(v < 1e-4 for v in e.values())
