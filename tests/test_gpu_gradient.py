"""Checkpointed discrete-adjoint misfit gradient on the GPU.

* the directional derivative from the adjoint sweep matches central finite
  differences of the misfit (FP64 oracle forward runs, eps = 3e-5) along
  five seeded smooth random directions of (dln rho, dln kappa, dln mu) to <= 1e-3
  relative;
* the gradient does not depend on the checkpoint spacing (recomputation is the
  same arithmetic; atomics reorder sums and the kappa terms cancel strongly, so
  <= 5e-5 relative; measured 1e-6 to 1.2e-5);
* the torch.autograd wrapper returns the gradient of a direct call (<= 1e-4:
  two separate device runs).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem(gpulib):
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from misfit_autograd import Problem
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=500, nshots=2, n=10)
    db_true = meshgen.build_database(cfg, material=G.true_material(cfg))
    observed = []
    for i in range(len(cfg["shots"])):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db_true, cfg, i), c, nlength=cfg["nstep"])
        s.run(cfg["nstep"], steps_per_graph=50)
        observed.append(s.seismograms())
        s.close()
    db0 = meshgen.build_database(cfg, material=G.background_material(cfg))
    return Problem(cfg, db0, observed, cfg["checkpoint_every"])


def _gradient(problem, every):
    from specfem3d_gb300 import gradient as G
    return G.misfit_gradient(lambda i: G.shot_database(problem.db, problem.cfg, i), problem.cfg,
                             problem.observed, every)


def test_gradient_matches_finite_differences(problem):
    """Central differences of the misfit computed by the FP64 oracle with
    eps = 3e-5: no FP32 rounding noise, and a truncation error below 1e-6
    (the waveform misfit is strongly non-linear in wave speed: at eps = 1e-3 the
    O(eps^2) term alone is 6e-4 relative).  The device's own FP32 forward runs
    (eps = 1e-3) give the same derivative to their noise and truncation (checked
    at 2e-2)."""
    from specfem3d_gb300 import gradient as G, meshgen
    from misfit_autograd import misfit_value, oracle_misfit
    J0, grad, timing = _gradient(problem, problem.every)
    assert J0 > 0
    db64 = meshgen.build_database(problem.cfg, material=G.background_material(problem.cfg), dtype=np.float64)
    for seed in (101, 202, 303, 404, 505):
        d = [G.smooth_direction(problem.cfg, seed + q, corr_len=800.0) for q in range(3)]
        gd = sum(float(np.sum(grad[k] * problem.stores[k] * dq))
                 for k, dq in zip(("rho", "kappa", "mu"), d))
        e64 = 3e-5
        fd = (oracle_misfit(problem, db64, *(e64 * dq for dq in d)) -
              oracle_misfit(problem, db64, *(-e64 * dq for dq in d))) / (2 * e64)
        eps = 1e-3
        rel = abs(gd - fd) / abs(fd)
        fd32 = (misfit_value(problem, *(eps * dq for dq in d)) - misfit_value(problem, *(-eps * dq for dq in d))) / (2 * eps)
        rel32 = abs(gd - fd32) / abs(fd32)
        print(f"direction {seed}: adjoint {gd:.9e}  FD (FP64 oracle) {fd:.9e} rel {rel:.2e}  "
              f"FD (device FP32) {fd32:.9e} rel {rel32:.2e}")
        assert rel < 1e-3, (seed, gd, fd)
        assert rel32 < 2e-2, (seed, gd, fd32)


def test_gradient_independent_of_checkpoint_spacing(problem):
    _, g1, _ = _gradient(problem, problem.every)
    _, g2, _ = _gradient(problem, int(problem.cfg["nstep"]))
    for k in ("rho", "kappa", "mu"):
        assert rel_l2(g1[k], g2[k]) < 5e-5, k


def test_autograd_wrapper(problem):
    torch = pytest.importorskip("torch")
    from specfem3d_gb300 import gradient as G
    from misfit_autograd import WaveformMisfit
    n = int(problem.db["nspec"])
    z = [torch.zeros((n, 125), dtype=torch.float64, requires_grad=True) for _ in range(3)]
    J = WaveformMisfit.apply(*z, problem)
    J.backward()
    _, grad, _ = _gradient(problem, problem.every)
    for t, k in zip(z, ("rho", "kappa", "mu")):
        # two device runs: atomics reorder the FP32 sums
        assert rel_l2(t.grad.numpy(), grad[k] * problem.stores[k]) < 1e-4


def test_fused_and_separate_adjoint_kernels_agree(problem):
    """K p and the gradient terms in one kernel per element (default) give the
    gradient of the stiffness kernel followed by the separate gradient kernel."""
    from specfem3d_gb300 import gradient as G
    _, g1, t1 = G.misfit_gradient(lambda i: G.shot_database(problem.db, problem.cfg, i), problem.cfg,
                                  problem.observed, problem.every, fused=True)
    _, g2, t2 = G.misfit_gradient(lambda i: G.shot_database(problem.db, problem.cfg, i), problem.cfg,
                                  problem.observed, problem.every, fused=False)
    for k in ("rho", "kappa", "mu"):
        assert rel_l2(g1[k], g2[k]) < 5e-5, k


def test_gradient_matches_reference_style_kernels(problem):
    """The checkpointed discrete adjoint against the reference's own method for the
    same shot: SIMULATION_TYPE = 3 through the reference's entry points (forward
    with SAVE_FORWARD and the Stacey record, then adjoint + time-reversed
    reconstruction + kernel accumulation; specfem3d_gb300.adjoint).  Both give
    rho / mu / kappa kernel densities.  With the reference's timing (adjoint sample
    NSTEP - it + 1, backward field replaced after the first step) its accumulation
    is the discrete adjoint of the Newmark step, so the two agree to FP32 rounding:
    <= 1e-4 relative L2 (measured 1.7e-6 to 2.5e-6)."""
    from specfem3d_gb300 import adjoint as ADJ, gradient as G
    cfg, db = problem.cfg, problem.db
    c0 = G.shot_config(cfg, 0)
    db0 = G.shot_database(db, cfg, 0)
    mg = G.MisfitGradient(db0, c0, cfg["checkpoint_every"])
    seis = mg.forward()
    _, res = G.misfit(seis, problem.observed[0], mg.dt)
    grad = mg.gradient(res)
    mg.close()
    ours = ADJ.gradient_as_kernel_density(db0, grad)
    s1, final, rec = ADJ.forward_with_boundary_record(db0, c0)
    assert rel_l2(s1, seis) < 1e-5
    kl = ADJ.kernel_run(db0, c0, s1.astype(np.float64) - problem.observed[0], final, rec)
    ref = ADJ.scaled_kernels(db0, kl)
    for k in ("rho", "mu", "kappa"):
        e = rel_l2(ours[k], ref[k])
        cc = np.corrcoef(ours[k].ravel(), ref[k].ravel())[0, 1]
        print(f"{k}: discrete adjoint vs SIMULATION_TYPE=3 kernels: rel L2 {e:.3e}, correlation {cc:.6f}")
        assert np.abs(ref[k]).max() > 0
        assert e < 1e-4 and cc > 0.99999


def test_set_sources_equals_a_fresh_solver(problem):
    """sf3d_set_sources: a solver prepared for shot 0 and given shot 1's sources
    records shot 1's traces as a solver prepared for shot 1 does (same build;
    atomics reorder sums, which over 200 steps gives ~2e-6: <= 1e-5), and returns
    to shot 0's traces after the sources are set back."""
    from specfem3d_gb300 import gradient as G
    from specfem3d_gb300.solver import GPUSolver
    cfg, db0 = problem.cfg, problem.db
    nstep = 200
    dbs = [G.shot_database(db0, cfg, i) for i in range(2)]
    cfgs = []
    for i in range(2):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        c["nstep"] = nstep
        cfgs.append(c)
    ref = []
    for i in range(2):
        s = GPUSolver(dbs[i], cfgs[i], nlength=nstep)
        s.run(nstep, steps_per_graph=50)
        ref.append(s.seismograms())
        s.close()
    assert rel_l2(ref[1], ref[0]) > 1e-2      # the shots differ
    s = GPUSolver(dbs[0], cfgs[0], nlength=nstep)
    for i in (1, 0):
        s.set_sources(dbs[i])
        s.reset()
        s.run(nstep, steps_per_graph=50)
        assert rel_l2(s.seismograms(), ref[i]) < 1e-5, i
    s.close()
