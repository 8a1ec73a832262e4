"""torch.autograd.Function around the checkpointed discrete-adjoint C ABI (test
harness only): the waveform misfit as a function of relative model
perturbations (dln rho, dln kappa, dln mu per GLL point), with the device
adjoint sweep as its backward."""
import numpy as np
import torch

from specfem3d_gb300 import gradient as G


class Problem:
    """Mesh, background model, shots and observed traces of a misfit."""

    def __init__(self, cfg, db_background, observed, checkpoint_every):
        self.cfg, self.db, self.observed, self.every = cfg, db_background, observed, checkpoint_every
        n = int(db_background["nspec"])
        self.stores = {k: db_background[s].reshape(n, -1).astype(np.float64)
                       for k, s in (("rho", "rhostore"), ("kappa", "kappastore"), ("mu", "mustore"))}


class WaveformMisfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, dln_rho, dln_kappa, dln_mu, problem):
        db = G.perturbed_database(problem.db, problem.cfg, dln_rho.detach().numpy(), dln_kappa.detach().numpy(),
                                  dln_mu.detach().numpy())
        J, grad, _ = G.misfit_gradient(lambda i: G.shot_database(db, problem.cfg, i), problem.cfg,
                                       problem.observed, problem.every)
        # m = m0 (1 + dln)  =>  dJ/d(dln) = m0 dJ/dm
        ctx.save_for_backward(*(torch.from_numpy(grad[k] * problem.stores[k]) for k in ("rho", "kappa", "mu")))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gr, gk, gm = ctx.saved_tensors
        return gJ * gr, gJ * gk, gJ * gm, None


def misfit_value(problem, dln_rho, dln_kappa, dln_mu):
    """Misfit of the perturbed model from plain graph-captured forward runs."""
    from specfem3d_gb300.solver import GPUSolver
    db = G.perturbed_database(problem.db, problem.cfg, dln_rho, dln_kappa, dln_mu)
    total = 0.0
    for i, obs in enumerate(problem.observed):
        cfg = G.shot_config(problem.cfg, i)
        cfg["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db, problem.cfg, i), cfg, nlength=int(cfg["nstep"]))
        s.run(int(cfg["nstep"]), steps_per_graph=50)
        J, _ = G.misfit(s.seismograms(), obs, float(s.deltat))
        s.close()
        total += J
    return total


def oracle_misfit(problem, db64, dln_rho, dln_kappa, dln_mu):
    """Misfit of the perturbed model from the FP64 CPU oracle (no FP32 rounding
    noise in the finite differences)."""
    import os
    from oracle import oracle as O
    db = G.perturbed_database(db64, problem.cfg, dln_rho, dln_kappa, dln_mu)
    total = 0.0
    for i, obs in enumerate(problem.observed):
        cfg = G.shot_config(problem.cfg, i)
        sim = O.make_sim(G.shot_database(db, problem.cfg, i), cfg, "f64", nthreads=os.cpu_count() or 1)
        sim.step(int(cfg["nstep"]))
        J, _ = G.misfit(O.seismograms(sim), obs, float(cfg["dt"]))
        total += J
    return total
