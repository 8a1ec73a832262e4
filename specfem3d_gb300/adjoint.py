"""Sensitivity kernels the reference's way: SIMULATION_TYPE = 3 through the
reference-named entry points.

The reference computes rho / mu / kappa kernels with two runs (iterate_time.F90:
219-330): a forward run with SAVE_FORWARD that keeps the final wavefield and the
Stacey boundary record (compute_stacey_viscoelastic.F90), then a kernel run that
advances the adjoint field, driven by time-reversed adjoint sources at the
receivers (compute_add_sources_viscoelastic.F90:182-254), together with the
forward field reconstructed backwards in time (b_deltat = -DT, the boundary
record replayed in reverse, the sources at (NSTEP - it) DT - t0; the backward
field is replaced by the saved final state after the first step,
read_forward_arrays), accumulating at every step
rho_kl += dt a_adj . b_u, mu_kl += dt eps_adj : b_eps, kappa_kl += 9 dt tr tr
(compute_kernels.f90:67-226), scaled at the end to K_rho = -rho rho_kl,
K_mu = -2 mu mu_kl, K_kappa = -kappa kappa_kl (save_adjoint_kernels.f90:325-343).

This module drives exactly that sequence on the device, for elastic meshes
without attenuation.  It is the reference's method, kept beside the
checkpointed discrete adjoint of :mod:`gradient` so the two can be compared.
"""
from __future__ import annotations

import numpy as np

from . import abi
from .meshgen import NGLL3, WGLL
from .solver import GPUSolver


def forward_with_boundary_record(db: dict, cfg: dict):
    """SIMULATION_TYPE = 1 with SAVE_FORWARD: (seismograms (nrec, 3, nstep), final
    (displ, veloc, accel), boundary record (nstep, 75 nfaces) or None)."""
    cfg = dict(cfg)
    cfg["record"] = ("displ",)
    nstep = int(cfg["nstep"])
    g = GPUSolver(db, cfg, nlength=nstep, save_forward=True)
    nf = int(db["num_abs_boundary_faces"]) if int(db.get("stacey", 0)) else 0
    rec = np.zeros((nstep, 75 * nf), np.float32) if nf else None
    g.absorb_record = rec
    g.run_per_call(nstep)
    seis = g.seismograms()
    final = g.fields()
    g.close()
    return seis, final, rec


def kernel_run(db: dict, cfg: dict, adjoint_source: np.ndarray, final_fields, absorb_record):
    """The SIMULATION_TYPE = 3 run: adjoint_source (nrec, 3, nstep) are the adjoint
    traces in forward time as the reference reads them from SEM/*.adj (for the L2
    waveform misfit: synthetics minus data).  Returns the raw FP64 accumulators
    rho_kl, mu_kl, kappa_kl, each (nspec, 125)."""
    if int(db.get("attenuation", 0)):
        raise ValueError("kernel_run: the time-reversed reconstruction is for meshes without attenuation")
    nstep = int(cfg["nstep"])
    g = GPUSolver(db, cfg, nlength=nstep, simulation_type=3)
    L, A = g.L, abi.Args()
    n3 = 3 * g.nglob
    # prepare_fields_elastic_adj_dev: backward fields and kernel accumulators
    L.prepare_fields_elastic_adj_dev_(g.mp, A.i(n3), *([A.af(None)] * 7), A.i(1), *([A.af(None)] * 10),
                                      A.i(0), A.i(0))
    abi.check()
    nrec = g.nrec
    # prepare_sim2_or_3_const_device: every receiver of this slice carries an adjoint source
    L.prepare_sim2_or_3_const_device_(g.mp, A.i(nrec), A.i(nstep), A.af(db["hxir"]), A.af(db["hetar"]),
                                      A.af(db["hgammar"]), A.i(nrec), A.ai(np.zeros(nrec, np.int32)),
                                      A.ai(db["ispec_selected_rec"]))
    abi.check()
    # source_adjoint(NDIM, nadj_rec_local, NTSTEP_BETWEEN_READ_ADJSRC), one block of nstep samples
    src = np.ascontiguousarray(np.asarray(adjoint_source, np.float32).transpose(2, 0, 1))
    stf = np.asarray(db["stf"], np.float64).reshape(g.nsources, -1)
    dt = np.float32(cfg["dt"])
    dt2, dtsq2 = np.float32(dt / np.float32(2)), np.float32(dt * dt / np.float32(2))
    bdt, bdt2 = np.float32(-dt), np.float32(-dt / np.float32(2))
    one, three, zero = A.i(1), A.i(3), A.i(0)
    d_fin, v_fin, a_fin = (np.ascontiguousarray(f, np.float32) for f in final_fields)
    for it in range(1, nstep + 1):
        B = abi.Args()
        L.update_displacement_cuda_(g.mp, B.f(dt), B.f(dt2), B.f(dtsq2), one)
        L.update_displacement_cuda_(g.mp, B.f(bdt), B.f(bdt2), B.f(dtsq2), three)
        # adjoint field (compute_forces_viscoelastic_calling)
        for iphase in (1, 2):
            L.compute_forces_viscoelastic_cuda_(g.mp, B.i(iphase), B.f(dt), B.i(g.nspec_outer),
                                                B.i(g.nspec_elastic), one, zero, one)
            if iphase == 1:
                L.compute_stacey_viscoelastic_cuda_(g.mp, one, None, one)
                if it < nstep:
                    L.add_sources_el_sim_type_2_or_3_(g.mp, B.af(src), B.i(nrec), B.i(nrec), B.i(nstep), B.i(it))
        L.kernel_3_a_cuda_(g.mp, B.f(dt2), B.f(bdt2), zero, one)
        # backward field (compute_forces_viscoelastic_backward_calling)
        for iphase in (1, 2):
            L.compute_forces_viscoelastic_cuda_(g.mp, B.i(iphase), B.f(bdt), B.i(g.nspec_outer),
                                                B.i(g.nspec_elastic), one, zero, three)
            if iphase == 1:
                rec = B.af(absorb_record[nstep - it]) if absorb_record is not None else None
                L.compute_stacey_viscoelastic_cuda_(g.mp, one, rec, three)
                if g.nsources:
                    L.compute_add_sources_el_s3_cuda_(g.mp, B.ad(np.ascontiguousarray(stf[:, nstep - it])),
                                                      B.i(g.nsources))
        L.kernel_3_a_cuda_(g.mp, B.f(dt2), B.f(bdt2), zero, three)
        if it == 1:
            # read_forward_arrays: the backward field starts from the saved final state
            L.transfer_b_fields_to_device_(B.i(n3), B.af(d_fin), B.af(v_fin), B.af(a_fin), g.mp)
        L.compute_kernels_elastic_cuda_(g.mp, B.f(dt))
    abi.check()
    n = g.nspec
    out = {k: np.zeros(n * NGLL3) for k in ("rho", "mu", "kappa")}
    L.sf3d_get_kernels_f64(g.mp, out["rho"].ctypes.data, out["mu"].ctypes.data, out["kappa"].ctypes.data)
    abi.check()
    g.close()
    return {k: v.reshape(n, NGLL3) for k, v in out.items()}


def scaled_kernels(db: dict, kl: dict) -> dict:
    """save_adjoint_kernels.f90:325-343: K_rho = -rho rho_kl, K_mu = -2 mu mu_kl,
    K_kappa = -kappa kappa_kl (densities per unit volume)."""
    n = int(db["nspec"])

    def m(name):
        return np.asarray(db[name], np.float64).reshape(n, NGLL3)

    return {"rho": -m("rhostore") * kl["rho"], "mu": -2.0 * m("mustore") * kl["mu"],
            "kappa": -m("kappastore") * kl["kappa"]}


def gradient_as_kernel_density(db: dict, grad: dict) -> dict:
    """Per-point dJ/dm of the discrete adjoint (nspec, 125) turned into the reference's
    kernel density: K_m = m dJ/dm / (w_i w_j w_k J) at each element point."""
    n = int(db["nspec"])
    irr = np.asarray(db["irregular_element_number"])
    jac = np.empty((n, NGLL3))
    reg = irr == 0
    jac[reg] = float(np.float32(db["jacobian_regular"]))
    if (~reg).any():
        jac[~reg] = np.asarray(db["jacobian"], np.float64).reshape(-1, NGLL3)[irr[~reg] - 1]
    w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1)
    vol = jac * w3[None, :]
    store = {"rho": "rhostore", "kappa": "kappastore", "mu": "mustore"}
    return {k: grad[k] * np.asarray(db[store[k]], np.float64).reshape(n, NGLL3) / vol for k in ("rho", "kappa", "mu")}
