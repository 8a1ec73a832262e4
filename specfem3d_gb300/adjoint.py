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
from .solver import N_SLS
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
    L = g.L
    n3 = 3 * g.nglob
    _prepare_adjoint(g, db, nstep)
    nrec = g.nrec
    # source_adjoint(NDIM, nadj_rec_local, NTSTEP_BETWEEN_READ_ADJSRC), one block of nstep samples
    src = np.ascontiguousarray(np.asarray(adjoint_source, np.float32).transpose(2, 0, 1))
    stf = np.asarray(db["stf"], np.float64).reshape(g.nsources, -1)
    dt = np.float32(cfg["dt"])
    dt2, dtsq2 = np.float32(dt / np.float32(2)), np.float32(dt * dt / np.float32(2))
    bdt, bdt2 = np.float32(-dt), np.float32(-dt / np.float32(2))
    A = abi.Args()
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
    return _kernels_f64(g)


def forward_with_boundary_record_coupled(db: dict, cfg: dict):
    """SIMULATION_TYPE = 1 with SAVE_FORWARD on a fluid-solid mesh: (seismograms,
    final elastic (displ, veloc, accel), final potentials (chi, chi_dot, chi_dot_dot),
    elastic boundary record (nstep, 75 nfaces), acoustic boundary record
    b_absorb_potential (nstep, 25 nfaces)); records are None without Stacey faces."""
    cfg = dict(cfg)
    nstep = int(cfg["nstep"])
    g = GPUSolver(db, cfg, nlength=nstep, save_forward=True)
    nf = int(db["num_abs_boundary_faces"]) if int(db.get("stacey", 0)) else 0
    g.absorb_record = np.zeros((nstep, 75 * nf), np.float32) if nf else None
    g.absorb_record_ac = np.zeros((nstep, 25 * nf), np.float32) if nf else None
    g.run_per_call(nstep)
    out = (g.seismograms(), g.fields(), g.potentials(), g.absorb_record, g.absorb_record_ac)
    g.close()
    return out


def kernel_run_coupled(db: dict, cfg: dict, adjoint_source: np.ndarray, final_el, final_ac, rec_el, rec_ac,
                       history=None, discrete_fluid_kernels: bool = False, hessian: bool = False):
    """The SIMULATION_TYPE = 3 run on a fluid-solid mesh (iterate_time.F90:219-330):
    per step the adjoint potentials and displacement (compute_forces_acoustic_
    forward_calling, then compute_forces_viscoelastic_calling: Stacey, coupling with
    the adjoint sign, adjoint sources of the receivers of each domain), then the
    backward potentials and displacement with b_deltat = -DT (the two boundary
    records replayed in reverse, coupling on the b_ fields, the sources at
    (NSTEP - it) DT - t0), both backward fields replaced by the saved final state
    after the first step, and the elastic and acoustic kernels accumulated.
    discrete_fluid_kernels: pair chi_adj_dd instead of chi_adj in the fluid kernels
    (sf3d_set_acoustic_kernel_pairing), which gives the discrete derivative.
    history: optional list receiving, after each step, a dict with the adjoint
    potential and its second derivative (chi, chi_dd) and the backward ones
    (b_chi, b_chi_dot, b_chi_dd).  hessian: APPROXIMATE_HESS_KL in the fluid
    (hess_ac, hess_rho_ac, hess_kappa_ac in the result, FP32 as
    transfer_kernels_hess_ac_tohost returns them).
    Returns the raw FP64 accumulators rho, mu, kappa (solid) and rho_ac, kappa_ac
    (fluid), each (nspec, 125)."""
    if int(db.get("attenuation", 0)):
        raise ValueError("kernel_run_coupled: the time-reversed reconstruction is for meshes without attenuation")
    if not np.asarray(db.get("ispec_is_acoustic", [0])).any():
        raise ValueError("kernel_run_coupled: the mesh has no fluid elements (use kernel_run)")
    nstep = int(cfg["nstep"])
    g = GPUSolver(db, cfg, nlength=nstep, simulation_type=3)
    L = g.L
    n3, n1 = 3 * g.nglob, g.nglob
    _prepare_adjoint(g, db, nstep)
    A = abi.Args()
    L.prepare_fields_acoustic_adj_dev_(g.mp, A.i(int(bool(hessian))))
    abi.check()
    if L.sf3d_set_acoustic_kernel_pairing(g.mp, int(bool(discrete_fluid_kernels))) != 0:
        abi.check()
    nrec = g.nrec
    src = np.ascontiguousarray(np.asarray(adjoint_source, np.float32).transpose(2, 0, 1))
    stf = np.asarray(db["stf"], np.float64).reshape(g.nsources, -1)
    dt = np.float32(cfg["dt"])
    dt2, dtsq2 = np.float32(dt / np.float32(2)), np.float32(dt * dt / np.float32(2))
    bdt, bdt2 = np.float32(-dt), np.float32(-dt / np.float32(2))
    fin_el = [np.ascontiguousarray(f, np.float32) for f in final_el]
    fin_ac = [np.ascontiguousarray(f, np.float32) for f in final_ac]
    nac = g.nspec_acoustic
    for it in range(1, nstep + 1):
        B = abi.Args()
        one, three, zero = B.i(1), B.i(3), B.i(0)
        L.update_displacement_cuda_(g.mp, B.f(dt), B.f(dt2), B.f(dtsq2), one)
        L.update_displacement_ac_cuda_(g.mp, B.f(dt), B.f(dt2), B.f(dtsq2), one)
        L.update_displacement_cuda_(g.mp, B.f(bdt), B.f(bdt2), B.f(dtsq2), three)
        L.update_displacement_ac_cuda_(g.mp, B.f(bdt), B.f(bdt2), B.f(dtsq2), three)
        for fa, d, d2 in ((one, dt, dt2), (three, bdt, bdt2)):
            backward = fa is three
            # acoustic domain (compute_forces_acoustic_forward/backward_calling)
            L.acoustic_enforce_free_surf_cuda_(g.mp, zero, fa)
            for iphase in (1, 2):
                L.compute_forces_acoustic_cuda_(g.mp, B.i(iphase), zero, B.i(nac), fa)
                if iphase == 1:
                    rec = B.af(rec_ac[nstep - it]) if (backward and rec_ac is not None) else None
                    L.compute_stacey_acoustic_cuda_(g.mp, one, rec, fa)
                    L.compute_coupling_ac_el_cuda_(g.mp, one, B.i(g.ncoupling), fa)
                    if backward:
                        if g.nsources:
                            L.compute_add_sources_ac_s3_cuda_(g.mp, B.i(g.nsources),
                                                              B.ad(np.ascontiguousarray(stf[:, nstep - it])), one)
                    elif it < nstep:
                        L.add_sources_ac_sim_2_or_3_cuda_(g.mp, B.af(src), B.i(nrec), B.i(nrec), B.i(nstep), B.i(it))
            L.kernel_3_acoustic_cuda_(g.mp, B.f(dt2), B.f(bdt2), fa)
            L.acoustic_enforce_free_surf_cuda_(g.mp, zero, fa)
            # elastic domain (compute_forces_viscoelastic_calling / _backward_calling)
            for iphase in (1, 2):
                L.compute_forces_viscoelastic_cuda_(g.mp, B.i(iphase), B.f(d), B.i(g.nspec_outer),
                                                    B.i(g.nspec_elastic), one, zero, fa)
                if iphase == 1:
                    rec = B.af(rec_el[nstep - it]) if (backward and rec_el is not None) else None
                    L.compute_stacey_viscoelastic_cuda_(g.mp, one, rec, fa)
                    L.compute_coupling_el_ac_cuda_(g.mp, one, B.i(g.ncoupling), fa)
                    if backward:
                        if g.nsources:
                            L.compute_add_sources_el_s3_cuda_(g.mp, B.ad(np.ascontiguousarray(stf[:, nstep - it])),
                                                              B.i(g.nsources))
                    elif it < nstep:
                        L.add_sources_el_sim_type_2_or_3_(g.mp, B.af(src), B.i(nrec), B.i(nrec), B.i(nstep), B.i(it))
            L.kernel_3_a_cuda_(g.mp, B.f(dt2), B.f(bdt2), zero, fa)
        if it == 1:
            # read_forward_arrays: both backward fields start from the saved final state
            L.transfer_b_fields_to_device_(B.i(n3), *(B.af(f) for f in fin_el), g.mp)
            L.transfer_b_fields_ac_to_device_(B.i(n1), *(B.af(f) for f in fin_ac), g.mp)
        L.compute_kernels_elastic_cuda_(g.mp, B.f(dt))
        L.compute_kernels_acoustic_cuda_(g.mp, B.f(dt))
        if hessian:
            # APPROXIMATE_HESS_KL in the fluid only (ELASTIC_SIMULATION = 0 here)
            L.compute_kernels_hess_cuda_(g.mp, B.f(dt), zero, one)
        if history is not None:
            h = {k: np.zeros(n1, np.float32) for k in ("chi", "chi_dd", "b_chi", "b_chi_dot", "b_chi_dd")}
            L.transfer_fields_ac_from_device_(B.i(n1), h["chi"].ctypes.data, None, h["chi_dd"].ctypes.data, g.mp)
            L.transfer_b_fields_ac_from_device_(B.i(n1), h["b_chi"].ctypes.data, h["b_chi_dot"].ctypes.data,
                                                h["b_chi_dd"].ctypes.data, g.mp)
            h["it"] = it
            history.append(h)
    abi.check()
    n = g.nspec
    ac = {k: np.zeros(n * NGLL3) for k in ("rho_ac", "kappa_ac")}
    if L.sf3d_get_kernels_ac_f64(g.mp, ac["rho_ac"].ctypes.data, ac["kappa_ac"].ctypes.data) != 0:
        abi.check()
    if hessian:
        hs = [np.zeros(n * NGLL3, np.float32) for _ in range(3)]
        L.transfer_kernels_hess_ac_tohost_(g.mp, *(x.ctypes.data for x in hs), B.i(n))
        abi.check()
        ac.update({k: x.reshape(n, NGLL3) for k, x in zip(("hess_ac", "hess_rho_ac", "hess_kappa_ac"), hs)})
    out = _kernels_f64(g)
    out.update({k: v.reshape(n, NGLL3) for k, v in ac.items()})
    return out


def _prepare_adjoint(g: GPUSolver, db: dict, nstep: int):
    """prepare_fields_elastic_adj_dev (backward fields, kernel accumulators and, with
    attenuation, the backward memory variables with the forward-time coefficients
    of an undo-attenuation run) and prepare_sim2_or_3_const_device (every receiver
    of this slice carries an adjoint source)."""
    L, A = g.L, abi.Args()
    n3 = 3 * g.nglob
    att = g.attenuation
    nsls = N_SLS * NGLL3 * g.nspec
    zsls = np.zeros(nsls, np.float32) if att else None
    zeps = np.zeros(NGLL3 * g.nspec, np.float32) if att else None
    coef = [A.af(db.get(n) if att else None) for n in ("alphaval", "betaval", "gammaval")]
    L.prepare_fields_elastic_adj_dev_(g.mp, A.i(n3), *([A.af(None)] * 7), A.i(nsls if att else 1),
                                      *(A.af(zsls) for _ in range(6)), A.af(zeps), *coef, A.i(0), A.i(0))
    abi.check()
    nrec = g.nrec
    L.prepare_sim2_or_3_const_device_(g.mp, A.i(nrec), A.i(nstep), A.af(db["hxir"]), A.af(db["hetar"]),
                                      A.af(db["hgammar"]), A.i(nrec), A.ai(np.zeros(nrec, np.int32)),
                                      A.ai(db["ispec_selected_rec"]))
    abi.check()


def _kernels_f64(g: GPUSolver) -> dict:
    n = g.nspec
    out = {k: np.zeros(n * NGLL3) for k in ("rho", "mu", "kappa")}
    g.L.sf3d_get_kernels_f64(g.mp, out["rho"].ctypes.data, out["mu"].ctypes.data, out["kappa"].ctypes.data)
    abi.check()
    g.close()
    return {k: v.reshape(n, NGLL3) for k, v in out.items()}


# ------------------------------------------------------------------ undo attenuation
def undo_attenuation_forward(db: dict, cfg: dict, nt_dump: int):
    """SIMULATION_TYPE = 1 with SAVE_FORWARD and UNDO_ATTENUATION_AND_OR_PML
    (iterate_time_undoatt.F90:280-395): before each subset of nt_dump steps the
    wavefield and, with attenuation, the memory variables are saved
    (save_forward_arrays_undoatt: displ, veloc, accel, R_xx..R_yz, R_trace).
    Returns (seismograms (nrec, 3, nstep), snapshots); snapshot s holds the state
    after s * nt_dump steps."""
    cfg = dict(cfg)
    cfg["record"] = ("displ",)
    nstep = int(cfg["nstep"])
    nsub = -(-nstep // int(nt_dump))
    g = GPUSolver(db, cfg, nlength=nstep, save_forward=True, undo_attenuation=True)
    snaps = []
    for s in range(nsub):
        d, v, a = g.fields()
        R = g.memory_variables()[0] if g.attenuation else None
        snaps.append({"displ": d, "veloc": v, "accel": a, "R": R})
        g.run_per_call(min(int(nt_dump), nstep - s * int(nt_dump)))
    seis = g.seismograms()
    g.close()
    return seis, snaps


def undo_attenuation_kernel_run(db: dict, cfg: dict, adjoint_source: np.ndarray, snapshots, nt_dump: int,
                                history=None):
    """SIMULATION_TYPE = 3 under UNDO_ATTENUATION_AND_OR_PML
    (iterate_time_undoatt.F90:396-570), for meshes with or without attenuation.
    Subsets are visited from the last forward one to the first: the snapshot is
    restored (read_forward_arrays_undoatt: transfer_b_fields_to_device,
    transfer_b_rmemory_to_device) and its strain recomputed
    (compute_strain_cuda, FORWARD_OR_ADJOINT = 3); the backward field is stepped
    forward in time over the subset (b_deltat = +DT, Stacey from b_veloc through
    compute_stacey_viscoelastic_undoatt_cuda, the sources at the forward time
    of compute_add_sources_viscoelastic.F90:743-809) and each b_displ buffered
    (transfer_b_displ_from_device); then the adjoint field advances through the
    subset while b_displ is restored from the buffer in reverse order
    (transfer_b_displ_to_device) and the kernels accumulate (the strain of the
    restored b_displ is recomputed inside compute_kernels_elastic_cuda).
    history: optional list that receives the recomputed b_displ of every forward
    step, keyed by the forward step number.  Returns the raw FP64 accumulators
    rho_kl, mu_kl, kappa_kl, each (nspec, 125)."""
    nstep, nt = int(cfg["nstep"]), int(nt_dump)
    nsub = len(snapshots)
    if nsub != -(-nstep // nt):
        raise ValueError("undo_attenuation_kernel_run: one snapshot per subset of nt_dump steps is needed")
    g = GPUSolver(db, cfg, nlength=nstep, simulation_type=3, undo_attenuation=True)
    L = g.L
    n3 = 3 * g.nglob
    _prepare_adjoint(g, db, nstep)
    nrec = g.nrec
    src = np.ascontiguousarray(np.asarray(adjoint_source, np.float32).transpose(2, 0, 1))
    stf = np.asarray(db["stf"], np.float64).reshape(g.nsources, -1)
    dt = np.float32(cfg["dt"])
    dt2, dtsq2 = np.float32(dt / np.float32(2)), np.float32(dt * dt / np.float32(2))
    att = g.attenuation
    nsls = N_SLS * NGLL3 * g.nspec
    it = 0
    for iteration_on_subset in range(1, nsub + 1):
        B = abi.Args()
        one, three = B.i(1), B.i(3)
        snap = snapshots[nsub - iteration_on_subset]
        L.transfer_b_fields_to_device_(B.i(n3), *(B.af(snap[k]) for k in ("displ", "veloc", "accel")), g.mp)
        if att:
            L.transfer_b_rmemory_to_device_(g.mp, *(B.af(r) for r in snap["R"]), B.i(nsls))
        L.compute_strain_cuda_(g.mp, three)
        abi.check()
        it_subset_end = nstep - (nsub - 1) * nt if iteration_on_subset == 1 else nt
        first = (nsub - iteration_on_subset) * nt  # forward steps before this subset
        buf = np.zeros((it_subset_end, n3), np.float32)
        for k in range(1, it_subset_end + 1):
            S = abi.Args()
            L.update_displacement_cuda_(g.mp, S.f(dt), S.f(dt2), S.f(dtsq2), three)
            for iphase in (1, 2):
                L.compute_forces_viscoelastic_cuda_(g.mp, S.i(iphase), S.f(dt), S.i(g.nspec_outer),
                                                    S.i(g.nspec_elastic), one, S.i(att), three)
                if iphase == 1:
                    L.compute_stacey_viscoelastic_undoatt_cuda_(g.mp, one, three)
                    if g.nsources:
                        # it_tmp = NSTEP - first - k + 1: the stf sample of forward step first + k
                        L.compute_add_sources_el_s3_cuda_(g.mp, S.ad(np.ascontiguousarray(stf[:, first + k - 1])),
                                                          S.i(g.nsources))
            L.kernel_3_a_cuda_(g.mp, S.f(dt2), S.f(dt2), S.i(0), three)
            L.transfer_b_displ_from_device_(S.i(n3), buf[k - 1].ctypes.data, g.mp)
            if history is not None:
                history.append((first + k, buf[k - 1].copy()))
        abi.check()
        # compute_strain_att: strain of the current adjoint field
        L.compute_strain_cuda_(g.mp, one)
        for k in range(1, it_subset_end + 1):
            S = abi.Args()
            it += 1
            L.transfer_b_displ_to_device_(S.i(n3), S.af(buf[it_subset_end - k]), g.mp)
            L.update_displacement_cuda_(g.mp, S.f(dt), S.f(dt2), S.f(dtsq2), one)
            for iphase in (1, 2):
                L.compute_forces_viscoelastic_cuda_(g.mp, S.i(iphase), S.f(dt), S.i(g.nspec_outer),
                                                    S.i(g.nspec_elastic), one, S.i(att), one)
                if iphase == 1:
                    L.compute_stacey_viscoelastic_cuda_(g.mp, one, None, one)
                    if it < nstep:
                        L.add_sources_el_sim_type_2_or_3_(g.mp, S.af(src), S.i(nrec), S.i(nrec), S.i(nstep), S.i(it))
            L.kernel_3_a_cuda_(g.mp, S.f(dt2), S.f(dt2), S.i(0), one)
            L.compute_kernels_elastic_cuda_(g.mp, S.f(dt))
        abi.check()
    return _kernels_f64(g)


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
