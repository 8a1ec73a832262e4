"""Host driver of the GPU time step: the caller side of the C ABI.

``GPUSolver`` does what the Fortran solver does around the reference's GPU
layer: it hands the mesh databases to prepare_constants_device and
prepare_fields_elastic_device (specfem3D/prepare_gpu.f90:67-165), then either
replays the per-step call sequence of iterate_time
(specfem3D/iterate_time.F90:219-330 with
compute_forces_viscoelastic_calling_routine.F90:107-417) through the same entry
points, or runs whole step blocks on the device with sf3d_iterate_time.
Everything below goes through libspecfem3d_gb300.so; nothing is computed on
the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi

NGLL3 = 125
N_SLS = 3
NUM_STIFFNESS_VARIANTS = 17       # sf3d_set_stiffness_variant accepts 0 .. 16


# the 21 anisotropic moduli per GLL point, in the order prepare_fields_elastic_device takes them
ANISO_NAMES = ["c11store", "c12store", "c13store", "c14store", "c15store", "c16store", "c22store", "c23store",
               "c24store", "c25store", "c26store", "c33store", "c34store", "c35store", "c36store", "c44store",
               "c45store", "c46store", "c55store", "c56store", "c66store"]


class GPUSolver:
    def __init__(self, db: dict, cfg: dict, nlength: int | None = None, simulation_type: int = 1,
                 save_forward: bool = False, record=("displ",), colors=None, tile: int = 0,
                 undo_attenuation: bool = False):
        """colors: optional colour per element (no two elements of a colour share a
        point, e.g. meshgen.block_colors); the phase lists are then ordered colour by
        colour and USE_MESH_COLORING_GPU is set, so assembly runs without atomics.
        undo_attenuation: UNDO_ATTENUATION_AND_OR_PML of prepare_constants_device (the
        kernel accumulation then recomputes the backward strain from b_displ)."""
        self.colors = None if colors is None else np.asarray(colors, np.int32)
        # tile > 0: phase lists in tiles of tile^3 elements of a block mesh, so that
        # elements sharing points are processed close in time (L2 reuse of the
        # gathered wavefield)
        self.tile = int(tile)
        self.L = abi.load()
        self.db, self.cfg = db, cfg
        self.nspec, self.nglob = int(db["nspec"]), int(db["nglob"])
        self.nstep = int(cfg["nstep"])
        self.nlength = int(nlength or self.nstep)
        self.nrec = int(db["nrec"])
        self.nsources = int(db["nsources"])
        self.attenuation = int(db.get("attenuation", 0))
        self.simulation_type = simulation_type
        dt = np.float32(cfg["dt"])
        self.deltat = dt
        self.deltatover2 = np.float32(dt / np.float32(2))
        self.deltatsqover2 = np.float32(dt * dt / np.float32(2))
        self.mesh = ctypes.c_long(0)
        self.mp = ctypes.addressof(self.mesh)
        self.record = tuple(cfg.get("record", record))
        self.isac = np.asarray(db.get("ispec_is_acoustic", np.zeros(self.nspec, np.int32)), np.int32)
        self.coupled = bool(self.isac.any())
        self.absorb_record = None
        self.absorb_record_ac = None
        self.undo_attenuation = bool(undo_attenuation)
        self._prepare_constants(db, save_forward)
        self._prepare_fields(db)
        self.pml = bool(db.get("pml", 0))
        if self.pml:
            self._prepare_pml(db)
        if self.coupled:
            self._prepare_acoustic(db)
        self.it = 1

    # ------------------------------------------------------------------ setup
    def _prepare_constants(self, db, save_forward):
        A = abi.Args()
        # MPI interfaces of a slice: ibool_interfaces (max_nibool, num_interfaces), 1-based
        self.num_interfaces = int(db.get("num_interfaces", 0))
        self.max_nibool = int(db.get("max_nibool_interfaces", 0))
        nspec, nirr = self.nspec, int(db["nspec_irregular"])
        nrec = self.nrec
        nu = np.tile(np.eye(3).reshape(-1, order="F"), max(nrec, 1))
        hx = np.asarray(db["hxir"], np.float32)
        he = np.asarray(db["hetar"], np.float32)
        hg = np.asarray(db["hgammar"], np.float32)
        args = [
            self.mp, A.i(5), A.i(nspec), A.i(self.nglob), A.i(nirr), A.ai(db["irregular_element_number"]),
            *(A.af(db[n]) for n in ("xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz")),
            A.f(db["xix_regular"]), A.f(db["jacobian_regular"]), A.ai(db["ibool"]),
            A.i(self.num_interfaces), A.i(self.max_nibool), A.ai(db.get("nibool_interfaces")),
            A.ai(db.get("ibool_interfaces")),
            A.af(db["hprime_xx"]), A.af(db["hprimewgll_xx"]), A.af(db["wgllwgll_xy"]), A.af(db["wgllwgll_xz"]),
            A.af(db["wgllwgll_yz"]),
            A.i(int(db.get("stacey", 1))), A.ai(db["abs_boundary_ispec"]), A.ai(db["abs_boundary_ijk"]),
            A.af(db["abs_boundary_normal"]), A.af(db["abs_boundary_jacobian2Dw"]),
            A.i(int(db["num_abs_boundary_faces"]) if (db.get("stacey", 1) or db.get("pml", 0)) else 0),
            A.ai(np.ones(nspec, np.int32)), A.i(self.nsources), A.i(self.nsources), A.af(db["sourcearrays"]),
            A.ai(np.zeros(max(self.nsources, 1), np.int32)), A.ai(db["ispec_selected_source"]),
            A.ai(db["ispec_selected_rec"]), A.i(nrec), A.i(nrec), A.i(self.simulation_type),
            A.i(int(self.colors is not None)),
            A.i(int(self.isac.sum())), A.i(int(nspec - self.isac.sum())), A.ai(self.isac), A.ai(1 - self.isac),
            A.i(0), A.i(int(save_forward)), A.af(hx), A.af(he), A.af(hg), A.ad(nu), A.ad(nu),
            A.ai(np.zeros(max(nrec, 1), np.int32)), A.i(self.nlength),
            A.i(int("displ" in self.record)), A.i(int("veloc" in self.record)), A.i(int("accel" in self.record)),
            A.i(int("pressure" in self.record)), A.i(1), A.i(0), A.i(int(self.undo_attenuation)), A.i(0),
        ]
        self.L.prepare_constants_device_(*args)
        abi.check()

    def _prepare_pml(self, db):
        """prepare_fields_elastic_pml (prepare_gpu.f90): the C-PML layers of a database
        from specfem3d_gb300.pml.setup."""
        from .meshgen import WGLL
        A = abi.Args()
        n = len(db["cpml_to_spec"])
        s2c = np.zeros(self.nspec, np.int32)
        s2c[np.asarray(db["cpml_to_spec"]) - 1] = np.arange(1, n + 1, dtype=np.int32)
        w3 = (WGLL[None, None, :] * WGLL[None, :, None] * WGLL[:, None, None]).reshape(-1).astype(np.float32)
        self.nspec_cpml = n
        self.L.prepare_fields_elastic_pml_(self.mp, A.i(n), A.ai(db["is_cpml"]), A.ai(db["cpml_to_spec"]),
                                           A.ai(s2c), *(A.af(np.asarray(db["pml_coef_" + k]).reshape(-1))
                                                        for k in ("alpha", "beta", "abar", "strain")),
                                           A.af(w3), A.af(db["rhostore"]))
        abi.check()

    def pml_displ(self):
        """(PML_displ_old, PML_displ_new), each (3, 125, nspec_cpml) Fortran order."""
        A = abi.Args()
        n = 3 * 125 * self.nspec_cpml
        o, w = np.zeros(n, np.float32), np.zeros(n, np.float32)
        self.L.transfer_pml_displ_from_device_(A.i(n), o.ctypes.data, w.ctypes.data, self.mp)
        abi.check()
        return o, w

    def _prepare_fields(self, db):
        A = abi.Args()
        nspec = self.nspec
        # phase_ispec_inner_elastic: outer elements (touching an MPI interface) in
        # column 1, inner elements in column 2 (1-based)
        solid = np.nonzero(self.isac == 0)[0] + 1
        outer = np.asarray(db.get("phase_outer", np.zeros(0, np.int32)), np.int32)
        inner = np.setdiff1d(solid, outer).astype(np.int32)
        if self.tile > 0:
            from .meshgen import Block
            B = Block(self.cfg)
            T = self.tile
            for lst in (outer, inner):
                ex, ey, ez = B.elem_xyz(lst - 1)
                key = np.lexsort((ex % T, ey % T, ez % T, ex // T, ey // T, ez // T))
                lst[:] = lst[key]
        ncol_out = ncol_in = 0
        elem_colors = None
        if self.colors is not None:
            # get_perm_color order: outer elements colour by colour, then inner ones
            counts = []
            for lst in (outer, inner):
                c = self.colors[lst - 1]
                order = np.argsort(c, kind="stable")
                lst[:] = lst[order]
                u, n = np.unique(c, return_counts=True)
                counts.append(n.astype(np.int32))
            ncol_out, ncol_in = len(counts[0]), len(counts[1])
            elem_colors = np.concatenate(counts).astype(np.int32)
        self.nspec_outer, self.nspec_elastic = len(outer), len(inner)
        phase = np.zeros((max(len(outer), len(inner), 1), 2), np.int32)
        phase[:len(outer), 0] = outer
        phase[:len(inner), 1] = inner
        att = self.attenuation
        strain = int(att or self.simulation_type == 3)
        aniso = int(db.get("anisotropy", 0))
        zsls = np.zeros(N_SLS * NGLL3 * nspec, np.float32) if att else None
        zeps = np.zeros(NGLL3 * nspec, np.float32) if strain else None
        args = [
            self.mp, A.af(db["rmassx"]), A.af(db["rmassy"]), A.af(db["rmassz"]), A.af(db["rho_vp"]),
            A.af(db["rho_vs"]), A.af(db["kappastore"]), A.af(db["mustore"]), A.i(phase.shape[0]),
            A.ai(phase.reshape(-1, order="F")), A.af(None), A.i(0), A.i(strain),
            *(A.af(zeps) for _ in range(5)), A.i(att), A.i(N_SLS * NGLL3 * nspec if att else 1),
            *(A.af(zsls) for _ in range(5)), A.af(db.get("factor_common") if att else None),
            A.af(zsls), A.af(zeps), A.af(db.get("factor_common_kappa") if att else None),
            A.af(db.get("alphaval", np.zeros(3))), A.af(db.get("betaval", np.zeros(3))),
            A.af(db.get("gammaval", np.zeros(3))), A.i(0), A.af(None), A.i(0), A.af(None), A.ai(None), A.ai(None),
            A.i(0), A.i(0), A.i(ncol_out), A.i(ncol_in), A.ai(elem_colors), A.i(aniso),
            *(A.af(db[n] if aniso else None) for n in ANISO_NAMES),
        ]
        self.L.prepare_fields_elastic_device_(*args)
        abi.check()
        self.strain = strain
        if self.nsources:
            stf = np.ascontiguousarray(np.asarray(db["stf"], np.float64).reshape(self.nsources, -1).T)
            if self.L.sf3d_set_stf_table(self.mp, stf.ctypes.data, self.nsources, stf.shape[0]) != 0:
                abi.check()

    def set_sources(self, db: dict):
        """Replace the sources by those of ``db`` (another shot on the same mesh and
        model: its sourcearrays, ispec_selected_source, stf): sf3d_set_sources."""
        ns = int(db["nsources"])
        sa = np.ascontiguousarray(np.asarray(db["sourcearrays"], np.float32).reshape(-1))
        isp = np.ascontiguousarray(np.asarray(db["ispec_selected_source"], np.int32).reshape(-1))
        stf = np.ascontiguousarray(np.asarray(db["stf"], np.float64).reshape(ns, -1).T)
        if self.L.sf3d_set_sources(self.mp, ns, isp.ctypes.data, sa.ctypes.data, stf.ctypes.data, stf.shape[0]) != 0:
            abi.check()
        self.db = dict(self.db)
        for k in ("sourcearrays", "ispec_selected_source", "stf", "nsources"):
            self.db[k] = db[k]
        self.nsources = ns

    def _prepare_acoustic(self, db):
        """prepare_fields_acoustic_device (specfem3D/prepare_gpu.f90:170-200)."""
        A = abi.Args()
        fluid = np.nonzero(self.isac)[0] + 1
        self.nspec_acoustic = len(fluid)
        phase = np.zeros((len(fluid), 2), np.int32)
        phase[:, 1] = fluid
        nfs = int(db["num_free_surface_faces"])
        ncp = int(db["num_coupling_ac_el_faces"])
        self.ncoupling = ncp
        self.L.prepare_fields_acoustic_device_(
            self.mp, A.af(db["rmass_acoustic"]), A.af(db["rhostore"]), A.af(db["kappastore"]), A.i(len(fluid)),
            A.ai(phase.reshape(-1, order="F")), A.i(0), A.i(nfs), A.ai(db["free_surface_ispec"]),
            A.ai(db["free_surface_ijk"]), A.i(0), A.af(None), A.i(1), A.i(ncp), A.ai(db["coupling_ac_el_ispec"]),
            A.ai(db["coupling_ac_el_ijk"]), A.af(db["coupling_ac_el_normal"]),
            A.af(db["coupling_ac_el_jacobian2Dw"]), A.i(0), A.i(0), A.ai(None))
        abi.check()

    # ---------------------------------------------------------- one step (ABI)
    def _stf_now(self, it):
        return np.ascontiguousarray(np.asarray(self.db["stf"], np.float64).reshape(self.nsources, -1)[:, it - 1])

    def _acoustic_step(self, A, it):
        """compute_forces_acoustic_forward_calling (compute_forces_acoustic_calling_routine.f90:54-343)."""
        L, one = self.L, A.i(1)
        L.acoustic_enforce_free_surf_cuda_(self.mp, A.i(0), one)
        for iphase in (1, 2):
            L.compute_forces_acoustic_cuda_(self.mp, A.i(iphase), A.i(0), A.i(self.nspec_acoustic), one)
            if iphase == 1:
                # SAVE_FORWARD runs hand a (nstep, 25*nfaces) float32 array here to
                # receive b_absorb_potential; otherwise NULL
                rec = self.absorb_record_ac
                L.compute_stacey_acoustic_cuda_(self.mp, A.i(1), A.af(rec[it - 1]) if rec is not None else None,
                                                one)
                L.compute_coupling_ac_el_cuda_(self.mp, A.i(1), A.i(self.ncoupling), one)
                if self.nsources:
                    L.compute_add_sources_ac_cuda_(self.mp, A.i(self.nsources), A.ad(self._stf_now(it)), A.i(1))
        L.kernel_3_acoustic_cuda_(self.mp, A.f(self.deltatover2), A.f(0.0), one)
        L.acoustic_enforce_free_surf_cuda_(self.mp, A.i(0), one)

    def step(self):
        """One time step through the per-call entry points, in the reference's order."""
        self.step_predict()
        self.step_forces(1)
        self.step_forces(2)
        self.step_finish()

    # the pieces of a step, for drivers that exchange MPI interface buffers
    # between the outer (iphase 1) and inner (iphase 2) element passes
    def step_predict(self):
        L, A, it = self.L, abi.Args(), self.it
        one = A.i(1)
        L.update_displacement_cuda_(self.mp, A.f(self.deltat), A.f(self.deltatover2), A.f(self.deltatsqover2), one)
        if self.coupled:
            L.update_displacement_ac_cuda_(self.mp, A.f(self.deltat), A.f(self.deltatover2),
                                           A.f(self.deltatsqover2), one)
            self._acoustic_step(A, it)

    def step_forces(self, iphase: int):
        """compute_forces_viscoelastic_calling (compute_forces_viscoelastic_calling_routine.F90:107-160)."""
        L, A, it = self.L, abi.Args(), self.it
        one = A.i(1)
        L.compute_forces_viscoelastic_cuda_(self.mp, A.i(iphase), A.f(self.deltat), A.i(self.nspec_outer),
                                            A.i(self.nspec_elastic), A.i(self.strain), A.i(self.attenuation), one)
        if iphase == 1:
            # SAVE_FORWARD runs hand a (nstep, 3*25*nfaces) float32 array here to
            # receive the boundary record; otherwise b_absorb_field is NULL
            rec = self.absorb_record
            buf = A.af(rec[it - 1]) if rec is not None else None
            L.compute_stacey_viscoelastic_cuda_(self.mp, A.i(1), buf, one)
            if self.coupled:
                L.compute_coupling_el_ac_cuda_(self.mp, A.i(1), A.i(self.ncoupling), one)
            if self.nsources:
                L.compute_add_sources_el_cuda_(self.mp, A.ad(self._stf_now(it)), A.i(self.nsources))

    def pack_interfaces(self) -> np.ndarray:
        """transfer_boun_accel_from_device: accel at the interface points, (num_interfaces, max_nibool, 3)."""
        buf = np.zeros((max(self.num_interfaces, 1), max(self.max_nibool, 1), 3), np.float32)
        A = abi.Args()
        self.L.transfer_boun_accel_from_device_(self.mp, buf.ctypes.data, A.i(1))
        abi.check()
        return buf

    def assemble_interfaces(self, recv: np.ndarray):
        """transfer_asmbl_accel_to_device: add the neighbours' contributions (same layout as pack)."""
        A = abi.Args()
        recv = np.ascontiguousarray(recv, np.float32)
        self.L.transfer_asmbl_accel_to_device_(self.mp, recv.ctypes.data, A.i(self.num_interfaces),
                                               A.i(self.max_nibool), A.ai(self.db.get("nibool_interfaces")),
                                               A.ai(self.db.get("ibool_interfaces")), A.i(1))
        abi.check()

    def step_finish(self):
        L, A, it = self.L, abi.Args(), self.it
        one = A.i(1)
        if getattr(self, "pml", False):
            # Dirichlet condition on the layers' outer faces, after the forces
            # (compute_forces_viscoelastic_calling_routine.F90:361-365)
            L.pml_impose_boundary_condition_elastic_cuda_(self.mp)
        L.kernel_3_a_cuda_(self.mp, A.f(self.deltatover2), A.f(0.0), A.i(0), one)
        if self.nrec:
            if not hasattr(self, "_seis_host"):
                self._seis_host = np.zeros(3 * self.nrec * self.nlength, np.float32)
            z = self._seis_host.ctypes.data
            cur = (it - 1) % self.nlength + 1
            L.compute_seismograms_cuda_(self.mp, z, z, z, z, A.i(cur), A.i(self.nlength), A.i(it),
                                        A.i(self.nstep), A.i(0), A.i(1), A.i(0))
        self.it += 1

    def run_per_call(self, nsteps: int):
        self._last_path = "per_call"
        for _ in range(nsteps):
            self.step()
        abi.check()

    # ------------------------------------------------- whole step blocks (fused)
    def run(self, nsteps: int, steps_per_graph: int = 50, timing: bool = False):
        """nsteps time steps on the device (fused predictor/corrector, graph-captured)."""
        self._last_path = "device"
        rc = self.L.sf3d_iterate_time(self.mp, self.it, self.it + nsteps - 1, float(self.deltat),
                                      int(steps_per_graph), int(bool(timing)))
        if rc != 0:
            abi.check()
        self.it += nsteps

    def last_timing(self):
        sm, sl, tm, tl = ctypes.c_float(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
        self.L.sf3d_last_timing(self.mp, ctypes.addressof(sm), ctypes.addressof(sl), ctypes.addressof(tm),
                                ctypes.addressof(tl))
        return dict(stiffness_ms=sm.value, stiffness_launches=sl.value, total_ms=tm.value, total_launches=tl.value)

    # ----------------------------------------------------------------- outputs
    def seismograms(self, kind: str = None) -> np.ndarray:
        """(nrec, 3, nlength) displacement traces (pressure runs: the per-call
        path's host array, pressure in component 0).  kind "displ", "veloc",
        "accel" or "pressure" reads that device buffer (enabled through
        ``record``); fluid receivers hold (1/rho) grad of the potential's
        matching time derivative."""
        if kind is not None:
            code = {"displ": 0, "veloc": 1, "accel": 2, "pressure": 3}[kind]
            out = np.zeros(3 * self.nrec * self.nlength, np.float32)
            if self.nrec:
                self.L.sf3d_get_seismograms_kind(self.mp, code, out.ctypes.data)
                abi.check()
            return out.reshape(self.nlength, self.nrec, 3).transpose(1, 2, 0)
        if "pressure" in self.record and getattr(self, "_last_path", "") == "per_call":
            return self._seis_host.reshape(self.nlength, self.nrec, 3).transpose(1, 2, 0).copy()
        out = np.zeros(3 * self.nrec * self.nlength, np.float32)
        if self.nrec:
            self.L.sf3d_get_seismograms(self.mp, out.ctypes.data)
            abi.check()
        return out.reshape(self.nlength, self.nrec, 3).transpose(1, 2, 0)

    def potentials(self):
        A = abi.Args()
        p, pd, pdd = (np.zeros(self.nglob, np.float32) for _ in range(3))
        self.L.transfer_fields_ac_from_device_(A.i(self.nglob), p.ctypes.data, pd.ctypes.data, pdd.ctypes.data,
                                               self.mp)
        abi.check()
        return p, pd, pdd

    def fields(self):
        A = abi.Args()
        d, v, a = (np.zeros(3 * self.nglob, np.float32) for _ in range(3))
        self.L.transfer_fields_el_from_device_(A.i(3 * self.nglob), d.ctypes.data, v.ctypes.data, a.ctypes.data,
                                               self.mp)
        abi.check()
        return d, v, a

    def reset(self):
        """Back to rest at step 1 (elastic meshes without attenuation or fluid: the
        displacement, velocity and acceleration are the whole state)."""
        if self.attenuation or getattr(self, "nspec_acoustic", 0):
            raise NotImplementedError("reset: the wavefield at rest is set up again by a new solver here")
        z = np.zeros(3 * self.nglob, np.float32)
        self.set_fields(z, z, z)
        self.it = 1

    def set_fields(self, d, v, a):
        A = abi.Args()
        self.L.transfer_fields_el_to_device_(A.i(3 * self.nglob), A.af(d), A.af(v), A.af(a), self.mp)
        abi.check()

    def memory_variables(self):
        A = abi.Args()
        n = N_SLS * NGLL3 * self.nspec
        R = [np.zeros(n, np.float32) for _ in range(6)]
        self.L.transfer_rmemory_from_device_(self.mp, *(r.ctypes.data for r in R), A.i(n))
        abi.check()
        E = [np.zeros(NGLL3 * self.nspec, np.float32) for _ in range(6)]
        self.L.transfer_strain_from_device_(self.mp, *(e.ctypes.data for e in E), A.i(NGLL3 * self.nspec))
        abi.check()
        return R, E

    def forces_only(self, iphase: int = 2):
        """One stiffness pass (compute_forces_viscoelastic_cuda) on the current fields."""
        A = abi.Args()
        self.L.compute_forces_viscoelastic_cuda_(self.mp, A.i(iphase), A.f(self.deltat), A.i(0),
                                                 A.i(self.nspec_elastic), A.i(self.strain), A.i(self.attenuation),
                                                 A.i(1))
        self.L.sf3d_synchronize(self.mp)
        abi.check()

    def set_stiffness_variant(self, variant: int):
        """Stiffness kernel build (sf3d_set_stiffness_variant: 0-16; 3 is the default)."""
        if self.L.sf3d_set_stiffness_variant(self.mp, int(variant)) != 0:
            abi.check()

    def autotune_stiffness(self, reps: int = 3):
        """Time every stiffness variant on the wavefield at rest (before the first
        step) and keep the fastest; returns (variant, ms per variant)."""
        ms = (ctypes.c_float * NUM_STIFFNESS_VARIANTS)()
        best = ctypes.c_int()
        if self.L.sf3d_autotune_stiffness(self.mp, int(reps), ms, ctypes.addressof(best)) != 0:
            abi.check()
        return best.value, [float(x) for x in ms]

    def set_geometry_precision(self, bits: int):
        """32: FP32 geometry and moduli; 16: the "fp16" packed format."""
        if self.L.sf3d_set_geometry_precision(self.mp, int(bits)) != 0:
            abi.check()

    GEOMETRY_FORMATS = {"fp32": 0, "fp16": 1, "bf16": 2, "packed-fp32": 3}

    def set_geometry_format(self, fmt: str):
        """Storage of the stiffness kernel's static element streams (sf3d_set_geometry_format):
        "fp32" (plain arrays), "fp16" / "bf16" (streams constant over an element stored
        once, varying ones as 16-bit rows with a per-element offset and scale), or
        "packed-fp32" (the same packing with FP32 rows: lossless)."""
        if fmt not in self.GEOMETRY_FORMATS:
            raise ValueError(f"geometry format {fmt!r} is not offered")
        if self.L.sf3d_set_geometry_format(self.mp, self.GEOMETRY_FORMATS[fmt]) != 0:
            abi.check()

    def geometry_pack_info(self):
        """(payload rows, device bytes) of the packed format in use."""
        r, b = ctypes.c_long(), ctypes.c_long()
        if self.L.sf3d_geometry_pack_info(self.mp, ctypes.addressof(r), ctypes.addressof(b)) != 0:
            abi.check()
        return r.value, b.value

    def check_stability(self, threshold: float = 1e25):
        m = ctypes.c_float()
        rc = self.L.sf3d_check_stability(self.mp, float(threshold), ctypes.addressof(m))
        return rc, m.value

    def close(self):
        if self.mesh.value:
            A = abi.Args()
            self.L.prepare_cleanup_device_(self.mp, A.i(0), A.i(1), A.i(0))
            self.mesh.value = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
