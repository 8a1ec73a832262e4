"""Benchmark of the spectral-element time step on GB300 (one JSON line on stdout).

Workload (N=1): the layered viscoelastic forward of the benchmark definition —
a 20x20x10 km block of 128x128x64 hexahedra (1,048,576 elements, 67,634,433
unique GLL points, NGLL=5), three layers with Qmu 40/150/400 and N_SLS=3
standard linear solids, Stacey on five faces, one moment-tensor source, 400
surface receivers, FP32 fields.  A "step" is one time step over the whole mesh.

Metric: GLL-point updates per second = NGLOB x steps / device time.
* ``value``: steps run by sf3d_iterate_time with all arrays resident in HBM
  (graph-captured step blocks), timed with CUDA events on the compute stream;
* ``e2e``: the same steps driven through the reference-named C-ABI entry
  points one call at a time (update_displacement_cuda, compute_forces_viscoelastic_cuda
  x2, compute_stacey_viscoelastic_cuda, compute_add_sources_el_cuda with the
  step's source time function copied host->device, kernel_3_a_cuda,
  compute_seismograms_cuda copying the step's 400 traces device->host);
* ``roofline``: the stiffness kernel, algorithmic bytes per launch
  (33,000 B per element + 48 B per unique point) over its mean launch time;
* ``cpu_baseline``: the CPU oracle (C restatement of the reference's CPU
  solver, OpenMP over all host cores) on a bounded sample of the same physics.

``--impl reference`` times that CPU implementation alone (the reference's
Fortran solver needs its autotools build, MPI and generated headers, so the
C restatement stands in for it).  Under torchrun with N>1
every rank runs an independent replica of the workload (no data-path
collective) and rank 0 reports the whole-job throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GLL-pt updates/s fwd and adjoint-grad s/shot, batched vs plain GPU, at stated L2 err"
UNIT = "GLL-pt updates/s"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic():
    """DRAM bytes (read + write) of one stiffness launch of the full bench mesh, measured
    with ncu (line 'dram_bytes_per_launch: N' of the committed summary), or None."""
    import re
    path = os.path.join(ROOT, "profiles", "stiffness_kernel_att_traffic_layered_128x128x64.md")
    try:
        m = re.search(r"dram_bytes_per_launch:\s*([0-9.]+)", open(path).read())
        return float(m.group(1)) if m else None
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a timed region."""

    def __init__(self):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        sm, smax, reasons = [], [], set()
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                sm.append(float(p[1]))
                smax.append(float(p[2]))
                for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"],
                                   p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        except Exception:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons)}


WORKLOAD = "layered viscoelastic 20x20x10 km, 128x128x64 hexes, N_SLS=3, Stacey 5 faces"


def cpu_baseline(steps: int, nthreads: int, warmup: int = 1, db=None, cfg=None):
    """CPU oracle (FP32 C restatement of the reference CPU solver, OpenMP over nthreads)
    on the bench workload itself: the full 128x128x64-element layered viscoelastic mesh,
    `warmup` untimed steps then `steps` timed ones.  db/cfg: an already built database
    of that workload (built here when absent)."""
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen
    if db is None:
        cfg = configs.layered_viscoelastic(nstep=steps + warmup + 2)
        db = meshgen.build_database(cfg)
    sim = O.make_sim(db, cfg, "f32", nthreads=nthreads)
    sim.step(max(1, warmup))
    t = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t
    del sim
    return db["nglob"] * steps / dt, dict(nspec=db["nspec"], nglob=db["nglob"], steps=steps, seconds=dt)


def _per_trace_rel_l2(a, ref):
    """rel-L2 of every receiver's trace (3 components x samples), float64."""
    a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
    r = np.asarray(ref, np.float64).reshape(ref.shape[0], -1)
    nr = np.linalg.norm(r, axis=1)
    e = np.linalg.norm(a - r, axis=1) / np.maximum(nr, 1e-300)
    return e, nr


def l2_error_leg(steps: int = 500, nx: int = 32, formats=("fp32", "fp16", "bf16", "packed-fp32")):
    """Per-seismogram relative L2 error of the device run against the FP64 oracle (the
    reference's algorithm with double-precision CUSTOM_REAL, on a database built in
    double precision) at a size the FP64 oracle finishes in seconds, for every
    geometry storage format, on two models:
    * "layered": the bench physics, 20x20x10 km at nx x nx x nx/2 elements (4/6/6
      element rows per layer), N_SLS = 3, Stacey, the source at 8 km depth, the 400
      surface receivers;
    * "perturbed": the batched-shots model (+-5 % Gaussian-correlated vp/vs per GLL
      point, no attenuation) at nx x nx x nx/2 elements, its first shot, 25 receivers."""
    from oracle import oracle as O
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.solver import GPUSolver
    out = {"metric": "rel-L2 per receiver trace (3 components x samples), float64", "nstep": steps,
           "oracle": "FP64 C restatement on an FP64 database"}
    cases = {}
    c = configs.layered_viscoelastic(nstep=steps, nx=nx, ny=nx, counts=(nx // 8, 3 * nx // 16, 3 * nx // 16))
    cases["layered"] = (c, meshgen.build_database(c), meshgen.build_database(c, dtype=np.float64),
                        f"layered viscoelastic 20x20x10 km, {nx}x{nx}x{nx // 2} hexes, N_SLS=3")
    c = G.shot_config(configs.batched_shots(nstep=steps, nshots=1, nx=nx), 0)
    mat = G.background_material(c)
    cases["perturbed"] = (c, meshgen.build_database(c, material=mat),
                          meshgen.build_database(c, material=mat, dtype=np.float64),
                          f"+-5% perturbed block 20x20x10 km, {nx}x{nx}x{nx // 2} hexes, no attenuation")
    for name, (cfg, db, db64, desc) in cases.items():
        t0 = time.perf_counter()
        sim = O.make_sim(db64, cfg, "f64", nthreads=os.cpu_count() or 1)
        sim.step(steps)
        ref = O.seismograms(sim)
        del sim, db64
        res = {"workload": desc, "receivers": int(db["nrec"]), "t_end_s": float(cfg["dt"]) * steps,
               "oracle_s": time.perf_counter() - t0}
        for fmt in formats:
            g = GPUSolver(db, cfg)
            g.set_geometry_format(fmt)
            rows = g.geometry_pack_info()[0]
            g.run(steps, steps_per_graph=50)
            seis = g.seismograms()
            g.close()
            e, nr = _per_trace_rel_l2(seis, ref)
            strong = nr >= 1e-2 * nr.max()
            res[fmt] = {"median": float(np.median(e)), "p95": float(np.percentile(e, 95)), "max": float(e.max()),
                        "max_strong_traces": float(e[strong].max()), "payload_rows": rows,
                        "all_traces": float(np.linalg.norm(np.asarray(seis, np.float64) - ref) / np.linalg.norm(ref))}
        out[name] = res
    return out


def adjoint_leg(nshots: int, nstep: int = 3000):
    """Seconds per shot of the checkpointed misfit gradient on the 64x64x32-element
    gradient workload (3000 steps, checkpoints every 200 steps): forward from rest,
    then the reverse sweep with recomputation; observed traces from the true model."""
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.adjoint_gradient(nstep=nstep, nshots=nshots, checkpoint_every=min(200, nstep))
    db_true = meshgen.build_database(cfg, material=G.true_material(cfg))
    observed = []
    for i in range(nshots):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db_true, cfg, i), c, nlength=cfg["nstep"])
        s.run(cfg["nstep"], steps_per_graph=50)
        observed.append(s.seismograms())
        s.close()
    del db_true
    db0 = meshgen.build_database(cfg, material=G.background_material(cfg))
    t0 = time.perf_counter()
    J, grad, timing = G.misfit_gradient(lambda i: G.shot_database(db0, cfg, i), cfg, observed,
                                        cfg["checkpoint_every"])
    wall = time.perf_counter() - t0
    fwd = sum(t[0] for t in timing) / 1000.0
    bwd = sum(t[1] for t in timing) / 1000.0
    # directional derivative along one seeded smooth direction against central
    # differences of the misfit from device FP32 forward runs (eps = 1e-3; FP32
    # rounding noise limits this check to ~1e-2; the FP64-oracle check at 1e-3 runs
    # in the test suite on a scaled-down copy of this workload)
    n = int(db0["nspec"])
    d = [G.smooth_direction(cfg, 101 + q, corr_len=1500.0) for q in range(3)]
    stores = {k: db0[s].reshape(n, -1).astype(np.float64)
              for k, s in (("rho", "rhostore"), ("kappa", "kappastore"), ("mu", "mustore"))}
    gd = sum(float(np.sum(grad[k] * stores[k] * dq)) for k, dq in zip(("rho", "kappa", "mu"), d))

    def misfit_of(sign, eps=1e-3):
        dbp = G.perturbed_database(db0, cfg, *(sign * eps * dq for dq in d))
        total = 0.0
        for i in range(nshots):
            c = G.shot_config(cfg, i)
            c["record"] = ("displ",)
            s = GPUSolver(G.shot_database(dbp, cfg, i), c, nlength=cfg["nstep"])
            s.run(cfg["nstep"], steps_per_graph=50)
            total += G.misfit(s.seismograms(), observed[i], float(s.deltat))[0]
            s.close()
        return total
    fd = (misfit_of(1.0) - misfit_of(-1.0)) / 2e-3
    return {"unit": "s/shot", "s_per_shot": wall / nshots, "device_s_per_shot": (fwd + bwd) / nshots,
            "fd_check": {"direction": "seeded smooth (dln rho, dln kappa, dln mu), 1.5 km correlation",
                         "adjoint": gd, "central_difference_fp32_device": fd, "eps": 1e-3,
                         "rel": abs(gd - fd) / abs(fd)},
            "forward_s_per_shot": fwd / nshots, "backward_s_per_shot": bwd / nshots, "shots": nshots,
            "nstep": cfg["nstep"], "checkpoint_every": cfg["checkpoint_every"], "nspec": db0["nspec"],
            "nglob": db0["nglob"], "misfit": J, "gradient_dtype": "f64 accumulation, f32 fields",
            "workload": "64x64x32 hexes, 20x20x10 km, perturbed background, +3% vs blob true model"}


def batch_leg(nshots: int, steps: int, nx: int = 64):
    """Per-shot GLL-point updates/s of the batched-shots workload (64x64x32 hexes,
    perturbed model, no attenuation): all shots advancing together with
    shot-innermost fields (autotuned stiffness kernel; FP32 arrays, then packed FP16
    moduli) against the plain single-shot path on the same mesh."""
    import ctypes
    from specfem3d_gb300 import abi, configs, gradient as G, meshgen
    from specfem3d_gb300.batch import BatchSolver
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.batched_shots(nstep=4 * steps + 32, nshots=nshots, nx=nx)
    db = meshgen.build_database(cfg, material=G.background_material(cfg))
    nglob, nspec = int(db["nglob"]), int(db["nspec"])
    b = BatchSolver(db, cfg, nlength=4 * steps + 32)
    tune = b.autotune(reps=3)
    b.run(3, steps_per_graph=0)
    with ClockSampler() as clk:
        ms_one = b.run(steps, steps_per_graph=50)
    ms_two = None
    if tune["kernel"] == "pencil" and nshots % (2 * tune["shots_per_block"]) == 0:
        # the two shot halves on two streams, correctors under the other half's stiffness
        b.set_halves(2)
        b.run(3, steps_per_graph=0)
        ms_two = b.run(steps, steps_per_graph=50)
    halves = 2 if (ms_two is not None and ms_two < ms_one) else 1
    b.set_halves(halves)
    ms_b = ms_one if halves == 1 else ms_two
    b.solver.set_geometry_format("fp16")
    rows = b.solver.geometry_pack_info()[0]
    b.run(3, steps_per_graph=0)
    ms_h = b.run(steps, steps_per_graph=50)
    b.close()
    plain = GPUSolver(db, G.shot_config(cfg, 0), nlength=steps + 8)
    # the plain path at its best: every stiffness variant timed at rest, the fastest kept
    msp = (ctypes.c_float * STIFFNESS_VARIANTS)()
    bestp = ctypes.c_int()
    if plain.L.sf3d_autotune_stiffness(plain.mp, 3, msp, ctypes.addressof(bestp)) != 0:
        abi.check()
    plain.run(3, steps_per_graph=50)
    plain.run(steps, steps_per_graph=50)
    ms_p = plain.last_timing()["total_ms"]
    plain.close()
    # shot-point updates per second: every shot's points advanced one step count once
    rate_b = nglob * steps * nshots / (ms_b / 1000.0)
    rate_h = nglob * steps * nshots / (ms_h / 1000.0)
    rate_p = nglob * steps / (ms_p / 1000.0)
    peak, kind = _peaks()
    # whole batched step, algorithmic bytes: per shot-point u v a read + written (72 B),
    # the u gather (12 B), per point rmass (12 B); per element ibool + kappa/mu (FP32
    # arrays 1,500 B; packed: ibool + record + FP16 rows)
    static32 = 1500.0 * nspec
    static16 = (500.0 + 160.0) * nspec + rows * 250.0
    dyn = (84.0 * nshots + 12.0) * nglob
    # FP32-SIMT ceiling of the batched stiffness: the minimal FMA count of the
    # element algorithm, 663 flop per unique GLL point and shot, over the chosen
    # tiling's pass time from the autotuner
    key = (f"pencil{tune['shots_per_block']}" if tune["kernel"] == "pencil" else
           f"{tune['shots_per_thread']}x{tune['shots_per_block']}x{tune['elements_per_block']}")
    st_ms = tune["ms"].get(key)
    simt = None
    if st_ms:
        tflops = 663.0 * nglob * nshots / (st_ms / 1000.0) / 1e12
        simt = {"flop_per_pt": 663, "stiffness_ms": st_ms, "achieved_tflops": tflops, "peak_tflops": SIMT_TFLOPS,
                "peak_kind": "nominal: 152 SMs x 128 FP32 lanes x 2 flop x 2.07 GHz", "frac": tflops / SIMT_TFLOPS}
    return {"unit": "GLL-pt updates/s summed over shots", "shots": nshots, "steps": steps, "nglob": nglob,
            "nspec": nspec, "batched": rate_b, "batched_fp16_moduli": rate_h, "plain_single_shot": rate_p,
            "speedup_per_shot": rate_b / rate_p, "speedup_per_shot_fp16_moduli": rate_h / rate_p,
            "batched_ms_per_step": ms_b / steps, "batched_fp16_ms_per_step": ms_h / steps,
            "plain_ms_per_step": ms_p / steps, "plain_stiffness_variant": stiffness_variant_name(bestp.value, att=False),
            "clocks_one_stream": clk.summary(),
            "tiling": tune, "halves": halves,
            "ms_per_step_one_stream": ms_one / steps,
            "ms_per_step_two_halves": None if ms_two is None else ms_two / steps,
            "step_hbm_frac": (dyn + static32) / (ms_b / steps / 1000.0) / 1e9 / peak,
            "step_hbm_frac_fp16_moduli": (dyn + static16) / (ms_h / steps / 1000.0) / 1e9 / peak,
            "peak_gbs": peak, "peak_kind": kind, "fp32_simt": simt,
            "workload": f"{nx}x{nx}x{nx // 2} hexes, 20x20x10 km, +-5% perturbed model, no attenuation, "
                        f"{nshots} CMT shots, Ricker 2 Hz"}


def coupled_leg(steps: int):
    """GLL-point updates/s of the coupled fluid-solid workload (96x96x48 hexes, top sixth
    water over a perturbed solid, pressure source, 256 hydrophones): device-resident
    graph-captured steps (value), and the per-call entry points in the reference's order
    (acoustic and elastic predictors, fluid stiffness, Sommerfeld faces, both coupling
    terms, sources, correctors, pressure seismograms), wall clock with the device
    synchronised on both sides (per_call)."""
    from specfem3d_gb300 import configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.coupled_fluid_solid(nstep=2 * steps + 10)
    db = meshgen.build_database(cfg)
    g = GPUSolver(db, cfg)
    variant, ms_var = g.autotune_stiffness()     # at rest, before the first step
    g.run_per_call(3)
    g.L.sf3d_synchronize(g.mp)
    t0 = time.perf_counter()
    g.run_per_call(steps)
    g.L.sf3d_synchronize(g.mp)
    dt = time.perf_counter() - t0
    # the same steps device-resident: graph-captured blocks of sf3d_iterate_time
    # (device stf table, pressure traces kept on the device), CUDA events
    g.run(3, steps_per_graph=50)
    with ClockSampler() as clk:
        g.run(steps, steps_per_graph=50)
    tm = g.last_timing()
    ok = bool(np.isfinite(g.seismograms()).all())
    nglob = int(db["nglob"])
    g.close()
    return {"unit": UNIT, "value": nglob * steps / (tm["total_ms"] / 1000.0), "ms_per_step": tm["total_ms"] / steps,
            "path": "sf3d_iterate_time, graph-captured blocks of 50 steps, CUDA events", "clocks": clk.summary(),
            "per_call": {"value": nglob * steps / dt, "ms_per_step": 1000 * dt / steps,
                         "path": "per-call FC_FUNC_ entry points, host stf per step, pressure traces, wall clock "
                                 "with the device synchronised on both sides"},
            "steps": steps, "nglob": nglob, "nspec": int(db["nspec"]),
            "fluid_elements": int(db["ispec_is_acoustic"].sum()), "finite": ok,
            "stiffness_variant": stiffness_variant_name(variant, att=False),
            "stiffness_ms_per_variant": [round(x, 4) for x in ms_var],
            "workload": "coupled fluid/solid 96x96x48 hexes, 20x20x10 km"}


def pml_leg(steps: int):
    """The reference's C-PML example (36x36x16 block, layers of three elements on five
    faces: 9036 of 20736 elements) through graph-captured device steps, against the
    same block with Stacey faces instead; device time of sf3d_iterate_time, and the
    per-step seismogram error against the reference's REF_SEIS over the full record
    (tests/golden/refex_cpml5sides.npz, 2400 steps)."""
    from specfem3d_gb300 import configs, meshgen, pml
    from specfem3d_gb300.solver import GPUSolver
    out = {"unit": UNIT, "steps": steps}
    cfg = configs.refex_cpml(nstep=2400)
    db = pml.setup(meshgen.build_database(cfg), cfg, nel=cfg["pml_elements"], f0=cfg["pml_f0"])
    g = GPUSolver(db, cfg)
    g.run(2400, steps_per_graph=100)
    seis = g.seismograms()
    g.close()
    ref = np.load(os.path.join(ROOT, "tests", "golden", "refex_cpml5sides.npz"))["displ"]
    out["rel_l2_vs_ref_seis"] = float(np.linalg.norm(seis.astype(np.float64) - ref) / np.linalg.norm(ref))
    for name in ("cpml", "stacey"):
        c = configs.refex_cpml(nstep=steps + 10)
        d = meshgen.build_database(c)
        if name == "cpml":
            d = pml.setup(d, c, nel=c["pml_elements"], f0=c["pml_f0"])
        g = GPUSolver(d, c)
        g.autotune_stiffness()                  # the elastic elements outside the layers
        g.run(5, steps_per_graph=0)
        g.run(steps, steps_per_graph=50)
        t = g.last_timing()
        g.close()
        out[name + "_ms_per_step"] = t["total_ms"] / steps
        out[name + "_value"] = float(d["nglob"]) * steps / (t["total_ms"] / 1000.0)
    out["cpml_over_stacey"] = out["cpml_ms_per_step"] / out["stacey_ms_per_step"]
    out["nspec"], out["cpml_elements"] = int(db["nspec"]), int(np.count_nonzero(db["cpml_regions"]))
    out["workload"] = ("CPML_examples/homogeneous_halfspace_HEX8_elastic_absorbing_CPML_5sides: 36x36x16 hexes, "
                       "134x134x60 km, point force, dt 0.11 s")
    return out


def aniso_leg(db: dict, cfg: dict, steps: int):
    """Stiffness launch time of the main workload with ANISOTROPY on (tilted TI per
    layer: 21 c_ij per GLL point on top of the attenuation arrays), CUDA events
    around every stiffness launch, against the HBM roofline with the extra
    21 x 4 B x 125 = 10,500 B per element."""
    from specfem3d_gb300 import models as M, solver
    lay = np.asarray(cfg["elem_layer"], np.int64)
    L = cfg["layers"]
    C = M.tilted_ti([m["rho"] for m in L], [m["vp"] for m in L], [m["vs"] for m in L])
    d = dict(db)
    for name, (a, b) in zip(M.ANISO_NAMES, M._UPPER):
        d[name] = np.repeat(C[lay, a, b].astype(np.float32), 125)
    d["anisotropy"] = 1
    g = solver.GPUSolver(d, cfg, nlength=1)
    g.run(3, steps_per_graph=0)
    per = {}
    # anisotropic builds: 4, 5, 6 CTAs per SM
    for variant, name in ((2, "4"), (3, "5"), (4, "6")):
        g.set_stiffness_variant(variant)
        g.run(steps, steps_per_graph=0, timing=True)
        t = g.last_timing()
        per[name] = t["stiffness_ms"] / max(t["stiffness_launches"], 1)
    g.close()
    best = min(per, key=per.get)
    ms = per[best]
    nspec, nglob = int(db["nspec"]), int(db["nglob"])
    alg = (33000.0 + 10500.0) * nspec + 48.0 * nglob
    peak, kind = _peaks()
    return {"mean_launch_ms": ms, "algorithmic_bytes_per_launch": alg, "achieved_gbs": alg / (ms / 1000.0) / 1e9,
            "frac": alg / (ms / 1000.0) / 1e9 / peak, "peak_kind": kind, "timed_launches": t["stiffness_launches"],
            "ms_by_ctas_per_sm": per, "kernel": f"stiffness_kernel<att, aniso, {best} CTAs/SM>",
            "workload": "main workload with a tilted transversely isotropic medium per layer"}


def smooth_leg(nx: int = 64, sigma: float = 312.5):
    """Gaussian smoothing of three kernels over an nx x nx x nx/2-element block (312.5 m
    cubes, sigma_h = sigma_v = one element): wall time of prepare / compute / get
    (host binning and copies included) and the point pairs it evaluates."""
    from specfem3d_gb300 import configs, meshgen, smooth as S
    from specfem3d_gb300.hexmesh import element_size_max
    cfg = configs.small_adjoint(nstep=10, nshots=1, n=nx)
    db = meshgen.build_database(cfg)
    xyz = meshgen.element_coordinates(cfg)
    n = int(db["nspec"]) * 125
    kern = np.random.default_rng(1).standard_normal((3, n)).astype(np.float32)
    S.smooth(db, xyz, kern, sigma, sigma)      # warm-up (module load, first launch)
    t0 = time.perf_counter()
    out = S.smooth(db, xyz, kern, sigma, sigma)
    dt = time.perf_counter() - t0
    # element pairs taking part (the inclusion rule on element centres, close to the
    # per-point rule): 125 x 125 point pairs each, one exp and ~12 flops per pair
    h2, v2, h3, v3 = S.smoothing_parameters(sigma, sigma, float(element_size_max(xyz).max()))
    h = float(cfg["x1"]) / nx
    rh, rv = int(np.ceil(float(h3) / h)), int(np.ceil(float(v3) / h))
    pairs_el = int(db["nspec"]) * (2 * rh + 1) ** 2 * (2 * rv + 1)
    return {"wall_s": dt, "nspec": int(db["nspec"]), "kernels": 3, "search_radius_m": float(h3),
            "approx_point_pairs": pairs_el * 125 * 125, "approx_pairs_per_s": pairs_el * 125 * 125 / dt,
            "finite": bool(np.isfinite(out).all())}


def stiffness_variant_name(v: int, att: bool = True) -> str:
    """The kernel build a stiffness variant number selects (sf3d_set_stiffness_variant);
    without attenuation the staged builds have no memory variables to stage."""
    if v == 1:
        return "stiffness_pipe_kernel<att>" if att else "stiffness_pipe_kernel<no att>"
    if v in (15, 16):
        return (f"elem_pencil_kernel<no att, 5 elements per CTA, {8 if v == 15 else 7} CTAs/SM>" if not att else
                "stiffness_kernel<att, 6 CTAs/SM>")
    ctas = [4, 0, 5, 6, 7, 6, 7, 8, 6, 7, 3, 4, 8, 9, 10][v] if att or v < 12 else [8, 10, 12][v - 12]
    kind = ("evict-first element streams" if v in (8, 9) else
            "3 threads per point" if v in (10, 11) else
            "" if not att else
            "cp.async-staged memory variables" if 5 <= v <= 7 else
            "bulk-copy-staged memory variables" if v >= 12 else "")
    name = "stiffness_split_kernel" if v in (10, 11) else "stiffness_kernel"
    return f"{name}<{'att' if att else 'no att'}, {ctas} CTAs/SM" + (f", {kind}>" if kind else ">")


REFERENCE_MAX_STEPS = 40
STIFFNESS_VARIANTS = 17          # sf3d_autotune_stiffness writes one time per variant
SIMT_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def run_reference(args, rank):
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    # about 1.3 s per step of the full mesh on 16 cores: at most 40 timed steps keep
    # the arm within about a minute and a half whatever --steps asks
    steps = max(1, min(args.steps, REFERENCE_MAX_STEPS))
    warm = max(1, min(args.warmup, 3))
    val, info = cpu_baseline(steps, nthreads, warmup=warm)
    sample = (f"CPU oracle (C restatement of the reference CPU solver, not the reference binary; FP32, OpenMP "
              f"over {nthreads} threads) on the full bench mesh ({info['nspec']} elements, {info['nglob']} points), "
              f"{steps} timed steps (of the {args.steps} requested) after {warm} warm-up steps; the reference's "
              f"Fortran solver cannot be built (no Fortran compiler or MPI)")
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": warm, "steps_requested": args.steps, "ms_per_step": 1000 * info["seconds"] / steps,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nspec": info["nspec"], "nglob": info["nglob"]},
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="scaled-down mesh for quick checks")
    ap.add_argument("--graph", type=int, default=50, help="steps per captured CUDA graph")
    ap.add_argument("--tile", type=int, default=4,
                    help="process elements in tiles of tile^3 (0: mesh order); 4 measured 1.3 %% faster "
                         "stiffness launches on the layered workload (L2 reuse of the gathered fields)")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-steps", type=int, default=10, help="timed CPU-oracle steps on the full bench mesh")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--variant", type=int, default=-1,
                    help="stiffness kernel variant (sf3d_set_stiffness_variant); -1: autotune at rest")
    ap.add_argument("--batch", type=int, default=32,
                    help="also time this many shots of the batched-shots workload against the plain path (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--batch-nx", type=int, default=64, help="elements along x and y of the batched mesh")
    ap.add_argument("--coupled", type=int, default=100, help="also time this many steps of the coupled workload")
    ap.add_argument("--aniso", type=int, default=0,
                    help="also time this many steps of the main workload with anisotropic stiffness (0: skip)")
    ap.add_argument("--smooth", action="store_true", help="also time the Gaussian smoothing of three kernels")
    ap.add_argument("--smooth-nx", type=int, default=64, help="elements along x and y of the smoothing block")
    ap.add_argument("--l2-steps", type=int, default=500,
                    help="steps of the seismogram-error run against the FP64 oracle (0: skip)")
    ap.add_argument("--adjoint", type=int, default=8,
                    help="also time the checkpointed misfit gradient over this many shots of the "
                         "8-shot 64x64x32 gradient workload (0: skip)")
    ap.add_argument("--adjoint-steps", type=int, default=3000, help="time steps of the gradient workload")
    ap.add_argument("--roofline-steps", type=int, default=20,
                    help="steps whose stiffness launches are bracketed by CUDA events")
    ap.add_argument("--pml-steps", type=int, default=200, help="timed steps of the C-PML example (0: skip)")
    ap.add_argument("--legs", default="main,batch,coupled,adjoint,l2,pml",
                    help="comma list of the parts to run: main (the headline workload and its e2e, roofline, "
                         "geometry, CPU-oracle lines), batch, coupled, adjoint, l2, pml; without main one JSON "
                         "line holds the selected legs only (profiling)")
    args = ap.parse_args()
    legs = set(x.strip() for x in args.legs.split(",") if x.strip())
    if "batch" not in legs:
        args.batch = 0
    if "coupled" not in legs:
        args.coupled = 0
    if "adjoint" not in legs:
        args.adjoint = 0
    if "l2" not in legs:
        args.l2_steps = 0
    if "pml" not in legs:
        args.pml_steps = 0
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import ctypes
    from specfem3d_gb300 import abi, build, configs, meshgen, solver
    build.build()
    L = abi.load()
    if "main" not in legs:
        out = {"legs": sorted(legs)}
        if args.batch > 0:
            out["batched"] = batch_leg(args.batch, args.batch_steps, args.batch_nx)
        if args.coupled > 0:
            out["coupled"] = coupled_leg(args.coupled)
        if args.adjoint > 0:
            out["adjoint"] = adjoint_leg(args.adjoint, args.adjoint_steps)
        if args.l2_steps > 0:
            out["l2_error"] = l2_error_leg(args.l2_steps)
        if args.pml_steps > 0:
            out["pml"] = pml_leg(args.pml_steps)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        lr = int(os.environ.get("LOCAL_RANK", "0"))
        A = abi.Args()
        L.initialize_gpu_device_(A.i(lr), A.i(0))
    W, K = max(3, args.warmup), max(1, args.steps)
    Kr = max(3, min(K, args.roofline_steps))
    nstep_total = W + 2 * K + 4 * Kr + args.e2e_steps + 4 + (3 * args.aniso + 3 if args.aniso > 0 else 0)
    if args.small:
        cfg = configs.layered_viscoelastic(nstep=nstep_total, nx=32, ny=32, counts=(4, 6, 6))
        workload = "layered viscoelastic 32x32x16 block (reduced)"
    else:
        cfg = configs.layered_viscoelastic(nstep=nstep_total)
        workload = WORKLOAD
    t0 = time.perf_counter()
    db = meshgen.build_database(cfg)
    t_db = time.perf_counter() - t0
    nspec, nglob = db["nspec"], db["nglob"]
    t0 = time.perf_counter()
    g = solver.GPUSolver(db, cfg, nlength=1, tile=args.tile)
    t_up = time.perf_counter() - t0
    # ---------------- value: device-resident, graph-captured steps ----------------
    if args.variant >= 0:
        g.set_stiffness_variant(args.variant)
        autotune = None
    else:
        # fields are at rest: time every stiffness variant and keep the fastest
        ms = (ctypes.c_float * STIFFNESS_VARIANTS)()
        best = ctypes.c_int()
        if L.sf3d_autotune_stiffness(g.mp, 3, ms, ctypes.addressof(best)) != 0:
            abi.check()
        autotune = {"ms_per_variant": [round(float(x), 4) for x in ms], "chosen": best.value}
        args.variant = best.value
    # the packed builds (6 or 7 CTAs/SM, or staged memory variables at 7 or 8),
    # autotuned per format while the wavefield is still at rest
    geom_variant = {}
    for fmt in ("fp16", "bf16", "packed-fp32"):
        g.set_geometry_format(fmt)
        msf = (ctypes.c_float * STIFFNESS_VARIANTS)()
        bestf = ctypes.c_int()
        if L.sf3d_autotune_stiffness(g.mp, 3, msf, ctypes.addressof(bestf)) != 0:
            abi.check()
        geom_variant[fmt] = (bestf.value, [round(float(x), 4) for x in msf])
    g.set_geometry_format("fp32")
    g.set_stiffness_variant(args.variant)
    g.run(W, steps_per_graph=args.graph)
    L.sf3d_synchronize(g.mp)
    if dist:
        dist.barrier()
    with ClockSampler() as clk:
        g.run(K, steps_per_graph=args.graph)
        tm = g.last_timing()
        # kernel-level timing: CUDA events on the compute stream around every
        # stiffness launch (steps launched one by one, not through a graph)
        g.run(Kr, steps_per_graph=0, timing=True)
        tk = g.last_timing()
    abi.check()
    from specfem3d_gb300.parallel_host import replica_throughput
    # whole-job units over the slowest rank's time (replicas: equal work per rank)
    value = replica_throughput(float(nglob) * K, tm["total_ms"])
    total_ms = float(nglob) * K * world / value * 1000.0
    stiff_ms = tk["stiffness_ms"] / max(tk["stiffness_launches"], 1)
    bytes_launch = 33000.0 * nspec + 48.0 * nglob
    peak, peak_kind = _peaks()
    achieved = bytes_launch / (stiff_ms / 1000.0) / 1e9
    traffic_pe = _traffic()
    # packed static element streams (constant streams stored once per element,
    # varying ones as FP16 / BF16 / FP32 rows): stiffness launches timed the same way
    geometry = {}
    for fmt in ("fp16", "bf16", "packed-fp32"):
        g.set_geometry_format(fmt)
        rows, pack_bytes = g.geometry_pack_info()
        g.set_stiffness_variant(geom_variant[fmt][0])
        g.run(Kr, steps_per_graph=0, timing=True)
        th = g.last_timing()
        ms = th["stiffness_ms"] / max(th["stiffness_launches"], 1)
        vb = 4 if fmt == "packed-fp32" else 2
        # ibool + per-element record + payload rows + memory variables / strains R+W
        alg = (500.0 + 160.0 + 24000.0) * nspec + rows * 125.0 * vb + 48.0 * nglob
        geometry[fmt] = {"mean_launch_ms": ms, "payload_rows": rows, "pack_device_bytes": pack_bytes,
                         "algorithmic_bytes_per_launch": alg, "achieved_gbs": alg / (ms / 1000.0) / 1e9,
                         "frac": alg / (ms / 1000.0) / 1e9 / peak, "speedup_vs_fp32_arrays": stiff_ms / ms,
                         "variant": geom_variant[fmt][0], "ms_per_variant": geom_variant[fmt][1]}
    # whole steps with the lossless packing (same results as the FP32 arrays)
    g.set_geometry_format("packed-fp32")
    g.run(K, steps_per_graph=args.graph)
    tp = g.last_timing()
    geometry["packed-fp32"]["step_value"] = float(nglob) * K / (tp["total_ms"] / 1000.0)
    geometry["packed-fp32"]["ms_per_step"] = tp["total_ms"] / K
    g.set_geometry_format("fp32")
    g.set_stiffness_variant(args.variant)
    abi.check()
    geometry["fp32_arrays_mean_launch_ms"] = stiff_ms
    geometry["note"] = ("streams constant over an element stored once (exact); the layered workload's "
                        "box elements and per-layer materials leave no varying stream")
    rc, maxu = g.check_stability(1e25)
    # ---------------- e2e: per-call C-ABI path, host buffers ----------------
    A = abi.Args()
    Ke = max(1, args.e2e_steps)
    L.sf3d_synchronize(g.mp)
    t0 = time.perf_counter()
    g.run_per_call(Ke)
    L.sf3d_synchronize(g.mp)
    t_e2e = time.perf_counter() - t0
    abi.check()
    e2e_value = replica_throughput(float(nglob) * Ke, t_e2e * 1000.0)
    h2d = 4 * g.nsources
    d2h = 4 * 3 * g.nrec
    g.close()
    # atomic-free assembly by mesh colouring (8 parity colours of the block), timed the
    # same way, to choose between red.global atomics and colouring by measurement
    gc = solver.GPUSolver(db, cfg, nlength=1, colors=meshgen.block_colors(cfg))
    gc.run(W, steps_per_graph=args.graph)
    gc.run(Kr, steps_per_graph=0, timing=True)
    tc = gc.last_timing()
    gc.close()
    abi.check()
    color_ms = tc["stiffness_ms"] / max(tc["stiffness_launches"], 1)
    aniso = aniso_leg(db, cfg, args.aniso) if args.aniso > 0 else None
    cpu = None
    if rank == 0 and not args.no_cpu and args.cpu_steps > 0:
        # the CPU oracle on this very mesh (same database, same physics)
        cpu = cpu_baseline(args.cpu_steps, os.cpu_count() or 1, warmup=1, db=db, cfg=cfg)
    del db
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded moment tensor, layered model of the benchmark definition)",
        "config": {"workload": workload, "nspec": nspec, "nglob": nglob, "nsteps_timed": K,
                   "steps_per_graph": args.graph, "l2": "inputs (~25 GB) far larger than L2; no flush needed",
                   "element_order": (f"phase lists in {args.tile}x{args.tile}x{args.tile} tiles of the block"
                                     if args.tile > 0 else "mesh order"),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": (traffic_pe if (traffic_pe and nspec == 1048576) else None),
                     "traffic_kind": "constant from a committed ncu profile, not measured in this run",
                     "traffic_note": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one stiffness launch "
                                      "of this mesh, read from profiles/stiffness_kernel_att_traffic_layered_128x128x64.md"),
                     "kernel": stiffness_variant_name(args.variant),
                     "autotune": autotune,
                     "algorithmic_bytes_per_launch": bytes_launch,
                     "mean_launch_ms": stiff_ms, "timed_launches": tk["stiffness_launches"]},
        "geometry": geometry,
        "assembly": {"atomic_stiffness_ms": stiff_ms, "colored_stiffness_ms": color_ms,
                     "chosen": "atomic" if stiff_ms <= color_ms else "colored",
                     "note": "colored: 8 launches per step (one per colour), plain read-modify-write scatter"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": Ke, "path": "per-call FC_FUNC_ entry points"},
        "gpu_launches": tm["total_launches"],
        "gpu_launches_note": "kernels launched by the timed sf3d_iterate_time call (value)",
        "clocks": clk.summary(),
        "setup": {"database_s": t_db, "upload_s": t_up},
        "stable": rc == 0,
    }
    if args.batch > 0:
        line["batched"] = batch_leg(args.batch, args.batch_steps, args.batch_nx)
    if args.coupled > 0:
        line["coupled"] = coupled_leg(args.coupled)
    if args.adjoint > 0:
        line["adjoint"] = adjoint_leg(args.adjoint, args.adjoint_steps)
    if aniso is not None:
        line["anisotropic"] = aniso
    if args.smooth:
        line["smoothing"] = smooth_leg(args.smooth_nx)
    if args.l2_steps > 0:
        line["l2_error"] = l2_error_leg(args.l2_steps)
    if args.pml_steps > 0:
        line["pml"] = pml_leg(args.pml_steps)
    if cpu is not None:
        cv, info = cpu
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"CPU oracle (FP32 C restatement, OpenMP) on the bench mesh itself "
                                          f"({info['nspec']} elements, {info['nglob']} points), {info['steps']} "
                                          f"steps after 1 warm-up step, {info['seconds']:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
