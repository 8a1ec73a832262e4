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
Fortran solver cannot be built here).  Under torchrun with N>1
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
    """DRAM bytes per stiffness launch from the committed ncu summary, scaled to the
    bench mesh by element count, or None."""
    path = os.path.join(ROOT, "profiles", "stiffness_att_traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        return float(t["dram_bytes_per_element"])
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


def cpu_baseline(steps: int, nthreads: int):
    """Oracle (FP32, OpenMP) on a bounded sample with the bench physics: a 32x32x16
    block of the same layered viscoelastic model (irregular elements, Stacey)."""
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen
    cfg = configs.cfg1(nstep=steps + 2, nx=32, ny=32, counts=(4, 6, 6))
    cfg["x1"] = 20000.0 * 32 / 128
    cfg["y1"] = 20000.0 * 32 / 128
    db = meshgen.build_database(cfg)
    sim = O.make_sim(db, cfg, "f32", nthreads=nthreads)
    sim.step(1)
    t = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t
    return db["nglob"] * steps / dt, dict(nspec=db["nspec"], nglob=db["nglob"], steps=steps, seconds=dt)


def run_reference(args, rank):
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    steps = max(1, args.steps)
    val, info = cpu_baseline(steps, nthreads)
    sample = (f"CPU oracle (C restatement of the reference CPU solver, not the reference binary) on a "
              f"32x32x16-element block with the bench physics ({info['nglob']} points), {steps} steps")
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1000 * info["seconds"] / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "cfg1 layered viscoelastic block, CPU sample", "sample_elements": info["nspec"]},
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
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-steps", type=int, default=40)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import ctypes
    from specfem3d_gb300 import abi, build, configs, meshgen, solver
    build.build()
    L = abi.load()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        lr = int(os.environ.get("LOCAL_RANK", "0"))
        A = abi.Args()
        L.initialize_gpu_device_(A.i(lr), A.i(0))
    W, K = max(3, args.warmup), max(1, args.steps)
    if args.small:
        cfg = configs.cfg1(nstep=W + K + args.e2e_steps + 2, nx=32, ny=32, counts=(4, 6, 6))
        workload = "cfg1-physics 32x32x16 block (reduced)"
    else:
        cfg = configs.cfg1(nstep=W + K + args.e2e_steps + 2)
        workload = "cfg1: layered viscoelastic 20x20x10 km, 128x128x64 hexes, N_SLS=3, Stacey 5 faces"
    t0 = time.perf_counter()
    db = meshgen.build_database(cfg)
    t_db = time.perf_counter() - t0
    nspec, nglob = db["nspec"], db["nglob"]
    t0 = time.perf_counter()
    g = solver.GPUSolver(db, cfg, nlength=1)
    t_up = time.perf_counter() - t0
    # ---------------- value: device-resident, graph-captured steps ----------------
    g.run(W, steps_per_graph=args.graph)
    L.sf3d_synchronize(g.mp)
    if dist:
        dist.barrier()
    with ClockSampler() as clk:
        g.run(K, steps_per_graph=args.graph, timing=True)
    tm = g.last_timing()
    total_ms = tm["total_ms"]
    if dist:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nglob * K * world / (total_ms / 1000.0)
    stiff_ms = tm["stiffness_ms"] / max(tm["stiffness_launches"], 1)
    bytes_launch = 33000.0 * nspec + 48.0 * nglob
    peak, peak_kind = _peaks()
    achieved = bytes_launch / (stiff_ms / 1000.0) / 1e9
    traffic_pe = _traffic()
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
    e2e_value = nglob * Ke * world / t_e2e
    h2d = 4 * g.nsources
    d2h = 4 * 3 * g.nrec
    g.close()
    del db
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded moment tensor, layered model of the benchmark definition)",
        "config": {"workload": workload, "nspec": nspec, "nglob": nglob, "nsteps_timed": K,
                   "steps_per_graph": args.graph, "l2": "inputs (~25 GB) far larger than L2; no flush needed",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": (traffic_pe * nspec if traffic_pe else None),
                     "kernel": "stiffness_kernel<att>", "algorithmic_bytes_per_launch": bytes_launch,
                     "mean_launch_ms": stiff_ms},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": Ke, "path": "per-call FC_FUNC_ entry points"},
        "gpu_launches": tm["total_launches"],
        "clocks": clk.summary(),
        "setup": {"database_s": t_db, "upload_s": t_up},
        "stable": rc == 0,
    }
    if rank == 0 and not args.no_cpu:
        cv, info = cpu_baseline(args.cpu_steps, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"CPU oracle, 32x32x16-element block with the bench physics "
                                          f"({info['nglob']} points), {info['steps']} steps, "
                                          f"{info['seconds']:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
