"""Extract the reference's golden seismograms into compact fixtures.

Run in a checkout where the SPECFEM3D reference tree is available (its path is
the first argument, or the environment variable SPECFEM3D_REFERENCE).  It reads the ASCII
traces (.semd, .semv, .sema) committed under the reference's example REF_SEIS
directories and writes float32 arrays (station, component, sample) plus the time
axis to tests/golden/*.npz.  The fixtures are used by the oracle and GPU parity tests,
which never read the reference tree at run time.
"""
import os
import sys

import numpy as np

EX = "EXAMPLES/applications"
STATIONS = ["X20", "X30", "X40", "X50"]


def read(root, example, ext, band="BX"):
    d = os.path.join(root, EX, example, "REF_SEIS")
    traces, t = [], None
    for st in STATIONS:
        comps = []
        for c in "XYZ":
            a = np.loadtxt(os.path.join(d, f"DB.{st}.{band}{c}.{ext}"))
            t = a[:, 0]
            comps.append(a[:, 1])
        traces.append(comps)
    return np.asarray(traces, np.float32), np.asarray(t, np.float64)


def read_waterlayered(root):
    """waterlayered_halfspace REF_SEIS: vertical (HXZ) traces; displacement (the
    nine X10..X90 stations it has) and velocity (all 22 stations).  Its
    acceleration traces are left out to keep the fixture small."""
    d = os.path.join(root, EX, "waterlayered_halfspace", "REF_SEIS")
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from specfem3d_gb300.configs import WATERLAYERED_STATIONS
    names = [n for n, _, _, _ in WATERLAYERED_STATIONS]
    out, t = {}, None
    for ext, key in (("semd", "displ"), ("semv", "veloc")):
        rows, have = [], []
        for n in names:
            f = os.path.join(d, f"DB.{n}.HXZ.{ext}")
            if os.path.exists(f):
                a = np.loadtxt(f)
                t = a[:, 0]
                rows.append(a[:, 1])
                have.append(n)
        out[key] = np.asarray(rows, np.float32)
        out[key + "_stations"] = np.array(have)
    out["t"] = np.asarray(t, np.float64)
    return out


def read_attenuation_benchmark(root):
    """EXAMPLES/benchmarks/attenuation/viscoelastic REF_SEIS: station CE.1,
    displacement FXX, FXY, FXZ."""
    d = os.path.join(root, "EXAMPLES/benchmarks/attenuation/viscoelastic/REF_SEIS")
    comps, t = [], None
    for c in "XYZ":
        a = np.loadtxt(os.path.join(d, f"CE.1.FX{c}.semd"))
        t = a[:, 0]
        comps.append(a[:, 1])
    return dict(displ=np.asarray([comps], np.float32), t=np.asarray(t, np.float64), stations=np.array(["CE.1"]))


def read_analytic_elastic(root):
    """EXAMPLES/benchmarks/analytic_examples/analytic_solution_elastic: REF_SEIS
    (the reference's run) and REF_ANALYTIC (Aki & Richards 4.32-4.33) for
    stations Z1..Z6, displacement FXX, FXY, FXZ; every 10th of the 14000
    samples (the signal has a 2 s half duration; dt is 1 ms) to keep the
    fixture small."""
    base = os.path.join(root, "EXAMPLES/benchmarks/analytic_examples/analytic_solution_elastic")
    out = {}
    for sub, key in (("REF_SEIS", "displ"), ("REF_ANALYTIC", "analytic")):
        tr, t = [], None
        for n in ["Z1", "Z2", "Z3", "Z4", "Z5", "Z6"]:
            comps = []
            for c in "XYZ":
                a = np.loadtxt(os.path.join(base, sub, f"DB.{n}.FX{c}.semd"))
                t = a[::10, 0]
                comps.append(a[::10, 1])
            tr.append(comps)
        out[key] = np.asarray(tr, np.float32)
        out["t_" + key] = np.asarray(t, np.float64)
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPECFEM3D_REFERENCE", "")
    if not root or not os.path.isdir(root):
        sys.exit("usage: %s <SPECFEM3D source tree> (or set SPECFEM3D_REFERENCE)" % sys.argv[0])
    out = os.path.dirname(os.path.abspath(__file__))
    d, t = read(root, "homogeneous_halfspace_HEX8_elastic_absorbing_Stacey_5sides", "semd")
    np.savez_compressed(os.path.join(out, "refex_stacey5sides.npz"), displ=d, t=t, stations=np.array(STATIONS))
    nd, t2 = read(root, "homogeneous_halfspace_HEX8_elastic_no_absorbing", "semd")
    np.savez_compressed(os.path.join(out, "refex_no_absorbing.npz"), displ=nd, t=t2, stations=np.array(STATIONS))
    # pure-fluid example: pressure traces (.semp, band code M, component P)
    ap, tp = [], None
    for st in STATIONS:
        a = np.loadtxt(os.path.join(root, EX, "homogeneous_acoustic", "REF_SEIS", f"DB.{st}.MXP.semp"))
        tp = a[:, 0]
        ap.append(a[:, 1])
    np.savez_compressed(os.path.join(out, "refex_acoustic.npz"), pressure=np.asarray(ap, np.float32),
                        t=np.asarray(tp, np.float64), stations=np.array(STATIONS))
    # C-PML example (dt 0.11 s: band code M)
    cd, t3 = read(root, "CPML_examples/homogeneous_halfspace_HEX8_elastic_absorbing_CPML_5sides", "semd", "MX")
    np.savez_compressed(os.path.join(out, "refex_cpml5sides.npz"), displ=cd, t=t3, stations=np.array(STATIONS))
    np.savez_compressed(os.path.join(out, "waterlayered.npz"), **read_waterlayered(root))
    np.savez_compressed(os.path.join(out, "attenuation_benchmark.npz"), **read_attenuation_benchmark(root))
    np.savez_compressed(os.path.join(out, "analytic_elastic.npz"), **read_analytic_elastic(root))


if __name__ == "__main__":
    main()
