"""Extract the reference's traveltime adjoint-source goldens into a compact fixture.

The reference study EXAMPLES/reproducible_study/sensitivity_kernels_liutromp2006
ships the displacement traces of its two forward runs (REF_SEIS/P_SV_simulation,
REF_SEIS/SH_simulation, station XX.R00-01, 6000 samples of 0.01 s from -10 s) and
the adjoint sources its README makes from them with
utils/adjoint_sources/traveltime (xcreate_adjsrc_traveltime t1 t2 ifile):
P (10 18 1) and PS+SP (24 30 1) from the P-SV traces, S (24 34 2) and SS
(34 44 2) from the SH traces (REF_ADJ_SRC/<case>/*.adj).  This script reads them
as the tool does (t0 = first time, dt = second time - first time, in double
precision) and writes tests/golden/liutromp2006_adjsrc.npz: the measured
component of each forward run (X of P-SV, Y of SH) in float64 and that component
of the four reference adjoint sources in float32 (the files carry 7 significant
digits; their other two components are zero, which the script checks).

Run where the SPECFEM3D reference tree is available (first argument, or the
environment variable SPECFEM3D_REFERENCE).
"""
import os
import sys

import numpy as np

STUDY = "EXAMPLES/reproducible_study/sensitivity_kernels_liutromp2006"
CASES = {"P": ("P_SV", 10.0, 18.0, 1), "PSSP": ("P_SV", 24.0, 30.0, 1),
         "S": ("SH", 24.0, 34.0, 2), "SS": ("SH", 34.0, 44.0, 2)}


def read(path):
    t, v = [], []
    with open(path) as f:
        for line in f:
            a, b = line.split()
            t.append(float(a))
            v.append(float(b))
    return np.array(t), np.array(v)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPECFEM3D_REFERENCE", "")
    if not root or not os.path.isdir(root):
        sys.exit("usage: %s <SPECFEM3D source tree> (or set SPECFEM3D_REFERENCE)" % sys.argv[0])
    d = os.path.join(root, STUDY)
    out = {}
    for run, comp in (("P_SV", "X"), ("SH", "Y")):
        t, v = read(os.path.join(d, "REF_SEIS", run + "_simulation", f"XX.R00-01.HX{comp}.semd"))
        out["syn_" + run] = v                                           # (nstep,) float64
        out["t0_" + run] = t[0]
        out["dt_" + run] = t[1] - t[0]
    for case, (run, ts, te, comp) in CASES.items():
        adj = [read(os.path.join(d, "REF_ADJ_SRC", case, f"XX.R00-01.HX{c}.adj"))[1] for c in "XYZ"]
        assert all(not np.any(adj[c]) for c in range(3) if c != comp - 1), case
        out["adj_" + case] = adj[comp - 1].astype(np.float32)
        out["win_" + case] = np.array([ts, te, comp], np.float64)
        out["run_" + case] = np.array(run)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "liutromp2006_adjsrc.npz"), **out)


if __name__ == "__main__":
    main()
