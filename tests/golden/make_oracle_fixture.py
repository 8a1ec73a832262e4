"""FP64 oracle seismograms of the reference's no-absorbing example (5000 steps).

The source of homogeneous_halfspace_HEX8_elastic_no_absorbing lies on a vertex
shared by 8 elements; its REF_SEIS run placed it in the element on the -x, +y, -z
side (configs.refex_no_absorbing).  This fixture holds the FP64 oracle's traces
of that set-up so the GPU run of the example is held to the oracle at FP32
accuracy, besides the REF_SEIS comparison.  Runs in a few minutes on 8 cores:

    python tests/golden/make_oracle_fixture.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main():
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen
    nstep = 5000
    cfg = configs.refex_no_absorbing(nstep)
    db = meshgen.build_database(cfg, dtype=np.float64)
    sim = O.make_sim(db, cfg, "f64", nthreads=os.cpu_count() or 1)
    sim.step(nstep)
    seis = O.seismograms(sim).astype(np.float32)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "refex_no_absorbing_oracle_f64.npz")
    np.savez_compressed(out, displ=seis)


if __name__ == "__main__":
    main()
