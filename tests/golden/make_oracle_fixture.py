"""FP64 oracle seismograms of the reference's no-absorbing example (5000 steps).

The reference's REF_SEIS for homogeneous_halfspace_HEX8_elastic_no_absorbing
differ from the FP32 and FP64 oracle by up to 6e-3 relative L2 (correlation
>= 0.99998; the reference's own CI accepts correlation >= 0.999), while the
Stacey example of the same mesh agrees to 3e-4.  This fixture holds the FP64
oracle's traces so the GPU run of that example is also held to the oracle at
FP32 accuracy.  Runs in a few minutes on 8 cores:

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
    cfg = configs.refex(nstep)
    cfg["stacey"] = False
    db = meshgen.build_database(cfg, dtype=np.float64)
    sim = O.make_sim(db, cfg, "f64", nthreads=os.cpu_count() or 1)
    sim.step(nstep)
    seis = O.seismograms(sim).astype(np.float32)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "refex_no_absorbing_oracle_f64.npz")
    np.savez_compressed(out, displ=seis)


if __name__ == "__main__":
    main()
