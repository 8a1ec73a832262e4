"""The oracle's C-PML restatement against the reference's own golden seismograms (CPU).

The reference example CPML_examples/homogeneous_halfspace_HEX8_elastic_absorbing_CPML_5sides
(the 36x36x16 block of the Stacey example with C-PML layers of three elements on
the four sides and the bottom, a 1e10 N point force with a 0.128 Hz Ricker,
dt 0.11 s) ships REF_SEIS displacement traces; tests/golden/refex_cpml5sides.npz
holds them.  The set-up (specfem3d_gb300.pml: regions, damping profiles,
recursive-convolution coefficients, PML mass) feeds the FP32 oracle, which runs
the first 300 steps (the direct P and S arrivals at all four stations) in about a
minute.  Over the whole 2400-step record, which the device test
(test_gpu_pml.py::test_pml_reference_golden_seismograms) holds to REF_SEIS, the
same oracle run measured 2.5e-6 relative L2 (worst trace 1.0e-5), correlation
1.000000 on every trace.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

NSTEP = 300


@pytest.fixture(scope="module")
def cpml_oracle():
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen, pml
    cfg = configs.refex_cpml(nstep=NSTEP)
    db = pml.setup(meshgen.build_database(cfg), cfg, nel=cfg["pml_elements"], f0=cfg["pml_f0"])
    sim = O.make_sim(db, cfg, "f32", nthreads=os.cpu_count() or 1)
    sim.step(NSTEP)
    return db, O.seismograms(sim)


def test_cpml_layers_like_reference(cpml_oracle):
    db, _ = cpml_oracle
    # absorbing_cpml_file of the example: 9036 CPML elements, per region (1..7)
    counts = np.bincount(db["cpml_regions"], minlength=8)
    assert list(counts[1:]) == [2340, 2340, 2700, 468, 540, 540, 108]
    # CPML_width_x / _y / _z of its output_generate_databases.txt
    assert np.allclose(db["pml_width"], [11166.667, 11166.667, 11250.0], rtol=1e-6)


def test_cpml_oracle_matches_reference_seismograms(cpml_oracle):
    _, seis = cpml_oracle
    ref = np.load(os.path.join(ROOT, "tests", "golden", "refex_cpml5sides.npz"))["displ"][:, :, :NSTEP]
    gmax = np.abs(ref).max()
    checked = 0
    for r in range(4):
        for c in range(3):
            d = ref[r, c]
            if np.abs(d).max() < 1e-3 * gmax:
                continue  # no signal yet at this station
            a = seis[r, c, :NSTEP]
            assert rel_l2(a, d) < 1e-4, (r, c, rel_l2(a, d))
            assert np.corrcoef(a, d)[0, 1] > 0.99999
            checked += 1
    assert checked >= 6
