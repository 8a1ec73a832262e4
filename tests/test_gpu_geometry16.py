"""16-bit geometric factors and moduli (sf3d_set_geometry_precision(16)).

* layered viscoelastic block: every metric row and modulus row is constant over
  an element, so the 16-bit storage is exact and the seismograms equal the FP32
  run's (<= 1e-6: atomics reorder sums);
* perturbed block (+-5 % Gaussian-correlated vp/vs per GLL point): the
  seismogram error against the FP64 oracle stays <= 1e-4 relative L2 (the bar
  of the benchmark definition) and within 1e-5 of the FP32 device run's own error
  (measured: 6.0e-6 vs 2.6e-6)."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_geometry16_exact_on_layered_block(gpulib):
    from specfem3d_gb300 import configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_layered(nx=8, ny=6, counts=(2, 2, 3), nstep=400, attenuation=True)
    db = meshgen.build_database(cfg)
    out = []
    for bits in (32, 16):
        g = GPUSolver(db, cfg)
        g.set_geometry_precision(bits)
        g.run(cfg["nstep"], steps_per_graph=50)
        out.append(g.seismograms())
        g.close()
    assert np.abs(out[0]).max() > 0
    assert rel_l2(out[1], out[0]) < 1e-6


def test_geometry16_error_on_perturbed_model(gpulib):
    from oracle import oracle as O
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=500, nshots=1, n=10)
    mat = G.background_material(cfg)
    db = meshgen.build_database(cfg, material=mat)
    db64 = meshgen.build_database(cfg, material=mat, dtype=np.float64)
    sim = O.make_sim(db64, cfg, "f64", nthreads=os.cpu_count() or 1)
    sim.step(cfg["nstep"])
    ref = O.seismograms(sim)
    err = {}
    for bits in (32, 16):
        g = GPUSolver(db, cfg)
        g.set_geometry_precision(bits)
        g.run(cfg["nstep"], steps_per_graph=50)
        err[bits] = rel_l2(g.seismograms(), ref)
        g.close()
    print(f"seismograms vs FP64 oracle: FP32 geometry {err[32]:.2e}, 16-bit geometry {err[16]:.2e}")
    assert err[16] < 1e-4
    assert err[16] < err[32] + 1e-5
