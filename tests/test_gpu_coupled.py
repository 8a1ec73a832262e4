"""GPU parity of the fluid-solid path: fluid stiffness, Sommerfeld faces,
coupling terms, pressure source and hydrophones, through the per-call C ABI in
the reference's call order, against the oracle's coupled step (FP32 both)."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_coupled_fluid_solid_vs_oracle(gpulib):
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.small_coupled(nstep=300)
    db = meshgen.build_database(cfg)
    assert db["num_coupling_ac_el_faces"] > 0 and db["ispec_is_acoustic"].sum() > 0
    sim = O.make_coupled_sim(db, cfg, "f32", nthreads=os.cpu_count() or 1)
    O.run_coupled(sim, cfg["nstep"])
    ref = O.seismograms(sim)
    g = solver.GPUSolver(db, cfg)
    g.run_per_call(cfg["nstep"])
    seis = g.seismograms()
    p, pd, pdd = g.potentials()
    d, v, a = g.fields()
    g.close()
    e_p = rel_l2(seis[:, 0], ref[:, 0])
    e_chi = rel_l2(p, sim.get("potential"))
    e_u = rel_l2(d, sim.get("displ"))
    print(f"coupled 300 steps: pressure {e_p:.2e}, potential {e_chi:.2e}, solid displacement {e_u:.2e}")
    assert np.abs(ref[:, 0]).max() > 0 and np.abs(sim.get("displ")).max() > 0
    assert e_p < 5e-5 and e_chi < 5e-5 and e_u < 1e-4


def test_coupled_fused_loop_equals_per_call(gpulib):
    """sf3d_iterate_time with the fluid domain fused into the graph-captured step
    gives the per-call path's hydrophone traces and fields within the tolerance
    the per-call path itself meets against the oracle (5e-5; measured 1.2e-5:
    atomics reorder sums and the fused corrector/predictor rounds differently)."""
    from specfem3d_gb300 import configs, meshgen, solver
    cfg = configs.small_coupled(nstep=300)
    db = meshgen.build_database(cfg)
    g = solver.GPUSolver(db, cfg)
    g.run_per_call(cfg["nstep"])
    s1, p1, d1 = g.seismograms(), g.potentials()[0], g.fields()[0]
    g.close()
    g = solver.GPUSolver(db, cfg)
    g.run(cfg["nstep"], steps_per_graph=50)
    s2, p2, d2 = g.seismograms(), g.potentials()[0], g.fields()[0]
    g.close()
    assert np.abs(s1[:, 0]).max() > 0
    assert rel_l2(s2[:, 0], s1[:, 0]) < 5e-5
    assert rel_l2(p2, p1) < 5e-5 and rel_l2(d2, d1) < 5e-5
