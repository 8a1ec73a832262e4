"""Batched shots on one mesh (sf3d_batch_*) against one plain run per shot.

Eight shots of a perturbed block advance together with shot-innermost fields;
each shot's seismograms and final displacement equal those of a separate
single-shot run through sf3d_iterate_time on the same mesh (same arithmetic
per shot; atomics reorder sums, so <= 1e-5 relative), for tilings of both
batched stiffness kernels (one shot per thread; four shots per thread with
float4 rows and vector atomics; on this all-regular mesh the 4-shot, one-group
tilings run the metric-free regular kernel) and for the one the autotuner
picks; a mesh with irregular elements runs the general float4 kernel."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plain_runs(gpulib):
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=300, nshots=8, n=10)
    db = meshgen.build_database(cfg, material=G.background_material(cfg))
    seis, disp = [], []
    for i in range(len(cfg["shots"])):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db, cfg, i), c)
        s.run(cfg["nstep"], steps_per_graph=50)
        seis.append(s.seismograms())
        disp.append(s.fields()[0].reshape(-1, 3))
        s.close()
    return cfg, db, np.stack(seis), np.stack(disp)


@pytest.mark.parametrize("tiling", [(8, 1, 1), (4, 2, 1), (2, 4, 1), (1, 1, 1), (4, 1, 4), (4, 2, 4), (4, 4, 4),
                                    (8, 2, 4), None])
def test_batched_shots_equal_plain_runs(plain_runs, tiling):
    from specfem3d_gb300.batch import BatchSolver
    cfg, db, seis_ref, disp_ref = plain_runs
    b = BatchSolver(db, cfg)
    if tiling is None:
        info = b.autotune(reps=2)
        print("autotuned tiling:", info)
    else:
        b.set_tiling(*tiling)
    b.run(cfg["nstep"] // 2, steps_per_graph=25)
    b.run(cfg["nstep"] - cfg["nstep"] // 2, steps_per_graph=25)
    seis = b.seismograms()
    disp = b.displacement()
    b.close()
    assert np.abs(seis_ref).max() > 0
    for s in range(len(cfg["shots"])):
        assert rel_l2(seis[s], seis_ref[s]) < 1e-5, s
        assert rel_l2(disp[s], disp_ref[s]) < 1e-5, s


def test_batched_shots_irregular_mesh(gpulib):
    """A taller bottom element row makes part of the mesh irregular (non-cube; no
    smaller spacing, so the time step stays stable): the general float4 kernel
    (metric per point) and the plain runs agree to 1e-5."""
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.batch import BatchSolver
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=200, nshots=4, n=8)
    z = list(cfg["zlev"])
    z[0] = z[0] - 0.3 * (z[1] - z[0])
    cfg["zlev"] = z
    db = meshgen.build_database(cfg, material=G.background_material(cfg))
    assert 0 < db["nspec_irregular"] < db["nspec"]
    b = BatchSolver(db, cfg)
    b.set_tiling(4, 1, 4)
    b.run(cfg["nstep"], steps_per_graph=25)
    seis = b.seismograms()
    b.close()
    for i in range(len(cfg["shots"])):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db, cfg, i), c)
        s.run(cfg["nstep"], steps_per_graph=50)
        ref = s.seismograms()
        s.close()
        assert np.abs(ref).max() > 0
        assert rel_l2(seis[i], ref) < 1e-5, i
