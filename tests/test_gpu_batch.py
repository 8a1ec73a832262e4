"""Batched shots on one mesh (sf3d_batch_*) against one plain run per shot and
against the oracle.

Sixteen shots of a perturbed block advance together with shot-innermost fields;
each shot's seismograms and final displacement equal those of a separate
single-shot run through sf3d_iterate_time on the same mesh (same arithmetic
per shot; atomics reorder sums, so <= 1e-5 relative), for tilings of every
batched stiffness kernel (one shot per thread; four shots per thread with
float4 rows and vector atomics, on this all-regular mesh the 4-shot, one-group
tilings run the metric-free regular kernel; the register-blocked pencil kernel
with 8 and 16 shots per CTA) and for the one the autotuner picks.  Two shots of
the autotuned batch are compared with the FP32 oracle directly.  32 shots run
the pencil kernel with 32 shots per CTA; a mesh with irregular elements runs the
general float4 kernel and the pencil kernel's metric path; packed FP16 / FP32
moduli feed the pencil kernel."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plain_runs(gpulib):
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=300, nshots=16, n=10)
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
                                    (8, 2, 4), (8, 1, 0), (16, 1, 0), None])
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
    if tiling is None:
        # the autotuned batch against the oracle (FP32 C restatement), shots 0 and 11
        import os
        from oracle import oracle as O
        from specfem3d_gb300 import gradient as G
        for shot in (0, 11):
            c = G.shot_config(cfg, shot)
            sim = O.make_sim(G.shot_database(db, cfg, shot), c, "f32", nthreads=os.cpu_count() or 1)
            sim.step(cfg["nstep"])
            assert rel_l2(seis[shot], O.seismograms(sim)) < 5e-5, shot


@pytest.mark.parametrize("lanes", [8])
def test_batched_two_halves_equal_plain_runs(plain_runs, lanes):
    """The two shot halves on two streams (each half's corrector under the other
    half's stiffness, graph-captured with event edges, and the remainder launched
    directly) give every shot its plain run."""
    from specfem3d_gb300.batch import BatchSolver
    cfg, db, seis_ref, disp_ref = plain_runs
    b = BatchSolver(db, cfg)
    b.set_tiling(lanes, 1, 0)
    b.set_halves(2)
    b.run(cfg["nstep"] // 2, steps_per_graph=25)
    b.run(cfg["nstep"] - cfg["nstep"] // 2, steps_per_graph=40)
    seis = b.seismograms()
    disp = b.displacement()
    b.close()
    for s in range(len(cfg["shots"])):
        assert rel_l2(seis[s], seis_ref[s]) < 1e-5, s
        assert rel_l2(disp[s], disp_ref[s]) < 1e-5, s


def test_batched_pencil_32_shots_and_packed_moduli(gpulib):
    """32 shots: the pencil kernel with 32 shots per CTA equals the per-point float4
    kernel to the atomic-order level, and three shots equal their plain runs; packed
    moduli (kappa / mu rows vary per point on this model) in FP32 rows give the FP32
    arrays' result, in FP16 rows stay within 2e-5 of it."""
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.batch import BatchSolver
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=200, nshots=32, n=8)
    db = meshgen.build_database(cfg, material=G.background_material(cfg))
    out = {}
    for name, tiling, fmt in (("float4", (4, 1, 4), "fp32"), ("pencil32", (32, 1, 0), "fp32"),
                              ("pencil16-packed32", (16, 1, 0), "packed-fp32"),
                              ("pencil8-fp16", (8, 1, 0), "fp16")):
        b = BatchSolver(db, cfg)
        b.solver.set_geometry_format(fmt)
        b.set_tiling(*tiling)
        b.run(cfg["nstep"], steps_per_graph=25)
        out[name] = b.seismograms()
        b.close()
    assert np.abs(out["float4"]).max() > 0
    assert rel_l2(out["pencil32"], out["float4"]) < 1e-5
    assert rel_l2(out["pencil16-packed32"], out["float4"]) < 1e-5
    assert rel_l2(out["pencil8-fp16"], out["float4"]) < 2e-5
    for i in (0, 17, 31):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db, cfg, i), c)
        s.run(cfg["nstep"], steps_per_graph=50)
        ref = s.seismograms()
        s.close()
        assert rel_l2(out["pencil32"][i], ref) < 1e-5, i


@pytest.mark.parametrize("tiling", [(4, 1, 4), (8, 1, 0)])
def test_batched_shots_irregular_mesh(gpulib, tiling):
    """A taller bottom element row makes part of the mesh irregular (non-cube; no
    smaller spacing, so the time step stays stable): the general float4 kernel
    (metric per point), the pencil kernel's metric path and the plain runs agree to
    1e-5."""
    from specfem3d_gb300 import configs, gradient as G, meshgen
    from specfem3d_gb300.batch import BatchSolver
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_adjoint(nstep=200, nshots=8, n=8)
    z = list(cfg["zlev"])
    z[0] = z[0] - 0.3 * (z[1] - z[0])
    cfg["zlev"] = z
    db = meshgen.build_database(cfg, material=G.background_material(cfg))
    assert 0 < db["nspec_irregular"] < db["nspec"]
    b = BatchSolver(db, cfg)
    b.set_tiling(*tiling)
    b.run(cfg["nstep"], steps_per_graph=25)
    seis = b.seismograms()
    b.close()
    for i in (0, 3, 7):
        c = G.shot_config(cfg, i)
        c["record"] = ("displ",)
        s = GPUSolver(G.shot_database(db, cfg, i), c)
        s.run(cfg["nstep"], steps_per_graph=50)
        ref = s.seismograms()
        s.close()
        assert np.abs(ref).max() > 0
        assert rel_l2(seis[i], ref) < 1e-5, i
