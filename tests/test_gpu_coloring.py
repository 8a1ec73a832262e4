"""Atomic-free assembly by mesh colouring (USE_MESH_COLORING_GPU): the phase lists
ordered colour by colour, one stiffness launch per colour with plain
read-modify-write scatter.  Seismograms and wavefield equal those of the atomic
assembly (<= 1e-5: the summation order at shared points differs)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("att", [False, True])
def test_colored_assembly_equals_atomic(gpulib, att):
    from specfem3d_gb300 import configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_layered(nx=8, ny=6, counts=(2, 2, 3), nstep=300, attenuation=att)
    db = meshgen.build_database(cfg)
    out = []
    for colors in (None, meshgen.block_colors(cfg)):
        g = GPUSolver(db, cfg, colors=colors)
        g.run(cfg["nstep"], steps_per_graph=50)
        out.append((g.seismograms(), g.fields()[0]))
        g.close()
    g = GPUSolver(db, cfg, colors=meshgen.block_colors(cfg))
    g.run_per_call(cfg["nstep"])
    out.append((g.seismograms(), g.fields()[0]))
    g.close()
    assert np.abs(out[0][0]).max() > 0
    for k in (1, 2):
        assert rel_l2(out[k][0], out[0][0]) < 1e-5
        assert rel_l2(out[k][1], out[0][1]) < 1e-5


def test_tiled_element_order_equals_natural(gpulib):
    """Processing the elements in tiles of 2x2x2 (phase lists reordered) gives the
    natural order's seismograms (<= 1e-5: atomic summation order)."""
    from specfem3d_gb300 import configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_layered(nx=8, ny=6, counts=(2, 2, 3), nstep=300, attenuation=True)
    db = meshgen.build_database(cfg)
    out = []
    for tile in (0, 2):
        g = GPUSolver(db, cfg, tile=tile)
        g.run(cfg["nstep"], steps_per_graph=50)
        out.append(g.seismograms())
        g.close()
    assert np.abs(out[0]).max() > 0
    assert rel_l2(out[1], out[0]) < 1e-5
