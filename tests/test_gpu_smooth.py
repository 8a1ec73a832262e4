"""Gaussian smoothing of kernels on the device (prepare/compute/get_smooth_gpu)
against the oracle's FP64 restatement of process_smooth: relative L2 <= 1e-6
(FP32 weights and per-element partial sums, FP64 totals; measured 2.3e-7), on a layered block and
on a block with moved interior nodes; a constant field stays constant to 1e-6
relative."""
import numpy as np
import pytest

from conftest import rel_l2
import hexmesh_cases as C

pytestmark = pytest.mark.gpu


def _case(which):
    from specfem3d_gb300 import configs, hexmesh, meshgen
    cfg = configs.small_layered(nstep=10, attenuation=False)
    if which == "block":
        db = meshgen.build_database(cfg)
        xyz = meshgen.element_coordinates(cfg)
    else:
        mesh = C.distorted(cfg)
        db = hexmesh.build_database(mesh, cfg)
        xyz = hexmesh.gll_points(mesh["nodes"][mesh["elems"]])
    return db, xyz


@pytest.mark.parametrize("which", ["block", "distorted"])
def test_smoothing_vs_oracle(gpulib, which):
    from oracle import oracle as O
    from specfem3d_gb300 import smooth as S
    from specfem3d_gb300.hexmesh import element_size_max
    db, xyz = _case(which)
    n = int(db["nspec"]) * 125
    rng = np.random.default_rng(3)
    kern = rng.standard_normal((3, n)).astype(np.float32)
    sh, sv = 100.0, 60.0
    got = S.smooth(db, xyz, kern, sh, sv)
    h2, v2, h3, v3 = S.smoothing_parameters(sh, sv, float(element_size_max(xyz).max()))
    ref = O.smooth_restated(xyz, xyz, kern, S.integ_factor(db), h2, v2, h3, v3)
    e = rel_l2(got, ref)
    print(f"smoothing ({which}) vs FP64 restatement: {e:.2e}; roughness reduced "
          f"{np.std(np.diff(kern[0])) / np.std(np.diff(got[0])):.1f}x")
    assert e < 1e-6
    const = S.smooth(db, xyz, np.full((1, n), 2.5, np.float32), sh, sv)
    assert np.abs(const - 2.5).max() < 2.5e-6
