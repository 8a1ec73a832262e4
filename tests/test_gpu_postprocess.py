"""Misfit post-processing on the device (sf3d_adjoint_sources, sf3d_sum_kernels)
against the oracle's restatement of the reference tools
(utils/adjoint_sources/*/create_adjsrc_*.f90, src/tomography/sum_kernels.f90):
FP64 on both sides; adjoint sources and norms to 1e-12 relative (the device sums
each trace's norm in another order), kernel sums bit-exact (same per-value order),
norms to 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _traces(nrec=17, nstep=600, seed=3):
    rng = np.random.default_rng(seed)
    t = np.arange(nstep) * 0.01
    syn = np.zeros((nrec, 3, nstep))
    for r in range(nrec):
        for c in range(3):
            syn[r, c] = rng.normal() * np.exp(-((t - 2.5 - 0.2 * rng.random()) / 0.3) ** 2) * np.sin(9 * t + r)
    dat = syn + 0.05 * rng.standard_normal(syn.shape) * np.abs(syn).max()
    return syn, dat


@pytest.mark.parametrize("kind", ["waveform", "traveltime", "amplitude"])
@pytest.mark.parametrize("component", [0, 2])
def test_adjoint_sources_match_oracle(gpulib, kind, component):
    from oracle import oracle as O
    from specfem3d_gb300 import postprocess as P
    syn, dat = _traces()
    args = (0.01, -0.2, 1.1, 4.37)
    adj, norms = P.adjoint_sources(kind, syn, dat, *args, component=component)
    ref, rn = O.adjoint_source(P.KINDS[kind], syn, dat, *args, component=component)
    assert np.abs(ref).max() > 0
    assert np.linalg.norm(adj - ref) <= 1e-12 * np.linalg.norm(ref)
    assert np.allclose(norms, rn, rtol=1e-12, atol=0)
    if component:
        keep = np.zeros(3, bool)
        keep[component - 1] = True
        assert not adj[:, ~keep].any()


@pytest.mark.parametrize("case", ["P", "PSSP", "S", "SS"])
def test_traveltime_adjoint_sources_match_reference_golden(gpulib, case):
    """The reference's traveltime adjoint sources of the Liu & Tromp (2006) study
    (REF_ADJ_SRC, tests/golden/liutromp2006_adjsrc.npz) from its REF_SEIS traces, on
    the device: to the 7 significant digits the files carry."""
    from test_postprocess_oracle import liutromp_case
    from specfem3d_gb300 import postprocess as P
    syn, dt, t0, ts, te, comp, ref = liutromp_case(case)
    adj, norms = P.adjoint_sources("traveltime", syn, None, dt, t0, ts, te, component=comp)
    a = adj[0, comp - 1]
    assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < 1e-6
    assert norms[0, comp - 1] > 0


def test_adjoint_sources_reject_bad_windows(gpulib):
    from specfem3d_gb300 import abi, postprocess as P
    syn, dat = _traces(nrec=2, nstep=100)
    with pytest.raises(abi.SF3DError, match="outside the trace"):
        P.adjoint_sources("waveform", syn, dat, 0.01, 0.0, 0.5, 2.0)
    with pytest.raises(abi.SF3DError, match="shorter than 20"):
        P.adjoint_sources("waveform", syn, dat, 0.01, 0.0, 0.2, 0.3)


@pytest.mark.parametrize("masked", [False, True])
def test_sum_kernels_match_oracle(gpulib, masked):
    from oracle import oracle as O
    from specfem3d_gb300 import postprocess as P
    rng = np.random.default_rng(7)
    n = 125 * 3001
    ks = [rng.standard_normal(n).astype(np.float32) * 10.0 ** q for q in range(-2, 3)]
    ms = [(rng.random(n) > 0.1).astype(np.float32) for _ in ks] if masked else None
    total, total32, norms = P.sum_kernels(ks, ms)
    ref, rn = O.sum_kernels(ks, ms)
    assert np.array_equal(total, ref)
    assert np.array_equal(total32, ref.astype(np.float32))
    assert np.allclose(norms, rn, rtol=1e-12, atol=0)
