"""The oracle's restatement of the reference's adjoint-source tools.

Pinned on the reference's own golden vectors: the traveltime adjoint sources of
EXAMPLES/reproducible_study/sensitivity_kernels_liutromp2006/REF_ADJ_SRC (P, PS+SP,
S, SS windows, made by utils/adjoint_sources/traveltime from that study's
REF_SEIS traces; tests/golden/liutromp2006_adjsrc.npz, written by
tests/golden/make_adjsrc_fixture.py) are reproduced to the 7 significant digits
the files carry (measured 7e-8 to 1.7e-7 relative L2).  Known answers for the
other tools: the waveform adjoint source of identical traces is zero; inside the
flat part of its window it is the residual; the traveltime adjoint source of a
pulse is -v tw / (dt sum tw v^2), so its inner product with the synthetic velocity
over the window is -1; the amplitude adjoint source's inner product with the
synthetic is +1; the kernel sum of k and -k is zero and masks multiply."""
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import oracle as O

CASES = ("P", "PSSP", "S", "SS")


def liutromp_case(case):
    """(syn (1, 3, nstep), dt, t0, ts, te, component, reference adjoint source (nstep,))."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "liutromp2006_adjsrc.npz"))
    run = str(g["run_" + case])
    ts, te, comp = g["win_" + case]
    comp = int(comp)
    syn = np.zeros((1, 3, g["syn_" + run].size))
    syn[0, comp - 1] = g["syn_" + run]
    return syn, float(g["dt_" + run]), float(g["t0_" + run]), float(ts), float(te), comp, g["adj_" + case]


@pytest.mark.parametrize("case", CASES)
def test_traveltime_adjoint_source_matches_reference_golden(case):
    syn, dt, t0, ts, te, comp, ref = liutromp_case(case)
    adj, norms = O.adjoint_source(1, syn, None, dt, t0, ts, te, comp)
    a = adj[0, comp - 1]
    assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < 1e-6
    assert not np.delete(adj[0], comp - 1, axis=0).any()
    assert norms[0, comp - 1] > 0


def _pulse(nstep=800, dt=0.005):
    t = np.arange(nstep) * dt
    s = np.exp(-((t - 2.0) / 0.2) ** 2) * np.cos(12 * t)
    syn = np.stack([np.stack([s, 0.5 * s, -s])] * 2)
    return syn, dt


def test_waveform_adjoint_source():
    syn, dt = _pulse()
    adj, norms = O.adjoint_source(0, syn, syn, dt, 0.0, 1.0, 3.0)
    assert not adj.any() and not norms.any()
    dat = syn * 0.9
    adj, norms = O.adjoint_source(0, syn, dat, dt, 0.0, 1.0, 3.0)
    j = int(2.0 / dt)                      # the middle of the window: taper weight 1
    assert np.allclose(adj[:, :, j], (syn - dat)[:, :, j])
    assert (norms > 0).all()


def test_traveltime_and_amplitude_normalisation():
    syn, dt = _pulse()
    adj, norms = O.adjoint_source(1, syn, None, dt, 0.0, 1.0, 3.0)
    v = np.gradient(syn, dt, axis=2)
    ip = dt * np.sum(adj * v, axis=2)
    assert np.allclose(ip, -1.0, atol=1e-3)
    adj, norms = O.adjoint_source(2, syn, None, dt, 0.0, 1.0, 3.0, component=3)
    ip = dt * np.sum(adj * syn, axis=2)
    assert np.allclose(ip[:, 2], 1.0) and not adj[:, :2].any()


def test_sum_kernels():
    k = np.linspace(-1, 1, 500).astype(np.float32)
    total, norms = O.sum_kernels([k, -k])
    assert not total.any() and np.allclose(norms, np.sum(k.astype(np.float64) ** 2))
    m = (np.arange(500) % 2).astype(np.float32)
    total, _ = O.sum_kernels([k, k], [m, m])
    assert np.array_equal(total, 2 * k.astype(np.float64) * m)
