"""The oracle's restatement of the reference's adjoint-source tools on cases with a
known answer (no reference golden vectors exist for these tools): the waveform
adjoint source of identical traces is zero; inside the flat part of its window it
is the residual; the traveltime adjoint source of a pulse is -v tw / (dt sum tw v^2),
so its inner product with the synthetic velocity over the window is -1; the
amplitude adjoint source's inner product with the synthetic is +1; the kernel sum
of k and -k is zero and masks multiply."""
import numpy as np

from oracle import oracle as O


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
