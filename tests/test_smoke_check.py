"""The comparison that __graft_entry__.smoke() applies to the device run, exercised on
CPU with oracle output standing in for the device output: it passes on identical
fields, fails on a field perturbed by 0.1 % at one point, fails on a field of the
magnitude of the smoke run that differs by values whose squares underflow float32,
and fails when the oracle field is still at rest."""
import numpy as np
import pytest

import __graft_entry__ as G


@pytest.fixture(scope="module")
def smoke_run():
    from oracle import oracle as O
    from specfem3d_gb300 import configs, meshgen
    O.build()
    cfg = configs.small_layered(nstep=400, attenuation=True)
    db = meshgen.build_database(cfg)
    sim = O.make_sim(db, cfg, "f32", nthreads=2)
    sim.step(cfg["nstep"])
    return O.seismograms(sim), sim.get("displ")


def test_smoke_run_reaches_a_propagated_wave(smoke_run):
    s, d = smoke_run
    # the Ricker source (t0 = 0.6 s) has acted: the field is far from zero and from
    # the float32 underflow range of the old comparison
    assert np.abs(d).max() > 1e-17 and np.abs(s).max() > 1e-17
    assert G.compare_with_oracle(s, s, d, d) == (0.0, 0.0)


def test_smoke_comparison_catches_a_perturbed_field(smoke_run):
    s, d = smoke_run
    d2 = np.array(d, copy=True)
    d2[int(np.argmax(np.abs(d)))] *= 1.001
    with pytest.raises(AssertionError, match="displacement"):
        G.compare_with_oracle(s, s, d2, d)
    s2 = np.array(s, copy=True)
    s2[..., -1] += 1e-3 * np.abs(s).max()
    with pytest.raises(AssertionError, match="seismograms"):
        G.compare_with_oracle(s2, s, d, d)


def test_smoke_comparison_does_not_underflow():
    # a field of ~5e-18 m with differences of ~5e-21 (1e-3 relative): the squares of
    # the differences (~2.5e-41) are float32 subnormals, so a float32 norm loses them;
    # the float64 comparison reports the true 1e-3 and fails the 5e-5 bar
    rng = np.random.default_rng(0)
    ref = (5e-18 * rng.standard_normal(5000)).astype(np.float32)
    dev = (ref.astype(np.float64) * (1.0 + 1e-3 * rng.standard_normal(5000))).astype(np.float32)
    _, errd = G.compare_with_oracle(ref, ref, dev, ref, tol=1.0)
    assert 5e-4 < errd < 2e-3
    with pytest.raises(AssertionError, match="displacement"):
        G.compare_with_oracle(ref, ref, dev, ref)


def test_smoke_comparison_rejects_a_field_at_rest():
    z = np.zeros(30, np.float32)
    with pytest.raises(AssertionError, match="zero"):
        G.compare_with_oracle(z, z, z, z)
