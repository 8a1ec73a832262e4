"""Unit checks of the oracle and product numerics against known values (CPU)."""
import math

import numpy as np
import pytest


def test_gll_points_and_weights():
    from oracle import oracle as O
    x, w = O.gll()
    assert np.allclose(x, [-1, -math.sqrt(3 / 7), 0, math.sqrt(3 / 7), 1], atol=1e-15)
    assert np.allclose(w, [0.1, 49 / 90, 32 / 45, 49 / 90, 0.1], atol=1e-15)


def test_derivation_matrix_known_values():
    from oracle import oracle as O
    from specfem3d_gb300 import meshgen
    d = O.derivation_matrices("f64")
    hp = d["hprime_d"].reshape(5, 5, order="F")
    assert abs(hp[0, 0] + 5.0) < 1e-14 and abs(hp[4, 4] - 5.0) < 1e-14  # -N(N+1)/4, N = 4
    assert np.allclose(hp.sum(axis=1), 0, atol=1e-13)     # derivative of a constant
    xg, _ = O.gll()
    assert np.allclose(hp @ xg, 1, atol=1e-13)            # derivative of x
    p = meshgen.derivation_matrices()
    assert np.array_equal(p["hprime_xx"], O.derivation_matrices("f32")["hprime_xx"])


def test_lagrange_interpolation():
    from oracle import oracle as O
    from specfem3d_gb300 import meshgen
    for xi in (-1.0, -0.3, 0.0, 0.77, 1.0):
        h, hp = O.lagrange_any(xi)
        h2, hp2 = meshgen.lagrange(xi)
        assert abs(h.sum() - 1) < 1e-13 and abs(hp.sum()) < 1e-12
        assert np.allclose(h, h2, atol=1e-14) and np.allclose(hp, hp2, atol=1e-12)


def test_source_time_functions():
    from oracle import oracle as O
    from specfem3d_gb300 import meshgen
    assert abs(O.lib().orc_stf(1, 0.0, 2.0) - 1.0) < 1e-15          # Ricker peak
    assert abs(O.lib().orc_stf(0, 0.0, 5.0) - 0.5) < 1e-15          # Heaviside midpoint
    t = np.linspace(-1, 1, 11)
    for k, kind, p in ((1, "ricker", 2.0), (0, "heaviside", 5.0), (2, "gaussian", 1.0)):
        a = np.array([O.lib().orc_stf(k, float(tt), p) for tt in t])
        assert np.allclose(a, meshgen.stf_value(kind, t, p), rtol=1e-13, atol=1e-15)


def test_time_step_rule():
    from specfem3d_gb300 import configs
    # reference example log: min GLL distance 642.7 m, vmax 2800 -> suggested 0.114772588
    dmin = configs.GLL_MIN_SPACING * 3722.2222
    assert abs(0.5 * dmin / 2800.0 - 0.114772588) < 1e-5
    assert configs.significant_dt(0.0734815) == 0.073
    assert configs.significant_dt(0.012847) == 0.0125
    assert configs.homogeneous_block()["dt"] == 0.0125


def test_attenuation_band_matches_reference_log():
    """EXAMPLES/benchmarks/attenuation/viscoelastic/REF_SEIS/output_generate_databases.txt:
    minimum period resolved 2.1090772E-02 -> period band 2.0879865E-02 / 1.174161 s,
    central frequency 6.386638 Hz."""
    from specfem3d_gb300 import attenuation
    ts, fc, minp, maxp = attenuation.band(2.1090772e-2)
    assert abs(minp - 2.0879865e-2) < 1e-8
    assert abs(maxp - 1.174161) < 1e-6
    assert abs(fc - 6.386638) < 1e-5


def test_attenuation_fit_reaches_constant_q():
    from specfem3d_gb300 import attenuation
    ts, fc, minp, maxp = attenuation.band(0.2)
    for Q in (20.0, 150.0):
        te = attenuation.tau_eps_for_q(Q, ts, minp, maxp)
        w = 2 * math.pi * np.logspace(math.log10(1 / maxp), math.log10(1 / minp), 50)
        den = 1 + (w[:, None] * ts[None, :]) ** 2
        A = ((1 + w[:, None] ** 2 * te * ts) / den).sum(1)
        B = (w[:, None] * (te - ts) / den).sum(1)
        assert np.max(np.abs(B / A * Q - 1)) < 0.1


def test_get_global_restatement_matches_brute_force():
    from oracle import oracle as O
    rng = np.random.default_rng(3)
    pts = rng.integers(0, 4, size=(300, 3)).astype(np.float64) * 0.5
    ib = np.zeros(300, np.int32)
    xs, ys, zs = (np.ascontiguousarray(pts[:, c]) for c in range(3))
    n = O.lib().orc_get_global(300, xs.ctypes.data, ys.ctypes.data, zs.ctypes.data, ib.ctypes.data, 1e-9)
    # brute force: first appearance numbering of distinct points
    seen = {}
    exp = []
    for p in map(tuple, pts):
        if p not in seen:
            seen[p] = len(seen) + 1
        exp.append(seen[p])
    assert n == len(seen)
    assert np.array_equal(ib, np.array(exp))
