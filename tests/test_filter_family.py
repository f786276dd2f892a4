"""Filter family of the FDK / FBP filter stage (CPU: the oracle's pieces).

Options beyond the reference's GPU filter (Shepp-Logan taps, full scan):
Ram-Lak taps (FBP_parallel.m:241-251, scaled by 1/2 to the S-L amplitude),
a Hamming smoothing window (FanProjection.m:265-270) and short-scan weights
(ParkFunction.m:6-16).  The reference holds no executable golden vectors for
them (the MATLAB forms are commented out or CPU-only), so each piece is pinned
to its published definition and to properties: the ramp's response at DC and
at Nyquist, numpy's Hamming window, Parker's complementarity
W(b, g) + W(b + pi + 2g, -g) = 1, and a short-scan reconstruction with the
amplitude and error of a full scan.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2


def _rl_matlab(pint, n):
    """FBP_parallel.m:241-251 (commented R-L form), 2n-1 taps, in double."""
    h = np.zeros(2 * n - 1)
    for i in range(n):
        if i == 0:
            h[n - 1] = 1.0 / (2 * pint) ** 2
        elif i % 2 == 0:
            h[n - 1 - i] = h[n - 1 + i] = 0.0
        else:
            h[n - 1 - i] = h[n - 1 + i] = -1.0 / (i * math.pi * pint) ** 2
    return h


def _park_matlab(beta, b0, gama, fan):
    """ParkFunction.m:6-16, line by line."""
    if b0 <= beta < b0 + fan - 2 * gama:
        return math.sin(math.pi / 4 * beta / (fan / 2 - gama)) ** 2
    if b0 + fan - 2 * gama <= beta <= b0 + math.pi - 2 * gama:
        return 1.0
    if b0 + math.pi - 2 * gama < beta <= b0 + math.pi + fan:
        return math.sin(math.pi / 4 * (math.pi + fan - beta) / (fan / 2 + gama)) ** 2
    return 0.0


def test_shepp_logan_kind_is_the_reference_taps(oracle):
    pint = np.float32(0.37)
    np.testing.assert_array_equal(oracle.ramp_taps(0, pint, 301), oracle.sl_filter(pint, 301))


def test_ram_lak_taps_are_half_the_matlab_form(oracle):
    pint = np.float32(0.4)
    g = oracle.ramp_taps(1, pint, 257)
    ref = (0.5 * _rl_matlab(float(pint), 257)).astype(np.float32)
    np.testing.assert_allclose(g, ref, rtol=1e-7, atol=0)
    assert g[256 + 2] == 0.0 and g[256 - 4] == 0.0


def test_ramp_responses_dc_and_nyquist(oracle):
    """Both taps are ramps (zero at DC); at Nyquist S-L = R-L * 2/pi (its sinc),
    so the two share one amplitude convention."""
    pint, n = np.float32(1.0), 8193
    sl = oracle.ramp_taps(0, pint, n).astype(np.float64)
    rl = oracle.ramp_taps(1, pint, n).astype(np.float64)
    alt = (-1.0) ** np.abs(np.arange(2 * n - 1) - (n - 1))
    assert abs(sl.sum()) < 1e-4 * sl[n - 1] and abs(rl.sum()) < 1e-4 * rl[n - 1]
    nyq_sl, nyq_rl = (sl * alt).sum(), (rl * alt).sum()
    assert nyq_rl == pytest.approx(0.25, rel=1e-4)                     # 1/(4 dP^2)
    assert nyq_sl / nyq_rl == pytest.approx(2 / math.pi, rel=1e-4)


def test_hamming_is_matlab_hamming(oracle):
    for m in (2, 10, 15, 64):
        np.testing.assert_allclose(oracle.hamming(m), np.hamming(m), rtol=0, atol=1e-15)
    assert oracle.hamming(1)[0] == 1.0


def test_parker_weights_follow_parkfunction(oracle):
    D = 300.0
    P = np.linspace(-120, 120, 41).astype(np.float32)
    fan = abs(math.atan(float(P[-1]) / D) - math.atan(float(P[0]) / D))
    beta = (np.arange(230) * (2 * math.pi / 360)).astype(np.float32)
    w = oracle.parker_weights(beta, P, D)
    for v in range(0, 230, 7):
        for p in range(0, 41, 5):
            ref = 2.0 * _park_matlab(float(beta[v]), float(beta[0]), math.atan(float(P[p]) / D), fan)
            assert w[v, p] == pytest.approx(ref, rel=1e-6, abs=1e-7)
    assert np.all(w >= 0) and np.all(w <= 2.0)


def test_parker_weights_are_complementary(oracle):
    """W(b, g) + W(b + pi + 2g, -g) = 1 for a scan starting at 0 (Parker)."""
    D = 400.0
    rng = np.random.default_rng(4)
    gmax = 0.3
    fan = 2 * gmax
    P = np.array([-D * math.tan(gmax), 0.0, D * math.tan(gmax)])
    for _ in range(200):
        g = rng.uniform(-gmax, gmax)
        b = rng.uniform(0, math.pi - 2 * g)       # conjugate at or beyond the scan end from fan - 2g on
        b2 = b + math.pi + 2 * g
        assert _park_matlab(b, 0.0, g, fan) + _park_matlab(b2, 0.0, -g, fan) == pytest.approx(1.0, abs=1e-12)
    # the oracle table at symmetric bins: conjugate rays of the middle bin (g = 0) are pi apart
    beta = np.array([0.0, 0.2, 0.2 + math.pi], np.float32)
    w = oracle.parker_weights(beta, P, D)
    assert w[1, 1] + w[2, 1] == pytest.approx(2.0, abs=1e-5)


def test_window_of_one_tap_is_identity(oracle, golden):
    P, xi, beta, D = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"], float(golden["fdk_D"])
    R = golden["fdk_proj"]
    for mode in (0, 1):
        base = oracle.fdk_filter(R, P, xi, D, mode=mode)
        np.testing.assert_array_equal(oracle.fdk_filter_ex(R, beta, P, xi, D, mode=mode, window=1), base)
        np.testing.assert_array_equal(oracle.fdk_filter_ex(R, beta, P, xi, D, mode=mode), base)


def test_window_is_the_smoothing_convolution(oracle, golden):
    P, beta = golden["f2_P150"], golden["f2_beta20"]
    sino = golden["f2_sino150"].astype(np.float32)
    base = oracle.fbpfan_filter_ex(sino, beta, P, 80.0, mode=0, kind=1).astype(np.float64)
    for m in (10, 15):
        h = np.hamming(m)
        c = m // 2
        ref = np.zeros_like(base)
        for i in range(m):
            k0 = i - c                       # out[p] += h[i] x[p + k0]
            if k0 >= 0:
                ref[:, :base.shape[1] - k0] += h[i] * base[:, k0:]
            else:
                ref[:, -k0:] += h[i] * base[:, :base.shape[1] + k0]
        ref /= h.sum()
        out = oracle.fbpfan_filter_ex(sino, beta, P, 80.0, mode=0, kind=1, window=m)
        assert rel_l2(out, ref) <= 1e-6


def test_short_scan_reconstruction_matches_full_scan(oracle):
    """Parker-weighted FBP over pi + fan angle has the amplitude and error of a
    full-turn FBP; without the weights the image is far off."""
    from ctgb import phantom
    n, D = 64, 200.0
    size = (64.0, 64.0)
    maxp = 1.1 * n * math.sqrt(2) / 2
    P = np.linspace(-maxp, maxp, 128)
    fan = abs(math.atan(P[-1] / D) - math.atan(P[0] / D))
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(8, seed=5)).numpy()
    yy, xx = np.mgrid[:n, :n]
    disc = (yy - n / 2 + 0.5) ** 2 + (xx - n / 2 + 0.5) ** 2 < (0.45 * n) ** 2
    db = 2 * math.pi / 180

    def rec(beta, short):
        sino = oracle.fan_fp(img, beta, P, size, D).astype(np.float32)
        rc = oracle.fbpfan_filter_ex(sino, beta, P, D, mode=0, short_scan=short)
        out = oracle.fbpfan_bp(rc, beta.astype(np.float32), P.astype(np.float32), size, (n, n), D)
        return np.linalg.norm((out - img)[disc]) / np.linalg.norm(img[disc]), out[disc].mean() / img[disc].mean()

    e_full, m_full = rec(np.arange(180) * db, False)
    short = np.arange(int(math.ceil((math.pi + fan) / db)) + 1) * db
    e_short, m_short = rec(short, True)
    e_none, m_none = rec(short, False)
    assert abs(m_short - 1) < 0.01 and abs(m_full - 1) < 0.01
    assert e_short < 1.2 * e_full + 0.01
    assert e_none > 3 * e_short
