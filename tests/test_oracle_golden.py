"""The FP64 oracle against the reference's own kernels (golden fixtures).

The fixtures were produced by running the reference kernel functions,
compiled as host code, on these inputs (tests/golden/make_golden.py).  The
oracle restates the same arithmetic in the same precision, so on one host
they agree bit for bit; the tolerance admits last-bit differences of another
libm.
"""
import numpy as np
import pytest

from conftest import rel_l2

TOL = 1e-6


def _cone(golden, k):
    g = {n: golden[f"cone_{k}_{n}"] for n in ("vol", "proj", "R", "bp", "P", "xi", "beta", "size", "D")}
    g["D"] = float(g["D"])
    return g


@pytest.mark.parametrize("case", ["a", "b", "c"])
def test_cone_fp_matches_reference(oracle, golden, case):
    g = _cone(golden, case)
    out = oracle.cone_fp(g["vol"], g["beta"], g["P"], g["xi"], g["size"], g["D"])
    assert out.shape == g["proj"].shape
    assert rel_l2(out, g["proj"]) <= TOL
    assert np.mean(out == g["proj"]) > 0.99


@pytest.mark.parametrize("case", ["a", "b", "c"])
def test_cone_bp_matches_reference(oracle, golden, case):
    g = _cone(golden, case)
    out = oracle.cone_bp(g["R"], g["beta"], g["P"], g["xi"], g["size"], g["D"], g["vol"].shape)
    assert rel_l2(out, g["bp"]) <= TOL
    assert np.mean(out == g["bp"]) > 0.99


def test_fdk_stages_match_reference(oracle, golden):
    P, xi, beta = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"]
    size, D = golden["fdk_size"], float(golden["fdk_D"])
    proj = golden["fdk_proj"]
    # taps of GFunction
    g = oracle.sl_filter(np.float32(abs(P[1] - P[0])), len(P))
    assert np.array_equal(g, golden["fdk_G"])
    # in-place cosine pre-weight
    w = oracle.fdk_weight_apply(proj, P, xi, D)
    assert np.array_equal(w, golden["fdk_weighted"])
    # weight + convolution (clean semantics equal the race-free reference run)
    conv = oracle.fdk_filter(proj, P, xi, D, mode=0)
    assert rel_l2(conv, golden["fdk_conv"]) <= TOL
    # weighted bilinear backprojection incl. the sticky out-of-detector value
    bp = oracle.fdk_bp(golden["fdk_conv"], beta, P, xi, size, D, (14, 16, 16), sticky=1)
    assert rel_l2(bp, golden["fdk_bp"]) <= TOL


def test_fdk_sticky_quirk_is_exercised(oracle, golden):
    """The FDK fixture's volume extends beyond the cone coverage, so the
    reference's sticky value differs from a zero fill there."""
    P, xi, beta = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"]
    size, D = golden["fdk_size"], float(golden["fdk_D"])
    zero = oracle.fdk_bp(golden["fdk_conv"], beta, P, xi, size, D, (14, 16, 16), sticky=0)
    assert rel_l2(zero, golden["fdk_bp"]) > 1e-3


def test_fan_and_parallel_fp_match_reference(oracle, golden):
    img, size = golden["f2_img"], golden["f2_size"]
    beta, P = golden["f2_beta"], golden["f2_P"]
    assert rel_l2(oracle.fan_fp(img, beta, P, size, 80.0), golden["f2_fp"]) <= TOL
    assert rel_l2(oracle.fan_fp(img, beta, golden["f2_P_wide"], size, 80.0), golden["f2_fp_wide"]) <= TOL
    assert rel_l2(oracle.par_fp(img, beta, P, size), golden["f2_par"]) <= TOL


def test_fan_bp_matches_reference(oracle, golden):
    size = golden["f2_size"]
    out = oracle.fan_bp(golden["f2_fp"].astype(np.float32), golden["f2_beta"].astype(np.float32),
                        golden["f2_P"].astype(np.float32), size, (30, 32), 80.0)
    assert rel_l2(out, golden["f2_bp"]) <= TOL


def test_fbpfan_stages_match_reference(oracle, golden):
    size, P, beta = golden["f2_size"], golden["f2_P150"], golden["f2_beta20"]
    sino = golden["f2_sino150"]
    assert np.array_equal(oracle.fbpfan_weight_apply(sino, P, 80.0), golden["f2_fbp_weighted"])
    assert rel_l2(oracle.fbpfan_filter(sino, P, 80.0, mode=0), golden["f2_fbp_conv"]) <= TOL
    out = oracle.fbpfan_bp(golden["f2_fbp_conv"], beta, P, size, (30, 32), 80.0)
    assert rel_l2(out, golden["f2_fbp_bp"]) <= TOL


def test_fbpparallel_matches_reference(oracle, golden):
    out = oracle.fbppar(golden["f2_par"].astype(np.float32), golden["f2_beta"].astype(np.float32),
                        golden["f2_P"].astype(np.float32), golden["f2_size"], (30, 32))
    assert rel_l2(out, golden["f2_fbppar"]) <= TOL


@pytest.mark.parametrize("t", [1, 10])
def test_iterative_fdk_error_matches_reference(oracle, golden, t):
    g = {n: golden[f"ifdk_{n}"] for n in ("pic", "beta", "U", "P", "G", "size", "D")}
    ref = golden[f"ifdk_err_t{t}"]
    out = oracle.iterfdk_err(g["pic"], g["beta"], g["U"], g["P"], g["G"], g["size"], float(g["D"]), t - 1)
    assert np.count_nonzero(ref) > ref.size // 2        # the case exercises the gathers
    assert rel_l2(out, ref) <= TOL
    assert np.mean(out == ref) > 0.99


def test_curved_fdk_filter_rows_match_reference(oracle, golden):
    """ImplementUI.cu PreWeightFiltration at its fixed 936 x 80 launch shape
    (run by the checker with a real barrier per block), 25 rows over five views
    across the Parker regions."""
    from ctgb.geometry import curved_fdk_case
    c = curved_fdk_case("filter")
    R = np.random.default_rng(77).random((len(c["beta"]), 80, 936))
    out = oracle.fdkui_filter(R, c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"], c["ds2d"])
    rows = out[golden["ui_filter_bs"], golden["ui_filter_xs"]]
    ref = golden["ui_filter_rows"]
    # the first view's rows are NaN in the reference: with a symmetric detector the
    # edge gamma is half the fan angle, (b0 + fan) - 2 gamma rounds above b0, and the
    # Parker ramp divides by fan/2 - gamma = 0 (ImplementUI.cu:54-55)
    nan = np.isnan(ref)
    assert nan[:5].all() and not nan[5:].any()
    np.testing.assert_array_equal(np.isnan(rows), nan)
    assert rel_l2(rows[~nan], ref[~nan]) <= 1e-12


def test_curved_fdk_bp_matches_reference(oracle, golden):
    from ctgb.geometry import curved_fdk_case
    c = curved_fdk_case("bp")
    rc = np.random.default_rng(78).random((len(c["beta"]), len(c["xi"]), len(c["gama"]))) - 0.5
    out = oracle.fdkui_bp(rc, c["size"], c["z_length"], c["beta"], c["D"], c["ds2d"], c["gama"], c["xi"])
    ref = golden["ui_bp"]
    assert np.count_nonzero(ref) > ref.size // 2
    assert rel_l2(out, ref) <= 1e-12
