"""Curved-detector short-scan FDK (ImplementUI.cu) on the GPU, through the C
ABI, against the reference kernel fixtures and the oracle.

The filter's weights run in double as the reference orders them (NaN rows
included); its convolution runs on float pairs and the filtered rows are
stored as float.  The backprojection computes the gamma position in double and
the per-voxel work in FP32 with float-pair sums.  Tolerance: rel-L2 <= 1e-5.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _smooth_R(c, seed):
    """Smooth projection-like data [beta][xi][gamma] with a little noise."""
    rng = np.random.default_rng(seed)
    b, x, g = np.meshgrid(c["beta"], c["xi"], c["gama"], indexing="ij")
    gmax = np.abs(c["gama"]).max()
    R = (1.0 + 0.3 * np.cos(b + 0.2 * x / (np.abs(c["xi"]).max() + 1))) * np.clip(1 - (g / gmax) ** 2, 0, None)
    return R + 0.01 * rng.standard_normal(R.shape)


def _small_case():
    gama = -(np.arange(200) - 99.5) * 0.004          # descending, fan 0.796 rad
    xi = (np.arange(12) - 5.5) * 2.0
    fan = abs(gama[-1] - gama[0])
    b0 = 0.0
    beta = b0 + np.arange(150) * ((np.pi + fan) / 149)  # one short scan
    return dict(gama=gama, xi=xi, beta=beta, b0=b0, maxg=fan, D=110.0, ds2d=200.0,
                size=np.array([48, 44, 11], np.int32), z_length=9)


def test_filter_rows_match_reference(golden):
    import torch
    from ctgb.device import fdkui_filter
    from ctgb.geometry import curved_fdk_case
    c = curved_fdk_case("filter")
    R = np.random.default_rng(77).random((len(c["beta"]), 80, 936))
    out = fdkui_filter(torch.from_numpy(R).cuda(), c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"],
                       c["ds2d"]).cpu().numpy()
    rows = out[golden["ui_filter_bs"], golden["ui_filter_xs"]].astype(np.float64)
    ref = golden["ui_filter_rows"]
    nan = np.isnan(ref)
    np.testing.assert_array_equal(np.isnan(rows), nan)      # the reference's NaN rows, reproduced
    assert rel_l2(rows[~nan], ref[~nan]) <= TOL


def test_bp_matches_reference(golden):
    import torch
    from ctgb.device import fdkui_bp
    from ctgb.geometry import curved_fdk_case
    c = curved_fdk_case("bp")
    rc = np.random.default_rng(78).random((len(c["beta"]), len(c["xi"]), len(c["gama"]))) - 0.5
    out = fdkui_bp(torch.from_numpy(rc.astype(np.float32)).cuda(), c["xi"], c["gama"], c["beta"], c["D"], c["ds2d"],
                   c["size"], c["z_length"]).cpu().numpy()
    ref = golden["ui_bp"]
    assert out.shape == ref.shape
    assert rel_l2(out, ref) <= TOL


def test_dropin_pipeline_matches_oracle(oracle):
    from ctgb import ops
    c = _small_case()
    R = _smooth_R(c, 3)
    rcov = oracle.fdkui_filter(R, c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"], c["ds2d"])
    ref = oracle.fdkui_bp(rcov, c["size"], c["z_length"], c["beta"], c["D"], c["ds2d"], c["gama"], c["xi"])
    assert np.isfinite(ref).all() and np.count_nonzero(ref) > ref.size // 2
    out = ops.ImplementUI(R.ravel(), c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"], c["ds2d"],
                          c["size"].astype(np.float64), c["z_length"])
    assert out.dtype == np.float64 and out.size == ref.size
    assert rel_l2(out, ref.ravel()) <= TOL


def test_stages_match_oracle_on_ascending_domains(oracle):
    """Ascending gamma and xi domains and a start angle off zero."""
    import torch
    from ctgb.device import fdkui_bp, fdkui_filter
    c = _small_case()
    c["gama"] = c["gama"][::-1].copy()
    c["xi"] = c["xi"][::-1].copy()
    c["b0"] = 0.3
    c["beta"] = c["beta"] + 0.3
    R = _smooth_R(c, 4)
    rcov = oracle.fdkui_filter(R, c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"], c["ds2d"])
    got = fdkui_filter(torch.from_numpy(R).cuda(), c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"],
                       c["ds2d"])
    fin = np.isfinite(rcov)
    np.testing.assert_array_equal(np.isfinite(got.cpu().numpy()), fin)
    assert rel_l2(got.cpu().numpy()[fin], rcov[fin]) <= TOL
    rcov = np.where(fin, rcov, 0.0)
    ref = oracle.fdkui_bp(rcov, c["size"], c["z_length"], c["beta"], c["D"], c["ds2d"], c["gama"], c["xi"])
    out = fdkui_bp(torch.from_numpy(rcov.astype(np.float32)).cuda(), c["xi"], c["gama"], c["beta"], c["D"],
                   c["ds2d"], c["size"], c["z_length"]).cpu().numpy()
    assert rel_l2(out, ref) <= TOL


def test_bad_arguments_raise():
    import torch
    from ctgb import _lib
    from ctgb.device import fdkui_bp
    c = _small_case()
    rc = torch.zeros((len(c["beta"]), len(c["xi"]), len(c["gama"])), dtype=torch.float32, device="cuda")
    with pytest.raises(_lib.CTError):
        fdkui_bp(rc, c["xi"], c["gama"], c["beta"], -1.0, c["ds2d"], c["size"], c["z_length"])
    bad = c["size"].copy()
    bad[0] = 0
    with pytest.raises(_lib.CTError):
        fdkui_bp(rc, c["xi"], c["gama"], c["beta"], c["D"], c["ds2d"], bad, c["z_length"])
