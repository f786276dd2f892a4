"""IterativeFDK error slice (IterativeFDKerrCompute.cu) on the GPU, through the
C ABI, against the reference kernel fixtures and the oracle.

The GPU kernel carries the reference's double term and its float-rounded
double accumulation as float pairs, so an output can differ from the
reference's in its last bit when a term lands within ~2^-46 of a rounding
boundary of the running sum.  Tolerance: rel-L2 <= 1e-5 (FP32), and almost all
outputs bit-identical.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.mark.parametrize("t", [1, 10])
def test_dropin_matches_reference_fixtures(golden, t):
    from ctgb import ops
    g = {n: golden[f"ifdk_{n}"] for n in ("pic", "beta", "U", "P", "G", "size", "D")}
    ref = golden[f"ifdk_err_t{t}"]
    nz, ns, nt = g["pic"].shape
    out = ops.IterativeFDKerrCompute(g["pic"].ravel(), nt, ns, nz, g["size"], g["beta"], g["U"], g["P"],
                                     float(g["D"]), g["G"], t)
    assert out.dtype == np.float64 and out.size == ref.size
    assert rel_l2(out, ref.ravel()) <= TOL
    assert np.mean(out.astype(np.float32) == ref.ravel()) > 0.95


def _case(shape, size, pint, D, nviews, seed, beta=None):
    from scipy.ndimage import gaussian_filter
    from ctgb import phantom
    from ctgb.geometry import iterative_fdk_setup
    nz, ns, nt = shape
    b, U, P, G = iterative_fdk_setup(size, shape, pint=pint, D=D, n_views=nviews)
    if beta is not None:
        b = np.asarray(beta, np.float32)
    pic = phantom.ellipsoids_3d(nt, ns, nz, phantom.ellipsoid_params(10, seed=seed)).numpy()
    pic = gaussian_filter(pic, 0.8).astype(np.float32)
    return pic, b, U, P, G


@pytest.mark.parametrize("shape,size,t", [((24, 200, 30), (60.0, 60.0, 48.0), 14),
                                          ((20, 36, 28), (28.0, 36.0, 20.0), 0)])
def test_device_api_matches_oracle(oracle, shape, size, t):
    import torch
    from ctgb.device import iterfdk_err
    pic, b, U, P, G = _case(shape, size, 0.5, 110.0, 12, seed=21)
    out = iterfdk_err(torch.from_numpy(pic).cuda(), b, U, P, G, size, 110.0, t).cpu().numpy()
    ref = oracle.iterfdk_err(pic, b, U, P, G, size, 110.0, t)
    assert np.count_nonzero(ref) > ref.size // 3
    assert rel_l2(out, ref) <= TOL
    assert np.mean(out == ref) > 0.95


def test_grid_aligned_geometry_exercises_exact_index_paths(oracle):
    """Unit voxels, half-unit bins and views at multiples of pi/2 put many
    filter positions and slice positions exactly on integers: the FP32
    estimates must hand those to the exact double evaluation."""
    import torch
    from ctgb.device import iterfdk_err
    shape, size = (16, 24, 20), (20.0, 24.0, 16.0)
    beta = np.array([0.0, 0.5, 1.0, 1.5, 2.0, 3.0]) * math.pi
    pic, b, U, P, G = _case(shape, size, 0.5, 64.0, 6, seed=5, beta=beta)
    P = np.round(P * 2) / 2                                  # exact multiples of 0.5
    U = np.round(U).astype(np.float32)                       # integer depths
    for t in (3, 10):
        out = iterfdk_err(torch.from_numpy(pic).cuda(), b, U, P, G, size, 64.0, t).cpu().numpy()
        ref = oracle.iterfdk_err(pic, b, U, P, G, size, 64.0, t)
        assert rel_l2(out, ref) <= TOL
        assert np.mean(out == ref) > 0.95


def test_wide_slice_beyond_one_reference_launch(oracle):
    """s_length above 512: every (s, z) is computed once (the reference's
    residual launches only cover s, z < 512 or multiples of 512)."""
    import torch
    from ctgb.device import iterfdk_err
    shape, size = (4, 520, 16), (40.0, 52.0, 8.0)
    pic, b, U, P, G = _case(shape, size, 1.0, 120.0, 4, seed=8)
    out = iterfdk_err(torch.from_numpy(pic).cuda(), b, U, P, G, size, 120.0, 7).cpu().numpy()
    ref = oracle.iterfdk_err(pic, b, U, P, G, size, 120.0, 7)
    assert out.shape == (4, 4, 520)
    assert rel_l2(out, ref) <= TOL


def test_bad_arguments_raise():
    import torch
    from ctgb import _lib
    from ctgb.device import iterfdk_err
    pic = torch.zeros((4, 5, 6), device="cuda")
    b = np.array([0.1, 0.2], np.float32)
    U = np.array([1.0, 0.0], np.float32)
    P = np.array([-1.0, 0.0, 1.0])
    G = np.zeros(5)
    with pytest.raises(_lib.CTError):
        iterfdk_err(pic, b, U, P, G, (6.0, 5.0, 4.0), 50.0, 6)           # slice index out of range
    with pytest.raises(_lib.CTError):
        iterfdk_err(pic, b, U, P, G, (6.0, 5.0, 4.0), -1.0, 2)           # negative distance
