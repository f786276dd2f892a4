"""ct_FBPfan_noalloc: the 2D fan FBP for callers that may not allocate device
memory while they run (services that reserve all device memory once at
start-up, or hosts whose framework owns the device pool, where a raw
cudaMalloc would bypass its accounting and cudaFree would synchronise the
device).  It takes device buffers for the sinogram and the image and keeps
everything else in one library-owned 8 MiB device array.

This test calls it through the C ABI twice in a row, on two geometries, and
checks each result against the oracle and against the allocating entry point
ct_FBPfan (rel-L2 <= 1e-5, FP32 against the reference's FP64 arithmetic).  It
also checks that the second call leaves the device's free memory unchanged
(the first call may commit the library's array: CUDA loads modules lazily).
Named to run after every other test file."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5
CASES = [(64, 90, 128, 200.0, 31), (48, 120, 150, 150.0, 32)]


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else C.c_void_p(a.data_ptr())


def _prepare(oracle, n, nviews, nbins, rscan, seed):
    from ctgb import ops, phantom
    from ctgb.geometry import fan_config
    g = fan_config(n, nviews, nbins, rscan, float(n))
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(10, seed=seed)).numpy()
    sino = oracle.fan_fp(img, g.beta, g.P, g.size, g.D).astype(np.float32)
    beta = g.beta.astype(np.float32)
    P = g.P.astype(np.float32)
    size = np.asarray(g.size, np.float64)
    ref_oracle = oracle.fbpfan(sino, beta, P, size, (g.ns, g.nt), g.D, filter_mode=1).ravel()
    ref_alloc = ops.FBPfan(sino.ravel(), beta, P, size, g.nt, g.ns, g.D)          # allocating entry point
    d_R = torch.from_numpy(sino.ravel().copy()).cuda()
    d_img = torch.full((g.ns * g.nt,), float("nan"), dtype=torch.float32, device="cuda")
    return dict(g=g, beta=beta, P=P, size=size, ref_oracle=ref_oracle, ref_alloc=ref_alloc, d_R=d_R, d_img=d_img)


def _call(lib, c, stream):
    g = c["g"]
    return lib.ct_FBPfan_noalloc(_ptr(c["d_img"]), _ptr(c["d_R"]), _ptr(c["P"]), _ptr(c["beta"]), len(c["beta"]),
                                 len(c["P"]), _ptr(c["size"]), g.nt, g.ns, float(g.D), stream)


def test_noalloc_fbp_matches_oracle_twice_without_allocating(oracle):
    from ctgb import _lib
    lib = _lib.load()
    cases = [_prepare(oracle, *k) for k in CASES]      # every torch / library allocation happens here
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert _call(lib, cases[0], stream) == 0, lib.ct_last_error()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert _call(lib, cases[1], stream) == 0, lib.ct_last_error()
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before, (free_before, free_after)
    for c in cases:
        out = c["d_img"].cpu().numpy()
        assert np.isfinite(out).all()
        assert rel_l2(out, c["ref_oracle"]) <= TOL
        assert rel_l2(out, c["ref_alloc"]) <= TOL


def test_noalloc_rejects_sizes_beyond_its_array():
    from ctgb import _lib
    lib = _lib.load()
    nb, npd = 2048, 1200            # the filtered sinogram alone needs 9.8 MB > 8 MiB
    beta = (np.arange(1, nb + 1) * 2 * np.pi / nb).astype(np.float32)
    P = np.linspace(-90, 90, npd).astype(np.float32)
    size = np.array([100.0, 100.0])
    d_R = torch.zeros(nb * npd, dtype=torch.float32, device="cuda")
    d_img = torch.zeros(64 * 64, dtype=torch.float32, device="cuda")
    st = lib.ct_FBPfan_noalloc(_ptr(d_img), _ptr(d_R), _ptr(P), _ptr(beta), nb, npd, _ptr(size), 64, 64, 400.0,
                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 1 and b"8 MiB" in lib.ct_last_error()
