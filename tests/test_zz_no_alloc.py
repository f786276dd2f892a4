"""ct_FBPfan_noalloc: the 2D fan FBP for callers that may not allocate device
memory (memory reserved once at start-up, or a framework that owns the device
pool).  It takes device buffers for the sinogram and the image and keeps
everything else in one library-owned device array; this test calls it through
the C ABI twice in a row, on two different geometries, and checks each result
against the allocating entry point ct_FBPfan.  Named to run after every other
test file."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _case(n, nviews, nbins, rscan, seed):
    from ctgb import phantom
    from ctgb.geometry import fan_config
    from oracle.oracle import Oracle
    g = fan_config(n, nviews, nbins, rscan, float(n))
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(10, seed=seed)).numpy()
    sino = Oracle().fan_fp(img, g.beta, g.P, g.size, g.D).astype(np.float32)
    return g, sino


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else C.c_void_p(a.data_ptr())


def test_noalloc_fbp_matches_allocating_entry_point_twice():
    from ctgb import _lib, ops
    lib = _lib.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, nviews, nbins, rscan, seed in [(64, 90, 128, 200.0, 31), (48, 120, 150, 150.0, 32)]:
        g, sino = _case(n, nviews, nbins, rscan, seed)
        beta = g.beta.astype(np.float32)
        P = g.P.astype(np.float32)
        size = np.asarray(g.size, np.float64)
        ref = ops.FBPfan(sino.ravel(), beta, P, size, g.nt, g.ns, g.D)          # allocating entry point
        d_R = torch.from_numpy(sino.ravel().copy()).cuda()
        d_img = torch.full((g.ns * g.nt,), float("nan"), dtype=torch.float32, device="cuda")
        st = lib.ct_FBPfan_noalloc(_ptr(d_img), _ptr(d_R), _ptr(P), _ptr(beta), len(beta), len(P), _ptr(size),
                                   g.nt, g.ns, float(g.D), stream)
        assert st == 0, lib.ct_last_error()
        torch.cuda.synchronize()
        out = d_img.cpu().numpy()
        assert np.isfinite(out).all()
        assert rel_l2(out, ref) <= TOL


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
