"""Edge cases of the drop-in operators on the GPU against the oracle:
volumes one voxel thick along each axis, a single view, a 2 x 2 detector,
views on the axes, odd and prime sizes, and rejected arguments (empty
domains, sizes beyond the index range) that must fail with CT_ERR_ARG
before any device work."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = [
    # (nz, ns, nt), views, LP, LXigama
    ((1, 1, 1), [0.0], 2, 2),
    ((3, 1, 5), [0.0], 3, 2),
    ((2, 7, 1), [0.0, np.pi / 2], 5, 3),
    ((1, 6, 6), [np.pi / 4, np.pi, 1.5 * np.pi], 9, 2),
    ((7, 11, 13), [0.3, 1.9, 3.1, 4.4, 5.9], 17, 7),
]


@pytest.mark.parametrize("shape,views,npd,nx", CASES)
def test_cone_fp_bp_small_and_degenerate(oracle, shape, views, npd, nx):
    from ctgb import ops
    nz, ns, nt = shape
    rng = np.random.default_rng(nz * 100 + ns * 10 + nt)
    vol = rng.random(shape).astype(np.float32) + 0.1
    size = np.array([nt * 1.0, ns * 0.9, nz * 1.1])
    beta = np.asarray(views, np.float32)
    P = np.linspace(-0.6 * max(nt, ns), 0.6 * max(nt, ns), npd).astype(np.float32)
    xi = np.linspace(-0.55 * nz, 0.55 * nz, nx).astype(np.float32)
    D = 4.0 * max(size)
    ref = oracle.cone_fp(vol, beta, P, xi, size, D)
    out = ops.ProjectionCone_3D(vol.ravel(), nt, ns, nz, size, beta, P, xi, D)
    if np.abs(ref).max() == 0:
        assert np.abs(out).max() == 0
    else:
        assert rel_l2(out, ref.ravel()) <= TOL
    R = rng.random(ref.shape).astype(np.float32)
    bref = oracle.cone_bp(R, beta, P, xi, size, D, shape)
    bout = ops.Backprojection3D(R.ravel(), xi, P, beta, D, size, nt, ns, nz)
    if np.abs(bref).max() == 0:
        assert np.abs(bout).max() == 0
    else:
        assert rel_l2(bout, bref.ravel()) <= TOL


@pytest.mark.parametrize("n,nviews,nbins", [(1, 1, 2), (2, 3, 4), (13, 7, 19)])
def test_fan_fp_bp_small(oracle, n, nviews, nbins):
    from ctgb import ops
    rng = np.random.default_rng(n)
    img = rng.random((n, n)).astype(np.float32)
    size = np.array([n * 1.0, n * 1.0])
    beta = np.arange(nviews) * (2 * np.pi / nviews) + 0.2
    P = np.linspace(-0.8 * n, 0.8 * n, nbins)
    D = 5.0 * n
    ref = oracle.fan_fp(img, beta, P, size, D)
    out = ops.ProjectionFan_2D(img.ravel(), n, n, size, beta, P, D)
    assert rel_l2(out, ref.ravel()) <= TOL or np.abs(ref).max() == 0
    R = rng.random(ref.shape).astype(np.float32)
    bref = oracle.fan_bp(R, beta.astype(np.float32), P.astype(np.float32), size, (n, n), D)
    bout = ops.BackprojectionFan2D(R.ravel(), beta, P, size, n, n, D)
    assert rel_l2(bout, bref.ravel()) <= TOL or np.abs(bref).max() == 0


def test_rejected_arguments_fail_cleanly():
    import ctypes as C
    from ctgb import _lib
    lib = _lib.load()
    plan = C.c_void_p()
    size = (C.c_double * 3)(10.0, 10.0, 10.0)
    beta = (C.c_float * 2)(0.0, 1.0)
    P = (C.c_float * 3)(-1.0, 0.0, 1.0)
    # no views
    assert lib.ct_cone_plan_create(C.byref(plan), 8, 8, 8, size, beta, 0, P, 3, P, 3, 50.0) == 1
    # 2^31 voxels or more
    assert lib.ct_cone_plan_create(C.byref(plan), 2048, 2048, 512, size, beta, 2, P, 3, P, 3, 50.0) == 1
    assert b"2^31" in lib.ct_last_error()
    # a source inside the volume
    assert lib.ct_cone_plan_create(C.byref(plan), 8, 8, 8, size, beta, 2, P, 3, P, 3, 5.0) == 1
    # non-finite domain values
    bad = (C.c_float * 3)(-1.0, float("nan"), 1.0)
    assert lib.ct_cone_plan_create(C.byref(plan), 8, 8, 8, size, beta, 2, bad, 3, P, 3, 50.0) == 1
    # a valid plan still works after the failures
    assert lib.ct_cone_plan_create(C.byref(plan), 8, 8, 8, size, beta, 2, P, 3, P, 3, 50.0) == 0
    assert lib.ct_cone_plan_destroy(plan) == 0
