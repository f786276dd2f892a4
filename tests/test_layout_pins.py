"""Pins of the reference's layout helpers and phantom rule, and an analytic
known-answer test of the forward projector.

* Img2vec_Mat2Cpp2D.m:2 (single(reshape(fliplr(Img'), numel(Img), 1))) and
  Vec2img_Cpp2Mat2D.m:2-3 (fliplr(reshape(v, height, width))'): a hand-worked
  MATLAB case and round trips.
* phantom3d.m:71-108: ctgb.phantom.phantom3d against a line-by-line numpy
  transliteration of the MATLAB loop (meshgrid, column-major flatten, Euler
  matrix, find), vectorised as SIRT3D.m:51-57 does (pic(t, s, z), t fastest).
* The analytic line integrals of constant ellipsoids (the 3-D form of
  AnalyticProjectionParal.m:51-63, oracle.ellipsoid_line_integral) against the
  oracle's cone projector of the same ellipsoids voxelised on a fine grid:
  the geometry conventions (source, virtual detector, axes) agree; the
  difference is the voxelisation, a few 1e-3.
"""
import numpy as np
import pytest

from conftest import rel_l2


def test_img2vec_matches_hand_worked_matlab_case():
    from ctgb.ops import Img2vec_Mat2Cpp2D, Vec2img_Cpp2Mat2D
    img = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])          # MATLAB [1 2 3; 4 5 6]
    # Img' = [1 4; 2 5; 3 6]; fliplr -> [4 1; 5 2; 6 3]; column-major -> 4 5 6 1 2 3
    v = Img2vec_Mat2Cpp2D(img)
    assert v.dtype == np.float32 and v.tolist() == [4, 5, 6, 1, 2, 3]
    # reshape(v, 3, 2) = [4 1; 5 2; 6 3]; fliplr -> [1 4; 2 5; 3 6]; ' -> [1 2 3; 4 5 6]
    np.testing.assert_array_equal(Vec2img_Cpp2Mat2D(v, 3, 2), img)


def test_img2vec_round_trips():
    from ctgb.ops import Img2vec_Mat2Cpp2D, Vec2img_Cpp2Mat2D
    rng = np.random.default_rng(0)
    for h, w in [(1, 1), (5, 7), (16, 9)]:
        img = rng.random((h, w)).astype(np.float32)
        np.testing.assert_array_equal(Vec2img_Cpp2Mat2D(Img2vec_Mat2Cpp2D(img), w, h), img)


def _phantom3d_matlab(n, e):
    """phantom3d.m:71-108 transliterated: MATLAB arrays as Fortran-ordered numpy."""
    rng = (np.arange(n) - (n - 1) / 2) / ((n - 1) / 2)
    x, y, z = np.meshgrid(rng, rng, rng)          # MATLAB meshgrid: x varies along the 2nd index
    coord = np.stack([x.ravel(order="F"), y.ravel(order="F"), z.ravel(order="F")])
    p = np.zeros(n ** 3)
    for A, a, b, c, x0, y0, z0, phi in e:
        ph = phi * np.pi / 180
        alpha = np.array([[np.cos(ph), np.sin(ph), 0], [-np.sin(ph), np.cos(ph), 0], [0, 0, 1]])
        cp = alpha @ coord
        shift = alpha @ np.array([x0, y0, z0])
        idx = np.nonzero((cp[0] - shift[0]) ** 2 / a ** 2 + (cp[1] - shift[1]) ** 2 / b ** 2
                         + (cp[2] - shift[2]) ** 2 / c ** 2 <= 1)
        p[idx] += A
    return p.reshape((n, n, n), order="F")          # pic(i, j, k)


def test_phantom3d_rule_and_layout():
    from ctgb.phantom import phantom3d
    rng = np.random.default_rng(4)
    e = np.column_stack([rng.uniform(-0.5, 1, 5), rng.uniform(0.2, 0.8, (5, 3)), rng.uniform(-0.3, 0.3, (5, 3)),
                         rng.uniform(0, 180, 5)])
    for n in (9, 16):
        pic = _phantom3d_matlab(n, e)
        # SIRT3D.m:51-57: picvector(num) = pic(t, s, z), num - 1 = (z * S + s) * T + t
        picvector = pic.ravel(order="F")
        ours = phantom3d(n, e).numpy()
        assert ours.shape == (n, n, n)
        np.testing.assert_allclose(ours.ravel(), picvector.astype(np.float32), rtol=0, atol=1e-6)


PARAMS = np.array([[0.6, 0.7, 0.5, 0.6, 0.05, -0.1, 0.0, 0.4],
                   [0.3, 0.25, 0.35, 0.3, -0.2, 0.25, 0.1, 1.1]])


def _analytic(geom, size):
    """Exact line integrals of PARAMS (world frame) along every ray of geom."""
    from ctgb.phantom import world_ellipsoids
    from oracle.oracle import ellipsoid_line_integral
    ells = world_ellipsoids(PARAMS, size)
    ref = np.zeros((len(geom.beta), len(geom.xi), len(geom.P)))
    for v, b in enumerate(geom.beta.astype(np.float32).astype(np.float64)):
        sb, cb = np.sin(b), np.cos(b)
        src = np.array([size[0] / 2 - geom.D * sb, size[1] / 2 + geom.D * cb, size[2] / 2])
        for x, xi in enumerate(geom.xi.astype(np.float64)):
            for p, P in enumerate(geom.P.astype(np.float64)):
                d = np.array([P * cb + geom.D * sb, P * sb - geom.D * cb, xi])
                ref[v, x, p] = ellipsoid_line_integral(src, src + 2.5 * d, ells)
    return ref


def _kat_errors(project, sizes, size, views, det):
    """rel-L2 of the projection of PARAMS voxelised at each grid size against
    the exact integrals: a wrong geometry convention leaves an O(1) error, the
    voxelisation an error that falls with the voxel size."""
    from ctgb.geometry import ConeGeometry, view_angles, centred_domain
    errs = []
    for n in sizes:
        geom = ConeGeometry(n, n, n, size, view_angles(views), centred_domain(det[0], det[2]),
                            centred_domain(det[1], det[2]), 120.0)
        errs.append(rel_l2(project(n, geom), _analytic(geom, size)))
    return errs


def test_analytic_line_integrals_match_the_oracle_projector(oracle):
    from ctgb.phantom import ellipsoids_3d

    def project(n, g):
        vol = ellipsoids_3d(n, n, n, PARAMS).numpy()
        return oracle.cone_fp(vol, g.beta, g.P, g.xi, g.size, g.D)

    e96, e192 = _kat_errors(project, (96, 192), (48.0, 48.0, 48.0), 4, (24, 16, 2.0))
    assert e96 < 0.03 and e192 < 0.6 * e96 and e192 < 0.015, (e96, e192)


@pytest.mark.gpu
def test_analytic_line_integrals_match_the_gpu_projector():
    from ctgb.device import ConePlan
    from ctgb.phantom import ellipsoids_3d

    def project(n, g):
        return ConePlan(g).fp(ellipsoids_3d(n, n, n, PARAMS, device="cuda")).cpu().numpy()

    e256, e512 = _kat_errors(project, (256, 512), (48.0, 48.0, 48.0), 6, (32, 24, 1.5))
    assert e256 < 0.012 and e512 < 0.6 * e256 and e512 < 0.006, (e256, e512)
