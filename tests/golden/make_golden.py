"""Generate tests/golden/reference_kernels.npz from the reference's own kernels.

Run where the CT-Research source tree is available (CT_REFERENCE_ROOT,
default /root/reference):  python tests/golden/make_golden.py
It compiles the reference kernel functions as host code (oracle/build.py,
build_ref) and records inputs and outputs of small cases of every operator on
the projector / backprojector path.  The fixtures pin the FP64 oracle
(oracle/ct_oracle.c) in tests/test_oracle_golden.py; the GPU tests then check
the CUDA kernels against the oracle and against these fixtures.

Cases cover odd and non-cubic sizes, views at multiples of pi/2, rays that
miss the volume, detector domains wider and narrower than the object,
residual launch tiles (LP not a multiple of the tile) and a descending domain.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "ct-research_gb300"))

from oracle import build as obuild  # noqa: E402
from oracle.oracle import RefCPU  # noqa: E402
from ctgb import phantom  # noqa: E402


def f32(a):
    return np.asarray(a, np.float32)


def main():
    obuild.build_ref()
    ref = RefCPU()
    rng = np.random.default_rng(12345)
    out = {}

    # --- cone geometries --------------------------------------------------
    cones = {
        "a": dict(shape=(12, 14, 16), size=[20.0, 18.0, 15.0], D=60.0,
                  P=f32((np.arange(24) - 11.5) * 1.1), xi=f32((np.arange(20) - 9.5) * 1.0),
                  beta=f32(np.arange(1, 13) * 2 * np.pi / 12)),
        "b": dict(shape=(20, 24, 24), size=[24.0, 24.0, 20.0], D=50.0,
                  P=f32((np.arange(40) - 19.5) * 0.9), xi=f32((np.arange(30) - 14.5) * 0.8),
                  beta=f32(np.arange(1, 17) * 2 * np.pi / 16)),
        # descending xi domain, odd z
        "c": dict(shape=(9, 10, 11), size=[11.0, 10.0, 9.0], D=40.0,
                  P=f32((np.arange(18) - 8.5) * 0.9), xi=f32((14.5 - np.arange(16)) * 0.8),
                  beta=f32(np.arange(1, 8) * 2 * np.pi / 7 + 0.1)),
    }
    for k, c in cones.items():
        nz, ns, nt = c["shape"]
        if k == "b":
            vol = phantom.ellipsoids_3d(nt, ns, nz, phantom.ellipsoid_params(12, seed=7)).numpy()
        else:
            vol = f32(rng.random(c["shape"]))
        proj = ref.cone_fp(vol, c["beta"], c["P"], c["xi"], c["size"], c["D"])
        R = f32(rng.random(proj.shape))
        bp = ref.cone_bp(R, c["beta"], c["P"], c["xi"], c["size"], c["D"], c["shape"])
        for name, v in dict(vol=vol, proj=proj, R=R, bp=bp, P=c["P"], xi=c["xi"], beta=c["beta"],
                            size=np.asarray(c["size"]), D=np.asarray(c["D"])).items():
            out[f"cone_{k}_{name}"] = v

    # --- FDK stages ---------------------------------------------------------
    c = dict(shape=(14, 16, 16), size=[16.0, 16.0, 14.0], D=45.0,
             P=f32((np.arange(300) - 149.5) * 0.08), xi=f32((np.arange(12) - 5.5) * 0.9),
             beta=f32(np.arange(1, 9) * 2 * np.pi / 8))
    vol = phantom.ellipsoids_3d(16, 16, 14, phantom.ellipsoid_params(6, seed=3)).numpy()
    proj = ref.cone_fp(vol, c["beta"], c["P"], c["xi"], c["size"], c["D"])
    w = ref.fdk_weight(proj, c["P"], c["xi"], c["D"])
    conv = ref.fdk_conv(w, c["P"], c["xi"])
    bp = ref.fdk_bp(conv, c["beta"], c["P"], c["xi"], c["size"], c["D"], c["shape"])
    G = ref.sl_filter(np.float32(abs(c["P"][1] - c["P"][0])), len(c["P"]))
    for name, v in dict(proj=proj, weighted=w, conv=conv, bp=bp, G=G, P=c["P"], xi=c["xi"], beta=c["beta"],
                        size=np.asarray(c["size"]), D=np.asarray(c["D"])).items():
        out[f"fdk_{name}"] = v

    # --- 2D ----------------------------------------------------------------
    img = phantom.ellipses_2d(32, 30, phantom.ellipse_params(10, seed=5)).numpy()
    size2 = [32.0, 30.0]
    beta_d = np.arange(1, 19) * 2 * np.pi / 18
    P_d = np.linspace(-25.0, 25.0, 40)
    P_wide = np.linspace(-40.0, 40.0, 33)
    fan = ref.fan_fp(img, beta_d, P_d, size2, 80.0)
    fan_wide = ref.fan_fp(img, beta_d, P_wide, size2, 80.0)
    par = ref.par_fp(img, beta_d, P_d, size2)
    Rf = f32(fan)
    fanbp = ref.fan_bp(Rf, f32(beta_d), f32(P_d), size2, (30, 32), 80.0)
    P150 = f32(np.linspace(-24.0, 24.0, 150))
    beta20 = f32(np.arange(1, 21) * 2 * np.pi / 20)
    fan150 = f32(ref.fan_fp(img, beta20.astype(np.float64), P150.astype(np.float64), size2, 80.0))
    fw = ref.fbpfan_weight(fan150, P150, 80.0)
    fconv = ref.fbpfan_conv(fw, P150)
    fbp = ref.fbpfan_bp(fconv, beta20, P150, size2, (30, 32), 80.0)
    fbppar = ref.fbppar(f32(par), f32(beta_d), f32(P_d), size2, (30, 32))
    for name, v in dict(img=img, size=np.asarray(size2), beta=beta_d, P=P_d, P_wide=P_wide, fp=fan,
                        fp_wide=fan_wide, par=par, bp=fanbp, P150=P150, beta20=beta20, sino150=fan150,
                        fbp_weighted=fw, fbp_conv=fconv, fbp_bp=fbp, fbppar=fbppar).items():
        out[f"f2_{name}"] = v

    # --- IterativeFDK error slice (IterativeFDKerrCompute.cu) -----------------
    from scipy.ndimage import gaussian_filter
    from ctgb.geometry import iterative_fdk_setup
    ishape, isize = (16, 18, 20), [20.0, 18.0, 16.0]
    ibeta, iU, iP, iG = iterative_fdk_setup(isize, ishape, pint=0.8, D=70.0, n_views=10)
    ipic = phantom.ellipsoids_3d(20, 18, 16, phantom.ellipsoid_params(8, seed=11)).numpy()
    ipic = f32(gaussian_filter(ipic, 0.7))
    for name, v in dict(pic=ipic, beta=ibeta, U=iU, P=iP, G=iG, size=np.asarray(isize), D=np.asarray(70.0)).items():
        out[f"ifdk_{name}"] = v
    for t in (1, 10):
        out[f"ifdk_err_t{t}"] = ref.iterfdk_err(ipic, ibeta, iU, iP, iG, isize, 70.0, t)

    # --- curved-detector FDK (ImplementUI.cu) ---------------------------------
    from ctgb.geometry import curved_fdk_case
    c = curved_fdk_case("filter")
    Rui = np.random.default_rng(77).random((len(c["beta"]), 80, 936))
    xs = np.array([0, 11, 39, 40, 79] * 5, np.int32)
    bs = np.repeat(np.arange(5, dtype=np.int32), 5)
    out["ui_filter_rows"] = ref.fdkui_filter_rows(Rui, c["xi"], c["gama"], c["beta"], c["b0"], c["maxg"], c["D"],
                                                  c["ds2d"], xs, bs)
    out["ui_filter_xs"], out["ui_filter_bs"] = xs, bs
    c = curved_fdk_case("bp")
    rc = np.random.default_rng(78).random((len(c["beta"]), len(c["xi"]), len(c["gama"]))) - 0.5
    out["ui_bp"] = ref.fdkui_bp(rc, c["size"], c["z_length"], c["beta"], c["D"], c["ds2d"], c["gama"], c["xi"])

    dst = Path(__file__).resolve().parent / "reference_kernels.npz"
    if dst.exists():
        old = np.load(dst)
        changed = [k for k in old.files if k in out and not np.array_equal(old[k], out[k])]
        if changed:
            print("warning: fixtures changed:", changed)
    np.savez_compressed(dst, **out)
    print(dst, sum(v.nbytes for v in out.values()), "bytes raw,", dst.stat().st_size, "on disk")


if __name__ == "__main__":
    main()
