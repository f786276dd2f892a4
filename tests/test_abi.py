"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/ctgb.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (REPO / "include" / "ctgb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ct_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_dropin_entry_points():
    names = declared_functions()
    for n in ["ct_ProjectionCone_3D", "ct_BackPro", "ct_FDKpro", "ct_ProjectionFan_2D",
              "ct_ProjectionParallel_2D", "ct_BackprojectionFan2D", "ct_FBPfan", "ct_FBPpara"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    from ctgb import _build, _lib
    path = _build.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_library_targets_sm_103a_only():
    from ctgb import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_version_and_error_strings_without_gpu():
    from ctgb import _lib
    lib = _lib.load()
    assert lib.ct_version().decode().startswith("ctgb")
    assert isinstance(lib.ct_last_error(), bytes)


def test_argument_validation_needs_no_gpu():
    """Host-side checks reject bad geometry before any CUDA call."""
    import ctypes as C
    import numpy as np
    from ctgb import _lib
    lib = _lib.load()
    h = C.c_void_p()
    size = np.array([10.0, 10.0, 10.0])
    beta = np.zeros(4, np.float32)
    P = np.linspace(-5, 5, 8).astype(np.float32)
    st = lib.ct_cone_plan_create(C.byref(h), 8, 8, 8, size.ctypes.data_as(C.c_void_p),
                                 beta.ctypes.data_as(C.c_void_p), 4, P.ctypes.data_as(C.c_void_p), 8,
                                 P.ctypes.data_as(C.c_void_p), 8, 1.0)   # source inside the volume
    assert st == 1
    assert b"Distance" in lib.ct_last_error()
    st = lib.ct_cone_plan_create(C.byref(h), 0, 8, 8, size.ctypes.data_as(C.c_void_p),
                                 beta.ctypes.data_as(C.c_void_p), 4, P.ctypes.data_as(C.c_void_p), 8,
                                 P.ctypes.data_as(C.c_void_p), 8, 100.0)
    assert st == 1


def test_unet_and_asd_argument_validation_needs_no_gpu():
    """The warm-start kernels' entry points reject bad shapes, channel counts
    and pointers before any CUDA call (the pointers here are never dereferenced)."""
    import ctypes as C
    from ctgb import _lib
    lib = _lib.load()
    p, q = C.c_void_p(0x10000), C.c_void_p(0x20000)        # 16-byte aligned, never used
    odd = C.c_void_p(0x10004)

    def conv(c1=32, c2=0, nz=4, ny=16, nx=16, taps=27, co1=32, co2=0, x1=p, out1=q):
        return lib.ct_unet_conv3d(x1, c1, p if c2 else None, c2, 1, nz, ny, nx, p, taps, None, 1, out1, co1,
                                  q if co2 else None, co2, None, None, None)

    assert conv(c1=16) == 1 and b"multiples of 32" in lib.ct_last_error()
    assert conv(co1=32, co2=16) == 1 and b"256" in lib.ct_last_error()
    assert conv(taps=9) == 1
    assert conv(nx=12) == 1 and b"128" in lib.ct_last_error()
    assert conv(x1=odd) == 1 and b"aligned" in lib.ct_last_error()
    assert conv(out1=None) == 1

    def wgrad(cin=32, cout=32, nx=16, ny=16, kper=4, taps=27):
        return lib.ct_unet_conv3d_wgrad(p, p, p, cin, q, cout, 1, 4, ny, nx, taps, kper, q, None)

    assert wgrad(cin=48) == 1
    assert wgrad(cout=96) == 1
    assert wgrad(nx=12) == 1 and b"multiple of 8" in lib.ct_last_error()
    assert wgrad(kper=0) == 1
    assert lib.ct_unet_pool2(p, q, 12, 1, 2, 2, 2, None) == 1
    assert lib.ct_unet_up2(p, None, 32, 1, 2, 2, 2, None) == 1
    assert lib.ct_unet_shift_t(p, 32, 1, 2, 2, 8, None, q, None, 48, 32, None) == 1
    assert lib.ct_unet_colsum(p, 48, 100, q, None) == 1
    assert lib.ct_unet_head(p, None, p, None, q, 100, None) == 1
    assert lib.ct_unet_im2col27(p, 1, 0, 4, 4, q, None) == 1
    assert lib.ct_tv_flow_asd(p, None, p, p, p, 4, 4, 4, 2, 1e-8, 0.0, 0.95, 0.95, None) == 1
    assert lib.ct_tv_flow_asd(p, p, p, p, p, 4, 4, 4, -1, 1e-8, 0.0, 0.95, 0.95, None) == 1
