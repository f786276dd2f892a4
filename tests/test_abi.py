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
