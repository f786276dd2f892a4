"""The reference's own MEX gateways link against the compatibility libraries.

The gateways (X.cpp) call the reference's host helpers by name with C++
linkage (e.g. ProjectionCone_3D.h:32-35, Backprojection3D.h:31-33).  Where
the reference tree is present, this test compiles each gateway as it is, with
a stub mex.h (MATLAB is not available) and the headers' Windows include
paths of the CUDA runtime pointed at this toolkit, into a shared object
linked against libctgb_compat.so (libctgb_compat_bpfan.so for the
unfiltered BackprojectionFan_2D gateway) with --no-undefined: every helper a
gateway calls must resolve, by its mangled C++ signature, in that library.
One gateway needs one more change to compile with g++: ProjectionFan_2D.cpp:15
declares its element count `const double LMat` and allocates `new double[LMat]`,
which MSVC accepts and g++ rejects; the copy declares it `long`.  Nothing is
written to the reference tree; the patched copies live in the test's temporary
folder only.  The compatibility libraries' exports are
checked everywhere.
"""
import ctypes as C
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
REF = Path("/root/reference")
LIBDIR = REPO / "ct-research_gb300" / "ctgb" / "_lib"

GATEWAYS = [
    ("GPU_accelerated_Operator/ProjectionCone_3D", "ProjectionCone_3D.cpp", "ctgb_compat"),
    ("GPU_accelerated_Operator/BackprojectionCone_3D", "Backprojection3D.cpp", "ctgb_compat"),
    ("GPU_accelerated_Operator/ProjectionFan_2D", "ProjectionFan_2D.cpp", "ctgb_compat"),
    ("GPU_accelerated_Operator/ProjectionParallel_2D", "ProjectionParallel_2D.cpp", "ctgb_compat"),
    ("GPU_accelerated_Operator/BackprojectionFan_2D", "BackprojectionFan2D.cpp", "ctgb_compat_bpfan"),
    ("Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FDK_GPU", "FDK.cpp", "ctgb_compat"),
    ("Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FBP_fan_GPU", "FBPfan.cpp", "ctgb_compat"),
    ("Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FBP_parallel_GPU", "FBPparallel.cpp",
     "ctgb_compat"),
    ("My_novel_algorithm/IterativeFDK", "IterativeFDKerrCompute.cpp", "ctgb_compat"),
    ("My_toolbox/Implement_UnitedImaging_Data", "ImplementUI.cpp", "ctgb_compat"),
]

# non-standard C++ of a gateway that g++ rejects: (file, text, replacement)
GXX_FIXES = [("ProjectionFan_2D.cpp", "const double LMat = LBeta * LP;", "const long LMat = LBeta * LP;")]

# MATLAB's C API as the gateways use it, defined (not just declared) so that
# the gateway links with --no-undefined and only the helpers are left to resolve
STUB_MEX_H = """#pragma once
#include <stddef.h>
typedef struct mxArray_tag mxArray;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
static inline double *mxGetPr(const mxArray *) { return 0; }
static inline double mxGetScalar(const mxArray *) { return 0.0; }
static inline size_t mxGetM(const mxArray *) { return 0; }
static inline mxArray *mxCreateDoubleMatrix(size_t, size_t, mxComplexity) { return 0; }
static inline int mexPrintf(const char *, ...) { return 0; }
"""

# the helper each gateway calls, with the C++ signature of its reference header
MANGLED = {
    "ctgb_compat": ["_Z17ProjectionCone_3DPKfPfS0_S0_S0_iiidddiiidPKd",
                    "_Z7BackProPfPKfS1_S1_S1_diiiPKdiii",
                    "_Z6FDKproPfPKfS1_S1_S1_diiiPKdiii",
                    "_Z16ProjectionFan_2DPKfPdPKdS3_iiddiidS3_",
                    "_Z21ProjectionParallel_2DPKfPdPKdS3_iiddiiS3_",
                    "_Z6FBPfanPfPKfS1_S1_iiPKdiid",
                    "_Z7FBPparaPfPKfS1_S1_iiPKdii",
                    "_Z22IterativeFDKerrComputePKfPfS0_S0_PKdS3_S3_iiidddiiiidS3_iffd",
                    "_Z5FDKUIPdPKdS1_S1_S1_ddddiiiPKii"],
    "ctgb_compat_bpfan": ["_Z6FBPfanPfPKfS1_S1_iiPKdiid"],
}


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return Path(nvcc).resolve().parent.parent / "include"


@pytest.fixture(scope="module")
def compat_libs():
    from ctgb import _build
    _build.build()
    return {name: LIBDIR / f"lib{name}.so" for name in MANGLED}


def test_compat_libraries_export_the_reference_helpers(compat_libs):
    for name, symbols in MANGLED.items():
        lib = C.CDLL(str(compat_libs[name]))
        for sym in symbols:
            assert hasattr(lib, sym), (name, sym)


@pytest.mark.skipif(not REF.exists(), reason="reference tree not present on this host")
@pytest.mark.parametrize("folder,gateway,lib", GATEWAYS)
def test_reference_gateway_links_against_compat_library(compat_libs, tmp_path, folder, gateway, lib):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = REF / folder
    (tmp_path / "mex.h").write_text(STUB_MEX_H)
    for f in list(src.glob("*.h")) + [src / gateway]:
        text = f.read_text(errors="replace")
        # the Windows paths of the CUDA runtime headers -> this toolkit's
        text = re.sub(r'#include\s+"[^"]*\\(cuda_runtime\.h|device_launch_parameters\.h)"', r"#include <\1>", text)
        for name, old, new in GXX_FIXES:
            if f.name == name:
                assert old in text
                text = text.replace(old, new)
        (tmp_path / f.name).write_text(text)
    out = tmp_path / "gateway.so"
    cmd = [gxx, "-std=c++17", "-shared", "-fPIC", "-w", "-I", str(tmp_path), "-I", str(_cuda_include()),
           str(tmp_path / gateway), "-o", str(out), f"-L{LIBDIR}", f"-l{lib}", "-Wl,--no-undefined",
           f"-Wl,-rpath,{LIBDIR}", f"-L{_cuda_include().parent / 'lib64'}", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert out.exists() and os.path.getsize(out) > 0
