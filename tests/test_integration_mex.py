"""The MEX gateway that INTEGRATION.md shows a maintainer compiles against
include/ctgb.h: extracted from the document and compiled with g++ and a stub
mex.h (MATLAB is not available here), so its calls match the C ABI."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]

STUB_MEX_H = """#pragma once
#include <stddef.h>
typedef struct mxArray_tag mxArray;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
void *mxGetData(const mxArray *a);
double *mxGetPr(const mxArray *a);
double mxGetScalar(const mxArray *a);
size_t mxGetM(const mxArray *a);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
"""


def test_documented_gateway_compiles_against_the_header(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    text = (REPO / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    gateways = [b for b in blocks if "mexFunction" in b]
    assert gateways, "INTEGRATION.md shows no MEX gateway"
    (tmp_path / "mex.h").write_text(STUB_MEX_H)
    src = tmp_path / "gateway.cpp"
    src.write_text(gateways[0])
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Werror", "-c", str(src), "-I", str(tmp_path), "-I",
                        str(REPO / "include"), "-o", str(tmp_path / "gateway.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
