"""The reference-named C++ helpers (libctgb_compat*.so) on the GPU, called the
way the reference's gateways call them: host pointers, then cudaDeviceReset
after every call (ProjectionCone_3D.cpp:53).  The calls run in a child process
(the device resets would tear down this process's torch context), through
ctypes on the helpers' mangled C++ names, and are checked against the oracle
(rel-L2 <= 1e-5, FP32 against the reference's FP64 arithmetic)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
REPO = Path(__file__).resolve().parents[1]

CHILD = r'''
import ctypes as C, json, sys
import numpy as np
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/ct-research_gb300"]
from oracle.oracle import Oracle
from ctgb import phantom
from ctgb.geometry import view_angles, centred_domain, fan_config
lib = C.CDLL(sys.argv[2])
bp_lib = C.CDLL(sys.argv[3])
cudart = C.CDLL("libcudart.so.13")
o = Oracle()
vp = lambda a: a.ctypes.data_as(C.c_void_p)
out = {}

def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))

def call(lib_, name, *args):
    f = getattr(lib_, name)
    f.restype = C.c_int
    st = f(*args)
    assert st == 0, (name, st)
    assert cudart.cudaDeviceReset() == 0          # what every reference gateway does next

nt, ns, nz = 24, 22, 20
size = np.array([24.0, 22.0, 20.0])
beta = view_angles(12).astype(np.float32)
P = centred_domain(40, 0.9).astype(np.float32)
xi = centred_domain(32, 0.8).astype(np.float32)
D = 60.0
vol = phantom.ellipsoids_3d(nt, ns, nz, phantom.ellipsoid_params(12, seed=4)).numpy().astype(np.float32)
res = size / np.array([nt, ns, nz])
proj = np.zeros(len(beta) * len(xi) * len(P), np.float32)
for rep in range(2):                               # a second call after the reset gives the same values
    call(lib, "_Z17ProjectionCone_3DPKfPfS0_S0_S0_iiidddiiidPKd", vp(vol), vp(proj), vp(beta), vp(P), vp(xi),
         nt, ns, nz, C.c_double(size[0] / 2), C.c_double(size[1] / 2), C.c_double(size[2] / 2), len(beta), len(P),
         len(xi), C.c_double(D), vp(res))
    ref = o.cone_fp(vol, beta, P, xi, size, D)
    out[f"ProjectionCone_3D#{rep}"] = rel(proj, ref.ravel())
R = ref.astype(np.float32).ravel()
disp = np.zeros(nt * ns * nz, np.float32)
call(lib, "_Z7BackProPfPKfS1_S1_S1_diiiPKdiii", vp(disp), vp(R), vp(xi), vp(P), vp(beta), C.c_double(D),
     len(beta), len(P), len(xi), vp(size), nt, ns, nz)
out["BackPro"] = rel(disp, o.cone_bp(R.reshape(len(beta), len(xi), len(P)), beta, P, xi, size, D, (nz, ns, nt)).ravel())
call(lib, "_Z6FDKproPfPKfS1_S1_S1_diiiPKdiii", vp(disp), vp(R), vp(xi), vp(P), vp(beta), C.c_double(D),
     len(beta), len(P), len(xi), vp(size), nt, ns, nz)
out["FDKpro"] = rel(disp, o.fdk(R.reshape(len(beta), len(xi), len(P)), beta, P, xi, size, D, (nz, ns, nt),
                                 filter_mode=1, sticky=1).ravel())
g = fan_config(40, 36, 64, 120.0, 40.0)
img = phantom.ellipses_2d(40, 40, phantom.ellipse_params(10, seed=8)).numpy().astype(np.float32)
sino = np.zeros(len(g.beta) * len(g.P), np.float64)
size2 = np.asarray(g.size, np.float64)
res2 = size2 / 40.0
call(lib, "_Z16ProjectionFan_2DPKfPdPKdS3_iiddiidS3_", vp(img), vp(sino), vp(g.beta), vp(g.P), 40, 40,
     C.c_double(20.0), C.c_double(20.0), len(g.beta), len(g.P), C.c_double(g.D), vp(res2))
fref = o.fan_fp(img, g.beta, g.P, g.size, g.D)
out["ProjectionFan_2D"] = rel(sino, fref.ravel())
s32 = fref.astype(np.float32).ravel()
b32, p32 = g.beta.astype(np.float32), g.P.astype(np.float32)
im = np.zeros(40 * 40, np.float32)
call(lib, "_Z6FBPfanPfPKfS1_S1_iiPKdiid", vp(im), vp(s32), vp(p32), vp(b32), len(b32), len(p32), vp(size2), 40, 40,
     C.c_double(g.D))
out["FBPfan"] = rel(im, o.fbpfan(s32.reshape(len(b32), len(p32)), b32, p32, size2, (40, 40), g.D, filter_mode=1).ravel())
call(bp_lib, "_Z6FBPfanPfPKfS1_S1_iiPKdiid", vp(im), vp(s32), vp(p32), vp(b32), len(b32), len(p32), vp(size2), 40,
     40, C.c_double(g.D))
out["FBPfan(BackprojectionFan_2D)"] = rel(im, o.fan_bp(s32.reshape(len(b32), len(p32)), b32, p32, size2, (40, 40), g.D).ravel())
print(json.dumps(out))
'''


def test_reference_named_helpers_survive_device_resets(tmp_path):
    from ctgb import _build
    _build.build()
    lib_dir = REPO / "ct-research_gb300" / "ctgb" / "_lib"
    script = tmp_path / "child.py"
    script.write_text(CHILD)
    r = subprocess.run([sys.executable, str(script), str(REPO), str(lib_dir / "libctgb_compat.so"),
                        str(lib_dir / "libctgb_compat_bpfan.so")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    errs = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(errs) == 7, errs
    for name, e in errs.items():
        assert e <= 1e-5, (name, e)
