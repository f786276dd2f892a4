"""Build recipes for the checker (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles oracle/ct_oracle.c (the FP64 CPU restatement)
  into oracle/_build/libct_oracle.so with gcc + OpenMP.  It runs on any host
  (x86 container, Arm GPU machine).
* ``build_ref()`` compiles the reference's own kernel functions as host C++
  into oracle/_ref/libref_<name>.so, so that the oracle can be checked against
  the reference's arithmetic on the CPU.  It needs the reference source tree
  (``CT_REFERENCE_ROOT``, default /root/reference) and is skipped when that
  tree is absent.  The kernel text is extracted by brace matching from the
  reference files where they lie and piped into g++ on stdin together with
  the header macros, the shim (oracle/shim/cuda_host_shim.h) and this repo's
  launch-loop harness; no reference source is written to disk.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_LIB = BUILD / "libct_oracle.so"

# (name, reference .cu, reference .h, kernels, harness file)
REF_UNITS = [
    ("cone", "GPU_accelerated_Operator/ProjectionCone_3D/ProjectionCone_3D.cu",
     "GPU_accelerated_Operator/ProjectionCone_3D/ProjectionCone_3D.h", ["ProjectionCone"], "harness_cone.cpp"),
    ("bp3d", "GPU_accelerated_Operator/BackprojectionCone_3D/Backprojection3D.cu",
     "GPU_accelerated_Operator/BackprojectionCone_3D/Backprojection3D.h", ["BackProjection3D"], "harness_bp3d.cpp"),
    ("fdk", "Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FDK_GPU/FDK.cu",
     "Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FDK_GPU/FDK.h",
     ["GFunction", "PreWeightFilter", "BackProjection"], "harness_fdk.cpp"),
    ("fan", "GPU_accelerated_Operator/ProjectionFan_2D/ProjectionFan_2D.cu",
     "GPU_accelerated_Operator/ProjectionFan_2D/ProjectionFan_2D.h", ["ProjectionFan"], "harness_fan.cpp"),
    ("par", "GPU_accelerated_Operator/ProjectionParallel_2D/ProjectionParallel_2D.cu",
     "GPU_accelerated_Operator/ProjectionParallel_2D/ProjectionParallel_2D.h", ["ProjectionParallel"],
     "harness_par.cpp"),
    ("fanbp", "GPU_accelerated_Operator/BackprojectionFan_2D/BackprojectionFan2D.cu",
     "GPU_accelerated_Operator/BackprojectionFan_2D/BackprojectionFan2D.h", ["BackProjection"],
     "harness_fanbp.cpp"),
    ("fbpfan", "Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FBP_fan_GPU/FBPfan.cu",
     "Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FBP_fan_GPU/FBPfan.h",
     ["GFunction", "PreWeightFilter", "BackProjection"], "harness_fbpfan.cpp"),
    ("fbppar", "Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FBP_parallel_GPU/FBPparallel.cu",
     "Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/FBP_parallel_GPU/FBPparallel.h",
     ["GFunction", "Filter", "BackProjection"], "harness_fbppar.cpp"),
    ("iterfdk", "My_novel_algorithm/IterativeFDK/IterativeFDKerrCompute.cu",
     "My_novel_algorithm/IterativeFDK/IterativeFDKerrCompute.h", ["IterativeFDKerr"], "harness_iterfdk.cpp"),
    ("fdkui", "My_toolbox/Implement_UnitedImaging_Data/ImplementUI.cu",
     "My_toolbox/Implement_UnitedImaging_Data/ImplementUI.h", ["GFunction", "PreWeightFiltration", "BackProjection"],
     "harness_fdkui.cpp"),
]
# units whose kernels synchronise a block between dependent phases: compiled
# with the shim's threaded mode (one OS thread per simulated thread, real barrier)
THREADED_UNITS = {"fdkui"}


def reference_root() -> Path:
    return Path(os.environ.get("CT_REFERENCE_ROOT", "/root/reference"))


def build_oracle(force: bool = False) -> Path:
    """Compile the FP64 oracle into a shared library (gcc, OpenMP)."""
    src = HERE / "ct_oracle.c"
    BUILD.mkdir(exist_ok=True)
    if not force and ORACLE_LIB.exists() and ORACLE_LIB.stat().st_mtime > src.stat().st_mtime:
        return ORACLE_LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
           "-o", str(ORACLE_LIB), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    return ORACLE_LIB


def _strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def _extract_function(text: str, name: str) -> str:
    m = re.search(r"__global__\s+void\s+" + re.escape(name) + r"\s*\(", text)
    if not m:
        raise RuntimeError(f"kernel {name} not found")
    i = text.index("{", m.end())
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[m.start(): j + 1]
    raise RuntimeError(f"unbalanced braces in {name}")


def _extract_macros(text: str) -> list[str]:
    out = []
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("#define") and not re.match(r"#define\s+__\w+_H__\s*$", s):
            out.append(s)
    return out


def _extract_device_consts(text: str) -> list[str]:
    return [m.group(0) for m in re.finditer(r"^__device__\s+const\s+double\s+\w+\s*=\s*[^;]+;", text, flags=re.M)]


def build_ref(force: bool = False) -> list[Path]:
    """Compile the reference kernels as host code into oracle/_ref/ (checker only)."""
    root = reference_root()
    if not root.is_dir():
        return []
    REF_OUT.mkdir(exist_ok=True)
    shim = (HERE / "shim" / "cuda_host_shim.h").read_text()
    outs = []
    for name, cu, h, kernels, harness in REF_UNITS:
        out = REF_OUT / f"libref_{name}.so"
        outs.append(out)
        if out.exists() and not force:
            continue
        cu_text = _strip_comments((root / cu).read_text(errors="replace"))
        h_text = _strip_comments((root / h).read_text(errors="replace"))
        parts = ["#define SHIM_THREADED 1\n"] if name in THREADED_UNITS else []
        parts += [shim, "\n"]
        parts += [m + "\n" for m in _extract_macros(h_text)]
        parts += [m + "\n" for m in _extract_macros(cu_text)]
        parts += [c + "\n" for c in _extract_device_consts(cu_text)]
        parts += [_extract_function(cu_text, k) + "\n" for k in kernels]
        parts.append((HERE / "shim" / harness).read_text())
        cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-pthread", "-x", "c++", "-",
               "-o", str(out)]
        subprocess.run(cmd, input="".join(parts).encode(), check=True)
    return outs


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    for p in build_ref(force="--force" in sys.argv):
        print(p)
