"""Build libctgb.so (the sm_103a kernels + C ABI) in-tree with nvcc.

Each .cu file compiles in parallel to an object, then one link step makes
``ctgb/_lib/libctgb.so``.  Only ``-gencode arch=compute_103a,code=sm_103a``
is generated: the library is for GB300 only.  Two small host-only libraries
carry the reference's own helper names with C++ linkage over it
(include/ctgb_compat.h): ``libctgb_compat.so`` and ``libctgb_compat_bpfan.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent                      # ct-research_gb300/
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libctgb.so"
OBJDIR = LIBDIR / "obj"
COMPAT = {"libctgb_compat.so": [], "libctgb_compat_bpfan.so": ["-DCTGB_COMPAT_BPFAN"]}

SOURCES = ["abi.cu", "cone_fp.cu", "cone_bp.cu", "filter.cu", "fan2d.cu", "sirt.cu", "ref_walk.cu", "fan_batch.cu",
           "noalloc.cu", "iterfdk.cu", "fdkui.cu", "sysmat.cu", "solvers.cu",
           "unet_conv.cu", "unet_ops.cu"]
# ref_walk.cu replays the reference's FP64 walk operation by operation: no FMA contraction
PER_FILE_FLAGS = {"ref_walk.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libctgb")
    return exe


def _env_flags() -> list[str]:
    """Extra nvcc flags from CTGB_NVCC_FLAGS (tuning builds, e.g. -DCT_FP_MINB=9)."""
    return os.environ.get("CTGB_NVCC_FLAGS", "").split()


def _flags(extra: list[str] | None = None) -> list[str]:
    # host code: no FMA contraction, so host-built tables round as the oracle's on every CPU
    return ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", f"-I{INCLUDE}",
            f"-I{CSRC}",
            "--expt-relaxed-constexpr", *_env_flags(), *(extra or [])]


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    if any(not (LIBDIR / n).exists() or (LIBDIR / n).stat().st_mtime < t for n in COMPAT):
        return True
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + [CSRC / "compat.cpp", INCLUDE / "ctgb.h",
                                                                       INCLUDE / "ctgb_compat.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def _build_compat(exe: str) -> None:
    """The reference-named C++ helpers, linked against libctgb.so (found next to them)."""
    for name, defs in COMPAT.items():
        out = LIBDIR / name
        tmp = out.with_suffix(".so.tmp")
        cmd = [exe, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", *defs,
               str(CSRC / "compat.cpp"), "-o", str(tmp), f"-L{LIBDIR}", "-lctgb", "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compat build failed ({name}):\n{r.stderr}")
        os.replace(tmp, out)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile the library if any source is newer than it; returns its path."""
    if not force and not ptxas_info and not _stale():
        return LIB
    OBJDIR.mkdir(parents=True, exist_ok=True)
    exe = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def one(src: str):
        obj = OBJDIR / (Path(src).stem + ".o")
        cmd = [exe, *_flags(extra + PER_FILE_FLAGS.get(src, [])), "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    jobs = min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(one, SOURCES))
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                print(err)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *[str(o) for o, _ in results], "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    _build_compat(exe)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
