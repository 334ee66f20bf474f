"""Build recipe for libfts.so (CUDA sm_103a kernels + C-ABI + host helpers).

Every translation unit under ``csrc/`` is compiled in parallel: ``.cu`` with
nvcc for sm_103a only, ``.cpp`` with the host C++ compiler and OpenMP.  The
objects are linked with nvcc into ``_build/libfts.so`` (CUDA runtime linked
statically, so the library needs nothing from CUDA at load time beyond the
driver).  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libfts.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfts.so")
    return cand


def _cxx() -> str:
    return os.environ.get("CXX", "g++")


def _headers() -> list[Path]:
    return sorted(INCLUDE.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, deps: list[Path], verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    if not _stale(obj, src, deps):
        return obj
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp", "-Xptxas", "-warn-spills", *inc,
               "-c", str(src), "-o", str(obj)]
    else:
        cmd = [_cxx(), "-O3", "-fPIC", "-fopenmp", "-std=c++17", "-Wall",
               "-I/usr/local/cuda/include", *inc, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and verbose:
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = _headers()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, deps, verbose), srcs))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    tmp = BUILD / "libfts.so.tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp),
           *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
