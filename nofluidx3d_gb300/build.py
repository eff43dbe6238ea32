"""Builds the native library libnfx.so in-tree (nofluidx3d_gb300/_build/).

The CUDA kernels are compiled for sm_103a only (GB300); host C++ compiles for whatever the
build machine is (x86-64 or aarch64). Translation units are compiled in parallel and linked
with the static CUDA runtime, so the library depends only on the driver's libcuda.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD_DIR = PKG / "_build"
LIB_NAME = "libnfx.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Device code generation: ptxas's least register-hungry allocation bias. At the 64-register cap
# of the element pass it leaves no spills and measured 0.6 % faster steps than the default level
# (level 8-10 1 % slower); it does not change the arithmetic.
DEVICE_FLAGS = ["-Xptxas=--register-usage-level=0"]

SOURCES = ["nfx_kernels.cu", "nfx_noalloc.cu", "nfx_mlp.cu", "nfx_api.cpp", "nfx_mesh.cpp", "nfx_batch.cpp"]
HEADERS = ["nfx_internal.h", "nfx_math.cuh"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put the CUDA toolkit on PATH)")


def lib_path() -> Path:
    return BUILD_DIR / LIB_NAME


def _inputs() -> list[Path]:
    return [CSRC / s for s in SOURCES + HEADERS] + [INCLUDE / "nfx.h", Path(__file__)]


def up_to_date() -> bool:
    lib = lib_path()
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _inputs())


def tuning_defines() -> list[str]:
    """Kernel tuning macros from NFX_NVCC_DEFINES (space-separated -DNAME=VALUE, e.g.
    -DNFX_NODE_MIN_BLOCKS=4); anything that is not a -D flag is rejected."""
    flags = os.environ.get("NFX_NVCC_DEFINES", "").split()
    for f in flags:
        if not f.startswith("-D") or len(f) < 3:
            raise ValueError(f"NFX_NVCC_DEFINES takes -DNAME[=VALUE] flags only, got {f!r}")
    return flags


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libnfx.so unless it is newer than every source. Returns its path."""
    if not force and up_to_date():
        return lib_path()
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}", *tuning_defines()]
    procs = []
    objs = []
    for src in SOURCES:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH_FLAGS, *DEVICE_FLAGS, "-lineinfo", *common, "-c", str(CSRC / src), "-o", str(obj)]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError(f"libnfx build failed:\n{msg}")
    tmp = BUILD_DIR / f"{LIB_NAME}.{os.getpid()}.tmp"
    link = [nvcc, *ARCH_FLAGS, "-shared", "-cudart", "static", *map(str, objs), "-o", str(tmp)]
    if verbose:
        print(" ".join(link), file=sys.stderr)
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"libnfx link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
