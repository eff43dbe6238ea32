"""Compile the reference's own OpenCL C kernels as host C++ into oracle/_ref/libnfxref.so.

ORACLE / TEST INFRASTRUCTURE ONLY. This is the recipe that lets the CPU restatement
(oracle/nfx_oracle.c) be pinned against the reference itself: the OpenCL runtime the
reference needs (pyopencl + an ICD such as pocl) is not installed, so the kernel sources are
compiled for the host instead, exactly as KernelBuilder would concatenate them
(nofluidx3d/KernelBuilder.py:17-22, 54-62): typedefs.h, atomicAdd.cl, matrix.h, matrix.cl, then
the kernel files.

Mechanical source transforms applied on the fly (nothing is written into the repository but
the built library, which stays untracked in oracle/_ref/):
  * `(T3)(a, b, c)` OpenCL vector literals -> `mk3<T3>(a, b, c)`; C++ would otherwise read
    them as a cast of a comma expression;
  * VelocityVerlet.cl's hard-coded damping `const double xi = 0.005;` (:11) -> a run-time value;
  * `#ifdef FIXED_TOP_BOTTOM ... #endif` (:17-22) -> a run-time branch;
  * clang's `overloadable` attribute dropped and `always_inline` -> `inline`.

Usage: python oracle/build_ref.py [reference_root]
The reference root is the argument, else the environment variable NFX_REFERENCE_ROOT, else
/root/reference (where this recipe's build host keeps the reference tree). Exit status 0 and a
message when the reference tree is absent (nothing to build).
"""

from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_ref"
OUT_LIB = OUT_DIR / "libnfxref.so"

KERNEL_FILES = [
    "typedefs.h",
    "atomicAdd.cl",
    "matrix.h",
    "matrix.cl",
    "Interactions/tetra.cl",
    "Interactions/Substrate.cl",
    "Interactions/Plane.cl",
    "Interactions/Sphere.cl",
    "Interactions/VelocityVerlet.cl",
    "InteractionFiniteStrainViscoplastic.cl",
    "velocityVerlet2.cl",
    "InteractionSphereIntegral.cl",
]

DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root(arg: str | os.PathLike | None = None) -> Path:
    """The reference tree this recipe reads: `arg`, else $NFX_REFERENCE_ROOT, else the build
    host's checkout."""
    if arg:
        return Path(arg)
    return Path(os.environ.get("NFX_REFERENCE_ROOT") or DEFAULT_REFERENCE_ROOT)


def reference_present(arg: str | os.PathLike | None = None) -> bool:
    return (reference_root(arg) / "nofluidx3d" / "kernels").is_dir()


_VEC_LITERAL = re.compile(r"\((ibmPrecisionFloat3|tetraPrecisionFloat3|double3|float3)\)\s*\(")


def transform(name: str, text: str) -> str:
    text = _VEC_LITERAL.sub(lambda m: f"mk3<{m.group(1)}>(", text)
    # clang's overloadable/always_inline attributes: C++ overloads natively, and g++ refuses
    # always_inline on interposable functions in a shared object
    text = text.replace("__attribute__((always_inline))", "inline")
    text = text.replace("__attribute__((overloadable))", "")
    if name.endswith("VelocityVerlet.cl"):
        text, n = re.subn(r"const double xi = 0\.005;", "const double xi = g_vv_xi;", text)
        if n != 1:
            raise RuntimeError("VelocityVerlet.cl: damping literal not found")
        text = text.replace("#ifdef FIXED_TOP_BOTTOM", "if (g_fixed_top_bottom) {")
        text = text.replace("#endif // FIXED_TOP_BOTTOM", "}")
    return text


def build(root: str | os.PathLike | None = None, quiet: bool = False) -> Path | None:
    kdir = reference_root(root) / "nofluidx3d" / "kernels"
    if not kdir.is_dir():
        if not quiet:
            print(f"build_ref: no reference kernels at {kdir}; nothing to build")
        return None
    parts = ['#include "ref_shim.hpp"\n']
    for rel in KERNEL_FILES:
        src = (kdir / rel).read_text()
        parts.append(f"// ---- {rel}\n#line 1 \"{rel}\"\n")
        parts.append(transform(rel, src) + "\n")
    parts.append('#include "ref_driver.inc"\n')
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    with tempfile.TemporaryDirectory() as td:
        tu = Path(td) / "nfxref_tu.cpp"
        tu.write_text("".join(parts))
        cmd = [
            "g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-ffp-contract=off",
            f"-I{HERE}", str(tu), "-o", str(OUT_LIB),
        ]
        subprocess.run(cmd, check=True)
    if not quiet:
        print(f"build_ref: wrote {OUT_LIB}")
    return OUT_LIB


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else None)
