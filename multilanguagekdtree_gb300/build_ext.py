"""Build recipe of libkdnbody.so: nvcc, sm_103a only, in-tree.

The CUDA translation units are compiled in parallel and linked into
``multilanguagekdtree_gb300/libkdnbody.so`` next to this file.  A rebuild happens only when
a source or header is newer than the library.
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
OBJDIR = PKG.parent / "_build" / "kdnbody"
LIB = PKG / "libkdnbody.so"
SOURCES = ["kd_build.cu", "kd_walk.cu", "kd_group.cu", "kd_adjoint.cu", "kd_generate.cu",
           "kd_api.cu", "kd_noalloc.cu", "kd_probe.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"] + ARCH


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libkdnbody.so")
    return exe


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libkdnbody.so if needed; return its path."""
    if not force and not _stale():
        return LIB
    OBJDIR.mkdir(parents=True, exist_ok=True)
    exe = nvcc()
    procs = []
    for src in SOURCES:
        obj = OBJDIR / (Path(src).stem + ".o")
        cmd = [exe, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT, text=True)))
    errors = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"$ {' '.join(cmd)}\n{out}")
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB.with_suffix(".so.tmp")
    objs = [str(OBJDIR / (Path(s).stem + ".o")) for s in SOURCES]
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n$ {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
