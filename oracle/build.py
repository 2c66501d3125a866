"""Build recipe of the CPU oracle (TEST INFRASTRUCTURE ONLY).

* ``liboracle.so`` -- the C restatement in ``kdoracle.c``.
* ``_ref/libkdref.so`` -- the reference's own C port of the path
  (MarkCLewis/MultiLanguageKDTree Parallel/CVersion/src/kdtree.c and particle.c), compiled
  straight from the reference checkout when it is present (its root is taken from the
  ``KD_REFERENCE_DIR`` environment variable).  It is used only to pin the
  restatement (tests/test_oracle.py, tests/golden/make_golden.py) and as an optional CPU
  baseline.  Nothing is copied from the reference; gcc reads the sources where they lie.

Both are compiled with -ffp-contract=off so no multiply-add is fused: the reference's
arithmetic (Rust, and C without -ffast-math) rounds every operation.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
# the reference checkout: KD_REFERENCE_DIR, else where this build's sources mount it
REF_ROOT = Path(os.environ.get("KD_REFERENCE_DIR", "/root/reference"))
REF_DIR = REF_ROOT / "Parallel" / "CVersion" / "src"
REF_LIB = HERE / "_ref" / "libkdref.so"
CFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def _cc() -> str:
    exe = shutil.which("gcc") or shutil.which("cc")
    if not exe:
        raise RuntimeError("no C compiler found")
    return exe


def _newer(out: Path, srcs) -> bool:
    return not out.exists() or any(Path(s).stat().st_mtime > out.stat().st_mtime for s in srcs)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "kdoracle.c"
    if force or _newer(ORACLE_LIB, [src]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        subprocess.run([_cc(), "-std=gnu11", *CFLAGS, str(src), "-o", str(tmp), "-lm"],
                       check=True)
        tmp.replace(ORACLE_LIB)
    return ORACLE_LIB


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference C port if the reference checkout is mounted; else None."""
    srcs = [REF_DIR / "kdtree.c", REF_DIR / "particle.c"]
    if not all(s.exists() for s in srcs):
        return REF_LIB if REF_LIB.exists() else None
    if force or _newer(REF_LIB, srcs):
        REF_LIB.parent.mkdir(parents=True, exist_ok=True)
        tmp = REF_LIB.with_suffix(".so.tmp")
        subprocess.run([_cc(), "-std=gnu17", *CFLAGS, f"-I{REF_DIR}", *map(str, srcs),
                        "-o", str(tmp), "-lm"], check=True)
        tmp.replace(REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
