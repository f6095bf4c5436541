"""Build recipe for the C restatement (oracle/sv_ref.c -> oracle/_build/liboracle_sv.so).

TEST INFRASTRUCTURE ONLY.  gcc with OpenMP, position-independent, no
architecture-specific flags (the same source builds on x86_64 and aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "sv_ref.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle_sv.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("gcc not found: needed for the C oracle")
    OUT_DIR.mkdir(exist_ok=True)
    tmp = OUT_DIR / (LIB.name + f".tmp{os.getpid()}")
    cmd = [cc, "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
