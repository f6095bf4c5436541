"""Build recipe for libtyxonq_gb300.so (sm_103a only).

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc and the
objects are linked into one shared library that exports the C ABI declared in
``include/tq_sv.h``.  The library is built in-tree (``tyxonq_gb300/_lib``) and
rebuilt only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_DIR = PKG_DIR / "_lib"
LIB_NAME = "libtyxonq_gb300.so"
LIB_PATH = LIB_DIR / LIB_NAME
# the checked variant: -DTQ_CHECKED (device-side index checks, tq_check_status)
CHECKED_LIB_NAME = "libtyxonq_gb300_checked.so"
CHECKED_LIB_PATH = LIB_DIR / CHECKED_LIB_NAME

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtyxonq_gb300.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def needs_build(checked: bool = False) -> bool:
    lib = CHECKED_LIB_PATH if checked else LIB_PATH
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile and link the library (checked: the -DTQ_CHECKED variant, objects
    in their own folder); returns its path."""
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    if not force and not needs_build(checked):
        return lib_path
    nvcc = nvcc_path()
    build_dir = BUILD_DIR / "checked" if checked else BUILD_DIR
    build_dir.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    procs = []
    objs = []
    for src in sources():
        obj = build_dir / (src.stem + ".o")
        objs.append(obj)
        cmd = [nvcc, *NVCC_FLAGS, *(["-DTQ_CHECKED"] if checked else []), "-I", str(INCLUDE), "-c", str(src),
               "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src.name}\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB_DIR / (lib_path.name + ".tmp")
    cuda_lib = Path(nvcc).resolve().parent.parent / "lib64"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-L", str(cuda_lib), "-lnvrtc",
           "-Xlinker", f"-rpath={cuda_lib}"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
