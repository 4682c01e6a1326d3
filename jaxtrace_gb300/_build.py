"""Build recipe of the native library ``libjaxtrace_gb300.so``.

Every CUDA translation unit under ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked into
one shared library next to this file.  No CMake, no torch extension
machinery: plain ``nvcc`` so the same recipe runs on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
LIB_NAME = "libjaxtrace_gb300.so"
LIB_PATH = PKG_DIR / LIB_NAME
OBJ_DIR = PKG_DIR / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply/add is ever contracted implicitly, so the exact
# (NumPy-compatible) arithmetic holds for scalar and packed float32x2 code;
# the fast paths ask for FMAs explicitly (fmaf, __ffma2_rn).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-fmad=false",
              "-Xptxas", "-warn-spills"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jaxtrace_gb300")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _compile(src: Path, verbose: bool, obj_dir: Path = OBJ_DIR, defines: tuple = ()) -> Path:
    obj = obj_dir / (src.stem + ".o")
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, *[f"-D{d}" for d in defines], "-I", str(INCLUDE), "-c", str(src),
           "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc_path(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(INCLUDE),
               "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout.strip() or res.stderr.strip()):
        print(res.stdout + res.stderr, flush=True)
    return obj


def build(verbose: bool = False, jobs: int | None = None, defines: tuple = (), out: Path | None = None) -> Path:
    """Compile every translation unit and link ``libjaxtrace_gb300.so``.

    ``defines`` (e.g. ``("JT_TRACK_MIN_BLOCKS=3",)``) and ``out`` build a
    tuning variant into another directory; the default build is in-tree."""
    lib_path = Path(out) if out is not None else LIB_PATH
    obj_dir = OBJ_DIR if out is None else lib_path.parent / "_build"
    obj_dir.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, obj_dir, tuple(defines)), srcs))
    if lib_path.exists() and lib_path.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return lib_path
    tmp = lib_path.with_suffix(".so.tmp")
    cmd = [nvcc_path(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
