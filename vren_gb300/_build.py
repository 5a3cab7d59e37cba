"""Builds the native libraries of vren_gb300 in-tree.

- ``libvren_gb300.so``: the CUDA kernels and the C ABI declared in ``include/vren_gb300.h``,
  compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), one nvcc process per
  translation unit, in parallel, then linked with ``nvcc -shared``.
- ``libvren_scene.so``: the seeded synthetic-scene generators (plain C, host only).

Objects go to ``vren_gb300/_build/``; libraries sit next to this file.  A library is rebuilt
when any of its sources or headers is newer than it.
"""
from __future__ import annotations

import concurrent.futures as _cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
INCLUDE_DIR = REPO_DIR / "include"

CUDA_LIB = PKG_DIR / "libvren_gb300.so"
SCENE_LIB = PKG_DIR / "libvren_scene.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-ffp-contract=off",
    "--expt-relaxed-constexpr",
    "-I" + str(INCLUDE_DIR),
]
# Translation units whose float arithmetic must match the CPU oracle bit for bit are also
# compiled without FMA contraction (the kernels use __f*_rn intrinsics on those paths too).
NO_FMAD_UNITS = {"clustered.cu", "batch.cu", "lbvh.cu", "lights.cu", "cluster_debug.cu", "kd_tree.cu"}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build vren_gb300")
    return cand


def _cuda_sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE_DIR.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    if verbose and proc.stderr:
        print(proc.stderr, file=sys.stderr)


def build_cuda(verbose: bool = False, jobs: int | None = None, extra_flags: list[str] | None = None) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    srcs = _cuda_sources()
    objs = []
    cmds = []
    for src in srcs:
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            flags = list(NVCC_FLAGS) + list(extra_flags or [])
            if src.name in NO_FMAD_UNITS:
                flags += ["--fmad=false"]
            cmds.append([nvcc, *ARCH_FLAGS, *flags, "-c", str(src), "-o", str(obj)])
    if cmds:
        n = jobs or min(len(cmds), os.cpu_count() or 4)
        with _cf.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(lambda c: _run(c, verbose), cmds))
    if cmds or _stale(CUDA_LIB, objs):
        tmp = CUDA_LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs)], verbose)
        os.replace(tmp, CUDA_LIB)
    return CUDA_LIB


def build_scene(verbose: bool = False) -> Path:
    src = CSRC / "scene_gen.c"
    deps = [src, INCLUDE_DIR / "vren_scene.h"]
    if _stale(SCENE_LIB, deps):
        cc = shutil.which("gcc") or shutil.which("cc")
        if cc is None:
            raise RuntimeError("a C compiler (gcc) is required to build the scene generator")
        tmp = SCENE_LIB.with_suffix(".so.tmp")
        _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
              "-I" + str(INCLUDE_DIR), str(src), "-o", str(tmp), "-lm"], verbose)
        os.replace(tmp, SCENE_LIB)
    return SCENE_LIB


def build(verbose: bool = False) -> None:
    build_scene(verbose)
    build_cuda(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
