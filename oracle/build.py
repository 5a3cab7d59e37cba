"""Builds the CPU oracle (test infrastructure) into oracle/_build/libvren_oracle.so.

The reference (loryruta/vren) cannot be compiled here: it needs the Vulkan SDK, volk, VMA,
SPIRV-Cross, glm, gtest and Google Benchmark, none of which are installed.  The oracle is a
plain-C restatement instead; see vren_oracle.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB = BUILD_DIR / "libvren_oracle.so"
SOURCES = [ORACLE_DIR / "vren_oracle.c"]
CXX_SOURCES = [ORACLE_DIR / "vren_oracle_shade.cpp"]
HEADERS = [ORACLE_DIR / "vren_oracle.h"]


def build(verbose: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    deps = SOURCES + CXX_SOURCES + HEADERS
    if LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cc is None or cxx is None:
        raise RuntimeError("gcc and g++ are required to build the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    common = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", f"-I{ORACLE_DIR}"]
    objs = []
    for src in SOURCES:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [cc, "-std=gnu11", *common, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        objs.append(obj)
    for src in CXX_SOURCES:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [cxx, "-std=c++17", *common, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        objs.append(obj)
    cmd = [cxx, "-shared", "-fopenmp", *map(str, objs), "-o", str(tmp), "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
