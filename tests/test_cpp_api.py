"""The C++20 drop-in header compiles against the C ABI (CPU), and a program written against it
runs on the GPU (gpu)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests/cpp/api_drop_in.cpp"


def _cxx_cmd(out: Path, syntax_only: bool):
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-std=c++20", "-O1", "-ffp-contract=off", f"-I{ROOT / 'include'}", f"-I{cuda_inc}", str(SRC)]
    if syntax_only:
        return cmd + ["-fsyntax-only"]
    lib_dir = ROOT / "vren_gb300"
    return cmd + ["-o", str(out), f"-L{lib_dir}", "-lvren_gb300", f"-Wl,-rpath,{lib_dir}",
                  "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_header_compiles(native):
    subprocess.run(_cxx_cmd(Path("/dev/null"), True), check=True)


@pytest.mark.gpu
def test_cpp_drop_in_program_runs(cuda, tmp_path):
    exe = tmp_path / "api_drop_in"
    subprocess.run(_cxx_cmd(exe, False), check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    assert "api ok" in res.stdout
