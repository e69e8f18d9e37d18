"""The C++ host API (include/lcx/accel_ext.hpp): compiles against the C ABI everywhere, runs on
a GPU."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _build_exe(tmp_path: Path) -> Path:
    from luisacompute_gb300 import build as b
    lib = b.build()
    cuda = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent
    exe = tmp_path / "test_accel_ext"
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}",
           str(ROOT / "tests" / "cpp" / "test_accel_ext.cpp"), "-o", str(exe), f"-L{lib.parent}", "-llcx_accel",
           f"-Wl,-rpath,{lib.parent}", f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_host_api_compiles(tmp_path):
    assert _build_exe(tmp_path).exists()


@pytest.mark.gpu
def test_cpp_host_api_runs(tmp_path):
    exe = _build_exe(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "accel_ext ok" in r.stdout
