"""The C++ facade (include/clear_cuda.hpp) compiles against the C ABI, links
the library and behaves: clr::Error with the status and message on failure
(CPU: constructing a builder without a GPU), a build, profiled pass times and
a closest-hit query through the facade (GPU)."""
import os
import subprocess
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "clear_gb300")
CUDA_INC = "/usr/local/cuda/include"


def _build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "facade_check")
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", f"-I{CUDA_INC}",
           os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"), "-o", exe, f"-L{PKG}", "-lclear_gb300",
           f"-Wl,-rpath,{PKG}", "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_facade_compiles_and_reports_errors(tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("the no-GPU path is checked where there is no GPU")
    res = subprocess.run([_build(tmp_path)], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "clr::Error" in res.stdout


@pytest.mark.gpu
def test_facade_builds_and_traces(cuda, tmp_path):
    res = subprocess.run([_build(tmp_path)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "hit 0 at t 1" in res.stdout
