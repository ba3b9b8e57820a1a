"""The C++ host API (include/degpu.hpp) compiles against the C ABI and, on a GPU, reproduces the
crate's known answers."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "host_api_example.cpp")
CSRC = os.path.join(REPO, "differential-equations_gb300", "csrc")


def build(out):
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), "-I", os.path.join(cuda, "include"), SRC,
           "-o", out, "-L", CSRC, "-ldegpu", f"-Wl,-rpath,{CSRC}"]
    subprocess.run(cmd, check=True)


def test_host_api_compiles_and_links(tmp_path):
    build(str(tmp_path / "host_api_example"))


@pytest.mark.gpu
def test_host_api_known_answers_on_gpu(tmp_path):
    exe = str(tmp_path / "host_api_example")
    build(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
