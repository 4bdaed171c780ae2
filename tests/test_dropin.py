"""The reference's C++ API as a user's program sees it: a C++ program
written against include/ (reference class names, reference call sequence)
compiles and links against libmultians_gb300.so on the CPU, and on a GPU
decodes its streams bit-exactly (tests/native/dropin_demo.cc)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path_factory, mg):
    cxx = shutil.which("g++")
    if not cxx or not os.path.isdir(os.path.join(CUDA, "include")):
        pytest.skip("g++ or the CUDA headers are not available")
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_demo")
    libdir = os.path.dirname(mg.LIB_PATH)
    cudalib = next((d for d in (os.path.join(CUDA, "lib64"), os.path.join(CUDA, "lib"),
                                os.path.join(CUDA, "targets", "sbsa-linux", "lib"),
                                os.path.join(CUDA, "targets", "x86_64-linux", "lib"))
                    if os.path.exists(os.path.join(d, "libcudart.so"))), None)
    if cudalib is None:
        pytest.skip("libcudart.so not found")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(CUDA, "include"),
                    os.path.join(ROOT, "tests", "native", "dropin_demo.cc"), "-o", out,
                    "-L", libdir, "-lmultians_gb300", "-L", cudalib, "-lcudart",
                    f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cudalib}"], check=True)
    return out


@pytest.fixture(scope="module")
def demo(tmp_path_factory, mg):
    return _build(tmp_path_factory, mg)


def test_dropin_program_builds_against_reference_api(demo):
    assert os.path.exists(demo)


@pytest.mark.gpu
def test_dropin_program_decodes_bit_exact(demo):
    r = subprocess.run([demo], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" ok") == 4, r.stdout
