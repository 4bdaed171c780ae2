"""CPU test of the serving loop's device-range allocator: first-fit
placement, release with neighbour merging and the bookkeeping invariants,
against a brute-force bitmap model (tests/native/arena_check.cc)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def arena_bin(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("arena") / "arena_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "multians_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "arena_check.cc"), "-o", out],
                   check=True)
    return out


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_arena_matches_first_fit_model(arena_bin, seed):
    r = subprocess.run([arena_bin, str(seed), "20000"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
