"""The header-only C++ facade (include/robast_gb.hpp) compiles against the
C ABI, translates status codes into exceptions and, on a GPU, traces through
rbg_trace_host with the reference's TraceNonSequential semantics."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "robast_gb300", "_build")


@pytest.fixture(scope="module")
def facade_bin(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from robast_gb300 import _native

    _native.lib()  # the library is built and loadable
    out = str(tmp_path_factory.mktemp("facade") / "facade_check")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"), "-L", LIBDIR, "-lrobast_gb",
           f"-Wl,-rpath,{LIBDIR}", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def _run(binary, mode):
    p = subprocess.run([binary, mode], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert f"facade_check {mode}: OK" in p.stdout


def test_facade_host_side(facade_bin):
    _run(facade_bin, "cpu")


@pytest.mark.gpu
def test_facade_trace(facade_bin):
    _run(facade_bin, "gpu")
