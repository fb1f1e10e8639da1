"""The C++ facade (include/wfpt.hpp, the reference's Tracer / RayGen /
RayBuffer / Renderer names over the C ABI), compiled with g++ against
libwfpt.so the way reference-side C++ would use it."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA = Path("/usr/local/cuda")


@pytest.fixture(scope="module")
def facade_bin(wf, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib_dir = ROOT / "vulkanwavefrontpathtracer_gb300"
    out = tmp_path_factory.mktemp("cxx") / "facade_test"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "cxx" / "facade_test.cpp"), "-o", str(out), "-L", str(lib_dir), "-lwfpt",
           "-L", str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return out


def test_facade_host_mode(facade_bin):
    res = subprocess.run([str(facade_bin), "host"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and "FACADE OK" in res.stdout, res.stdout + res.stderr


@pytest.mark.gpu
def test_facade_trace_sort_matches_trace(facade_bin):
    res = subprocess.run([str(facade_bin), "gpu"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and "FACADE OK" in res.stdout, res.stdout + res.stderr
