"""The Universe<K> drop-in (include/CosmosGB300.cuh) from C++: compiled with
g++ against libcosmos_pm.so and run through the reference's main.cu sequence
(tests/cpp/universe_test.cpp), for both accuracy modes."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cosmossimulationwithcuda_gb300")


@pytest.fixture(scope="module")
def universe_exe(tmp_path_factory):
    from cosmossimulationwithcuda_gb300 import _lib
    _lib.load()  # the library must exist
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("universe") / "universe_test")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "universe_test.cpp"), "-L", PKG, "-lcosmos_pm",
           f"-Wl,-rpath,{PKG}", "-pthread", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


@pytest.mark.parametrize("low_accuracy", [1, 0])
def test_universe_dropin(universe_exe, low_accuracy):
    r = subprocess.run([universe_exe, str(low_accuracy)], capture_output=True, text=True, timeout=300)
    lines = [l for l in r.stdout.splitlines() if l.startswith(("PASS", "FAIL"))]
    assert r.returncode == 0 and lines and lines[-1].startswith("PASS"), r.stdout + r.stderr
