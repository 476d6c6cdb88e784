"""CPU checks of the C ABI: the library builds, loads, and exports every
function include/*.h declares.  No compute calls (no GPU needed)."""
import ctypes
import glob
import os
import re

from tests.conftest import ROOT


def _declared_functions():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith("cosmos_"):
                names.add(name)
    return names


def test_header_declares_api():
    names = _declared_functions()
    assert "cosmos_pm_create" in names and "cosmos_pm_step" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(cosmos_lib):
    lib = ctypes.CDLL(cosmos_lib.LIB_PATH)
    missing = [n for n in sorted(_declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header(cosmos_lib):
    assert set(cosmos_lib.EXPORTS) >= {n for n in _declared_functions() if n.startswith(("cosmos_pm_", "cosmos_ensemble_"))}


def test_version_and_default_config(cosmos_lib):
    # pure host functions: no device work
    L = cosmos_lib.load()
    assert L.cosmos_pm_version().decode().count(".") == 2
    c = cosmos_lib.default_config()
    assert c.lattice_n == 2048 and c.deposit == cosmos_lib.DEPOSIT_CIC and c.use_graph == 1
    assert ctypes.sizeof(cosmos_lib.Config) == 4 * 4 + 8 + 4 * 5 + 4 * 7  # matches cosmos_pm_config


def test_default_blur_width(cosmos_lib):
    assert cosmos_lib.default_config().blur_r == 3


def test_universe_dropin_header_compiles():
    """include/CosmosGB300.cuh (the Universe<K> drop-in) compiles with plain
    g++ as the reference's user code would include it."""
    import shutil
    import subprocess
    import pytest
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "universe_test.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ensemble_config_layout(cosmos_lib):
    import ctypes as C
    assert C.sizeof(cosmos_lib.EnsembleConfig) == 4 * 8 + 4 * 8  # matches cosmos_ensemble_config


def test_ic_params_layout(cosmos_lib):
    import ctypes as C
    assert C.sizeof(cosmos_lib.IcParams) == 88  # matches cosmos_ic_params
