"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(mrmd_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from mrmd_gb300 import build as B

    path = B.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "mrmd_lj_apply" in names and "mrmd_nlist_build" in names
    assert len(names) > 50


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from mrmd_gb300 import _abi

    missing = sorted(set(declared_functions()) - set(_abi.SIGNATURES))
    assert not missing, missing


def test_binary_targets_sm_103a(lib):
    from mrmd_gb300 import build as B

    flags = " ".join(B.NVCC_FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags


def test_version_string(lib):
    lib.mrmd_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.mrmd_version()


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from mrmd_gb300 import _abi

    monkeypatch.setattr(_abi, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(_abi, "_lib", None)
    with pytest.raises(_abi.MrmdError):
        _abi.lib()


def test_library_exports_nothing_undeclared(lib):
    """Every exported mrmd_* symbol is declared in include/*.h: no entry point
    outside the documented boundary."""
    import shutil
    import subprocess

    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    from mrmd_gb300 import build as B

    out = subprocess.run([nm, "-D", "--defined-only", B.LIB], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.split() and line.split()[-1].startswith("mrmd_")}
    assert exported, "no mrmd_* exports found"
    undeclared = sorted(exported - set(declared_functions()))
    assert not undeclared, undeclared
