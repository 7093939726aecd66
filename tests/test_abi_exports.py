"""CPU checks of the C-ABI library: it builds for sm_103a, loads, and exports
every function that include/spws/*.h declares (no compute calls: there is no
GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include", "spws")


def declared_functions():
    names = set()
    for f in sorted(os.listdir(INC)):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(INC, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", src):
            name = m.group(1)
            if name in ("if", "for", "while", "return", "sizeof"):
                continue
            names.add(name)
    return sorted(names)


@pytest.fixture(scope="module")
def built():
    from sparsews_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("spws_csr_csr_hash_compute", "CSR_CSR_hash", "spws_spgemm_csr_device", "spws_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_status_strings_without_gpu(built):
    from sparsews_gb300 import lib
    L = lib()
    assert L.spws_status_string(0) == b"ok"
    assert L.spws_status_string(1) == b"invalid argument"
    assert b"sm_103a" in L.spws_version()


def test_package_fails_loudly_without_library(tmp_path, monkeypatch):
    import sparsews_gb300 as pkg
    monkeypatch.setattr(pkg, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(pkg, "_lib", None)
    with pytest.raises(ImportError):
        pkg.lib()
