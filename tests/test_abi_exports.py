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


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_c_and_cpp_callers_compile_link_and_run(built, tmp_path, lang):
    """A caller in C11 or C++17 includes every public header under -Wall
    -Wextra -Werror, takes the address of every declared entry point (so the
    link resolves each one against libspws.so), and runs a non-compute call."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("needs gcc/g++")
    names = declared_functions()
    heads = [f for f in sorted(os.listdir(INC)) if f.endswith(".h")]
    src = [f'#include "spws/{h}"' for h in heads] + ["#include <stdio.h>", "typedef void (*fp)(void);",
                                                     "static fp table[] = {"]
    src += [f"  (fp){n}," for n in names] + ["};", "int main(void) {",
                                            '  printf("%s %d\\n", spws_version(), (int)(sizeof table / sizeof *table));',
                                            "  return 0;", "}"]
    ext = "c" if lang == "c" else "cpp"
    (tmp_path / f"caller.{ext}").write_text("\n".join(src) + "\n")
    libdir = os.path.dirname(built)
    std = "-std=c11" if lang == "c" else "-std=c++17"
    r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(tmp_path / f"caller.{ext}"), "-o", str(tmp_path / "caller"), f"-L{libdir}", "-lspws",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(tmp_path / "caller")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "sm_103a" in r.stdout and r.stdout.split()[-1] == str(len(names))
