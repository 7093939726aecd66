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
        src = re.sub(r"^\s*#[^\n]*", "", src, flags=re.M)  # preprocessor lines
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
    # C++ overloads the collision-counting wrappers (int& forms): name the C ones by their type
    cxx_sig = {"CSC_CSR_T_hash": "double(*)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, int32_t, int32_t*)",
               "CSC_CSR_T_hash_nonfuse": "double(*)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, "
                                         "int32_t, int32_t*)"}
    src += [f"  (fp)static_cast<{cxx_sig[n]}>({n})," if lang == "c++" and n in cxx_sig else f"  (fp){n},"
            for n in names] + ["};", "int main(void) {",
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


# The reference drivers' own call lines, verbatim (file:line in each comment):
# with only the include swapped they must compile and link against the library.
REFERENCE_CALLS = """
#include "spws/taco_abi.h"
#include <cstdio>
void calls(taco_tensor_t A, taco_tensor_t B, taco_tensor_t C, taco_tensor_t D, taco_tensor_t C_noT) {
    int w_cap = 1024, warmup = 5, repeat = 10;
    int collisions = 0;
    double duration_taco;
    duration_taco = CSR_CSR_hash(&A, &B, &C, w_cap, warmup, repeat, true);  // bench_hash_row_noT.cpp:46
    duration_taco = DCSC_DCSR_hash(&A, &B, &C, w_cap, warmup, repeat, true);  // bench_hash_outer_cc_noT.cpp:61
    DCSC_DCSR_coord(&A, &B, &C, w_cap);  // bench_coord_outer_cc_noT.cpp:52
    duration_taco = COO_CSF_DCSR_DCSR_hash(&A, &B, &C, &D, w_cap, warmup, repeat, true /* in bench*/, false/* verbose*/);  // bench_hash_mttkrp.cpp:37
    COO_CSF_DCSR_DCSR_coord(&A, &B, &C, &D, w_cap);  // bench_coord_mttkrp.cpp:45
    duration_taco = COO_CSF_DCSR_hash(&A, &B, &C, w_cap, warmup, repeat, true/*in bench*/);  // bench_hash_ttm.cpp:50
    duration_taco = COO_CSF_DCSR_bucket(&A, &B, &C, w_cap, warmup, repeat, true/*in bench*/);  // bench_bucket_ttm.cpp:43
    COO_CSF_DCSR_coord(&A, &B, &C, w_cap);  // bench_coord_ttm.cpp:45
    CSC_CSR_T_hash(&A, &B, &C, w_cap, collisions);  // get_collision_output.cpp:39
    CSC_CSR_T_hash_nonfuse(&A, &B, &C_noT, &C, w_cap, collisions);  // evaluate/CSC_CSR_T_hash_record_nofuse.h:405
    duration_taco = CSC_CSR_T_hash(&A, &B, &C, w_cap, warmup, repeat, true);  // DCSC_DCSR_T_hash.h:361 form
    CSC_CSR_T_coord(&A, &B, &C, w_cap);  // DCSC_DCSR_T_coord_index_chase_flex.h:381 form
    duration_taco = CSR_CSR_taco(&A, &B, &C, warmup, repeat, true);  // CSR_CSR_taco.h:108 form
    duration_taco = DCSC_DCSR_taco(&A, &B, &C, warmup, repeat, true);  // DCSC_DCSR_taco.h:136 form
    std::printf("%f %d\\n", duration_taco, collisions);
}
int main(int argc, char**) {
    if (argc > 99) calls(taco_tensor_t{}, taco_tensor_t{}, taco_tensor_t{}, taco_tensor_t{}, taco_tensor_t{});
    std::printf("%s\\n", spws_version());
    return 0;
}
"""


@pytest.mark.parametrize("select", ["", "-DSPWSBUCKET"])
def test_reference_call_sites_compile_unedited(built, tmp_path, select):
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("needs g++")
    (tmp_path / "drivers.cpp").write_text(REFERENCE_CALLS)
    libdir = os.path.dirname(built)
    cmd = [cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-Wno-unused-but-set-variable"]
    cmd += [select] if select else []
    cmd += ["-I", os.path.join(ROOT, "include"), str(tmp_path / "drivers.cpp"), "-o", str(tmp_path / "drivers"),
            f"-L{libdir}", "-lspws", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(tmp_path / "drivers")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "sm_103a" in r.stdout
    if select:  # the bucket selector routes the shared wrapper names to the bucket workspaces
        nm = subprocess.run(["nm", "-u", str(tmp_path / "drivers")], capture_output=True, text=True).stdout
        assert "DCSC_DCSR_bucket" in nm and "COO_CSF_DCSR_DCSR_bucket" in nm and "DCSC_DCSR_T_bucket" in nm
