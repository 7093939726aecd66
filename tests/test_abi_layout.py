"""CPU check that the ctypes mirrors of the C structs in include/spws/*.h have
the C compiler's sizes and field offsets (a mismatch would make the Python
front end pass garbage through the C ABI)."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def mirrors():
    import sparsews_gb300 as sp
    from sparsews_gb300 import served, taco
    return {
        "spws_csr_dev": sp.CsrDev,
        "spws_spgemm_stats": sp.SpgemmStats,
        "spws_spgemm_t_stats": sp.SpgemmTStats,
        "spws_batch_stats": sp.BatchStats,
        "spws_tuning": sp.Tuning,
        "taco_tensor_t": taco.TacoTensor,
        "spws_csf3_dev": served.Csf3Dev,
        "spws_factor_dev": served.FactorDev,
        "spws_coo_dev": served.CooDev,
        "spws_server_config": served.ServerConfig,
        "spws_request_info": served.RequestInfo,
        "spws_server_stats": served.ServerStats,
    }


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_struct_layouts_match_c(tmp_path):
    structs = mirrors()
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "spws/spws_server.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            a, b, v = line.split()
            got[(a, b)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, f"{cname}.{fname}"
