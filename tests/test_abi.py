"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
function that include/crtm_gpu.h declares (no compute calls here)."""
import ctypes as ct
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "crtm_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|long long|void|const char\*)\s+(crtm_gpu_\w+)\s*\(",
                                 src, flags=re.M)))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for f in ("crtm_gpu_init", "crtm_gpu_destroy", "crtm_gpu_forward", "crtm_gpu_k_matrix",
              "crtm_gpu_adjoint", "crtm_gpu_last_error"):
        assert f in names


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="no nvcc")
def test_library_exports_every_declared_symbol():
    from crtmv3_gb300 import build
    lib = ct.CDLL(build.build())
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_api_fails_loudly_without_library(monkeypatch, tmp_path):
    from crtmv3_gb300 import api
    monkeypatch.setattr(api, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(api, "_lib", None)
    with pytest.raises(RuntimeError):
        api.library()


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_ctypes_structs_match_the_header_layout(tmp_path):
    """Every field of the ctypes mirrors in crtmv3_gb300/api.py sits at the
    offset the C header gives it, and the structs have the same size."""
    import subprocess
    from crtmv3_gb300 import api
    structs = {"crtm_gpu_batch": api.CBatch, "crtm_gpu_rtsolution": api.CRTSolution,
               "crtm_gpu_kmatrix": api.CKMatrix, "crtm_gpu_adjoint_out": api.CAdjoint,
               "crtm_gpu_tl_in": api.CTLIn, "crtm_gpu_tuning": api.CTuning}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "crtm_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for line in out:
        if not line:
            continue
        cname, field, value = line.split()
        py = structs[cname]
        got = ct.sizeof(py) if field == "size" else getattr(py, field).offset
        assert got == int(value), (cname, field, got, value)
        seen += 1
    assert seen == sum(len(p._fields_) + 1 for p in structs.values())
