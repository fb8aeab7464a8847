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
