"""The roofline numerator of the cloudy K-matrix's layer reverse sweep:
bench.py's per-layer operation table against a count taken by running the
kernel's own header code (phase blocks, loss-form MOM and its reverse sweep,
the phase blocks' adjoint) on an operation-counting number type."""
import ctypes as ct
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def fc(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("fc") / "libfc.so")
    subprocess.run([cxx, "-O1", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "crtmv3_gb300", "csrc"),
                    "-o", out, os.path.join(HERE, "harness", "flop_count.cpp")], check=True)
    lib = ct.CDLL(out)
    lib.fc_layer_ops.restype = ct.c_longlong
    lib.fc_layer_ops.argtypes = [ct.c_int, ct.c_double, ct.c_double, ct.c_double]
    return lib


def test_reverse_layer_ops_table(fc):
    import bench
    for nleg in (2, 4, 6, 8, 16):
        nz = (nleg + 2) // 2 + 1
        counts = [fc.fc_layer_ops(nleg, mu, w, tau) for mu in (0.6, 0.73, 0.91, 0.99)
                  for w, tau in ((0.5, 0.3), (0.95, 3.0), (0.2, 0.01), (0.99, 30.0))]
        assert min(counts) > 0
        table = bench.REVERSE_LAYER_OPS[nz]
        # the Jacobi sweep count varies a little with the layer
        assert 0.95 * table <= min(counts) and max(counts) <= 1.05 * table, (nz, min(counts), max(counts))
