"""Build the GPU library in-tree: crtmv3_gb300/libcrtm_gb300.so (sm_103a only)."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libcrtm_gb300.so")
# Translation units, compiled in parallel: the host runtime with the ODPS and
# forward scattering kernels, and per angle capacity one unit of the
# scattering K-matrix kernels per arithmetic form and one of the SOI layers'
# contraction.
SOURCES = ["crtm_gpu.cu", "scatter_k_d5.cu", "scatter_k_d10.cu", "scatter_k_d5f.cu", "scatter_k_d10f.cu",
           "scatter_soi_d5.cu", "scatter_soi_d10.cu"]
HEADERS = ["odps_physics.cuh", "odps_prep.cuh", "odps_kernels.cuh", "optran.cuh", "scatter_physics.cuh",
           "scatter_kernels.cuh", "scatter_adjoint.cuh", "scatter_launch.h", "dual.cuh", "dd.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "--expt-relaxed-constexpr", "-lineinfo", "-Xcompiler", "-fPIC"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "crtm_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    objdir = os.path.join(HERE, "_build")
    os.makedirs(objdir, exist_ok=True)
    procs = []
    for src in SOURCES:
        obj = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", "-o", obj, os.path.join(CSRC, src)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((obj, subprocess.Popen(cmd, cwd=CSRC, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                            text=True)))
    errors = []
    for obj, pr in procs:
        out, _ = pr.communicate()
        if pr.returncode != 0:
            errors.append(out)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + [o for o, _ in procs]
    res = subprocess.run(cmd, cwd=CSRC, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB
