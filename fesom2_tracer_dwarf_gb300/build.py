"""In-tree build of libfesom_tracer_gb300.so for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked with nvcc. The
FP64 step is compiled with ``-fmad=false`` so that it rounds exactly as the
reference's statement order; host geometry code uses ``-ffp-contract=off``
for the same reason (aarch64 compilers contract by default).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUTDIR = os.path.join(PKG, "_build")
LIB_NAME = "libfesom_tracer_gb300.so"
LIB_PATH = os.path.join(PKG, "lib", LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
CXX_COMMON = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wextra",
              "-I", INCLUDE, "-I", CSRC]

SOURCES = [
    ("fgb_hmesh.cpp", "cxx", []),
    ("fgb_hmesh_files.cpp", "cxx", []),
    ("fgb_capi.cpp", "cxx", []),
    ("fgb_restart.cpp", "cxx", []),
    ("fgb_api.cu", "nvcc", []),
    ("fgb_step_f64.cu", "nvcc", ["-fmad=false"]),
    ("fgb_step_f64fast.cu", "nvcc", []),
    ("fgb_step_f32.cu", "nvcc", []),
    ("fgb_fast_kv1.cu", "nvcc", []),
    ("fgb_fast_kv2.cu", "nvcc", []),
    ("fgb_fast_kv4.cu", "nvcc", []),
    ("fgb_static_ws.cu", "nvcc", []),
    ("fgb_probe.cu", "nvcc", []),
    ("fgb_check.cu", "nvcc", []),
]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(f) for f in files + [__file__])


def _compile(src, kind, extra, nvcc):
    obj = os.path.join(OUTDIR, src + ".o")
    path = os.path.join(CSRC, src)
    if kind == "nvcc":
        cmd = [nvcc, *ARCH, *NVCC_COMMON, *extra, "-c", path, "-o", obj]
    else:
        cmd = ["g++", *CXX_COMMON, "-I", os.path.join(_cuda_home(nvcc), "include"), *extra, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (when sources changed) and return the library path."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _deps():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, s, k, e, nvcc) for s, k, e in SOURCES]
        objs = []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if verbose and log:
                sys.stderr.write(log)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
