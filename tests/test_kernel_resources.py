"""Register budgets of the FP32 step's kernels, read from ptxas's resource
report (`-Xptxas -v`) for sm_103a; no GPU is needed.

The kernels the 2048x2048x64 residual-form step runs (the whole-column LO
kernel with compensated sums, the lean whole-column ratio kernel, the update
with the rounding residual, the tiled edge-flux kernel, the volume fluxes;
the node kernels also for groups of 2 tracers) compile without local-memory
spills at their launch bounds. A spill keeps a thread's values in local
memory, read back through L1 inside the gathers; the compensated LO kernel
once lost 17 % of its time to one. The register counts must also fit the
resident blocks the launch bounds ask for.
"""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# kernel -> blocks of 128 threads per SM its launch bounds ask for (None: 256-thread
# or tile kernels, checked for spills only)
EXPECTED = {
    "kf_lo64<3, 4, false, false, false>": 7,
    "kf_lo64<3, 4, false, false, true>": 7,
    "kf_ratio64<4, true, false>": 8,
    "kf_ratio64<4, false, false>": 7,
    "kf_update<4, 1, false, false, false>": 9,
    "kf_update<4, 1, false, false, true>": 8,
    "kf_hflux_tile<1, true, 4>": None,
    "kf_hflux_tile<2, true, 4>": None,
    "kf_vflux": None,
    "kf_lo64<3, 2, false, false, true>": 7,
    "kf_ratio64<2, true, false>": 8,
    "kf_update<2, 1, false, false, true>": 8,
}


def _resource_report(tmp_path):
    from fesom2_tracer_dwarf_gb300 import build as B

    try:
        nvcc = B._nvcc()
    except RuntimeError:
        pytest.skip("nvcc is not installed")
    if shutil.which("c++filt") is None:
        pytest.skip("c++filt is not installed")
    cmd = [nvcc, *B.ARCH, *B.NVCC_COMMON, "-Xptxas", "-v", "-c", os.path.join(HERE, "kernel_resources.cu"),
           "-o", str(tmp_path / "kernel_resources.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    text = subprocess.run(["c++filt"], input=r.stdout + r.stderr, capture_output=True, text=True).stdout
    out, cur = {}, None
    for line in text.splitlines():
        m = re.search(r"Compiling entry function '(?:void )?(?:fgb::fast::)?([^(']+)", line)
        if m:
            cur = m.group(1).strip()
            out[cur] = {}
            continue
        if cur is None:
            continue
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m:
            out[cur]["spill"] = (int(m.group(1)), int(m.group(2)))
        m = re.search(r"Used (\d+) registers", line)
        if m:
            out[cur]["regs"] = int(m.group(1))
    return out


def test_step_kernels_compile_without_spills(tmp_path):
    rep = _resource_report(tmp_path)
    for name, blocks in EXPECTED.items():
        assert name in rep, f"{name} not in the report: {sorted(rep)}"
        info = rep[name]
        assert info.get("spill") == (0, 0), f"{name} spills: {info}"
        if blocks is not None:
            # 65536 registers per SM over `blocks` blocks of 128 threads
            assert info["regs"] <= 65536 // (blocks * 128), f"{name}: {info['regs']} registers for {blocks} blocks"
