"""The argument checks of fgb_adv_step_static, on the CPU: the decision
function (csrc/fgb_static_ws_check.hpp, free of CUDA) is compiled into a small
program with g++ and driven with a mesh device that is not the current one, an
unknown precision, a bad tracer count and a mesh too large for the static
array. No GPU is needed and no device call is made."""
import os
import shutil
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fesom2_tracer_dwarf_gb300", "csrc")

PROGRAM = textwrap.dedent(r"""
    #include <cstdio>
    #include <cstdlib>
    #include <string>
    #include "fgb_static_ws_check.hpp"
    int main(int argc, char** argv) {
      if (argc != 7) return 2;
      std::string err;
      int rc = fgb::static_ws_precheck(atoi(argv[1]), atoi(argv[2]), atoll(argv[3]), atoll(argv[4]),
                                       atoi(argv[5]), atoi(argv[6]), &err);
      printf("%d %s\n", rc, err.c_str());
      return 0;
    }
""")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("static_ws")
    src, exe = d / "check.cpp", d / "check"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)

    def run(precision, ntracers, need, cap, mesh_dev, cur_dev):
        out = subprocess.run([str(exe), *map(str, (precision, ntracers, need, cap, mesh_dev, cur_dev))],
                             capture_output=True, text=True, check=True).stdout
        rc, _, msg = out.strip().partition(" ")
        return int(rc), msg

    return run


CAP = 64 << 20


def test_accepts_a_fitting_call_on_the_mesh_device(checker):
    assert checker(0, 2, 1 << 20, CAP, 0, 0) == (0, "")
    assert checker(1, 4, CAP, CAP, 3, 3) == (0, "")


def test_rejects_a_mesh_on_another_device(checker):
    rc, msg = checker(1, 4, 1 << 20, CAP, 1, 0)
    assert rc == -1
    assert "device 1" in msg and "current device is 0" in msg


def test_rejects_an_unknown_precision(checker):
    rc, msg = checker(3, 1, 1 << 20, CAP, 0, 0)
    assert rc == -1 and "unknown precision 3" in msg


def test_rejects_a_bad_tracer_count(checker):
    rc, msg = checker(0, 0, -1, CAP, 0, 0)
    assert rc == -1 and "tracer count" in msg


def test_rejects_meshes_beyond_the_static_array(checker):
    rc, msg = checker(0, 1, CAP + 1, CAP, 0, 0)
    assert rc == -1 and "static workspace" in msg and str(CAP) in msg
