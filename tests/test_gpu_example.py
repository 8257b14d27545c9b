"""The drop-in C++ API run end to end on the GPU by a program that makes the
calls an Oz-AIE user makes (example/oztest.cpp: ozAIE_setup(256, 512, 128,
accurate) and ozAIE_DGEMM on std::vector arrays, the shape and calls of the
reference's example program), built against include/oz_aie.h and
liboz_gb300.so; it exits 0 when every entry equals the exact K.  The
reference's own example source compiles unchanged against the same header
(test_abi_host.py), where its sources are present."""
import os
import subprocess

import pytest

from conftest import HAVE_GPU, ROOT

pytestmark = pytest.mark.gpu


def test_example_program_runs_on_gpu(ozlib, tmp_path):
    if not HAVE_GPU:
        pytest.skip("no GPU")
    from ozaie_gb300 import _lib
    libdir = os.path.dirname(_lib.lib_path())
    exe = tmp_path / "oztest"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "example", "oztest.cpp"), "-L", libdir, "-loz_gb300",
                           "-Wl,-rpath," + libdir, "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "max |C - 128| = 0" in r.stdout
