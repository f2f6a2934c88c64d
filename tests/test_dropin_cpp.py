"""The C++ drop-in header (include/nsl_gb300/nsl_dropin.hpp) compiles inside the reference's own templates.

Compile-only check against the reference NSL headers where the reference checkout is present (it is not on GPU
hosts); the classes are exercised on the GPU through the same C ABI by the -m gpu tests.
"""
import os
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("NSL_REFERENCE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "NSL")), reason="reference checkout not present")
def test_dropin_header_compiles_against_reference():
    torch = pytest.importorskip("torch")
    tdir = os.path.dirname(torch.__file__)
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-DFMT_HEADER_ONLY", "-w", f"-I{REF}/src/NSL", f"-I{REF}/src",
           f"-I{tdir}/include", f"-I{tdir}/include/torch/csrc/api/include",
           "-I" + os.path.join(ROOT, "oracle", "ref_harness"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_compile.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
