"""The C++ drop-in classes (include/vvgpu_modules.hpp) compile against libvvhd's own
headers and are used the way the reference driver uses stree / MConvectiveFast /
MEpsilonFast / MDiffusiveFast (type-level drop-in check; needs no GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_HEADERS = os.path.join(os.environ.get("VVD_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference")),
                           "libvvhd", "headers")


@pytest.mark.skipif(not os.path.isdir(REF_HEADERS), reason="reference headers not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_dropin_compiles_against_reference_headers():
    src = os.path.join(ROOT, "tests", "cxx", "simulate_like.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", REF_HEADERS,
                        "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_dropin_step_driver_compiles():
    """tests/cxx/dropin_step.cpp (run on the GPU by test_gpu_dropin.py) against the project's
    minimal host Space."""
    src = os.path.join(ROOT, "tests", "cxx", "dropin_step.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "tests", "cxx"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
