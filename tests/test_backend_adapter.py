"""The C++ adapter (helios::RayTracingBackend over the C ABI) and its runBand driver compile
against the reference's own plugin headers -- the drop-in boundary -- and against the test
stand-in the GPU test uses (tests/cpp/helios_api).  The reference tree's location comes from
the oracle's build recipe (oracle/refcast.py, HELIOS_REFERENCE); skipped where it is absent."""
import os
import shutil
import subprocess

import pytest

import refcast

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = refcast.reference_root()
HAVE_REF = os.path.isdir(os.path.join(REF, "plugins", "radiation", "include"))
SOURCES = [os.path.join(ROOT, "helios_gb300", "backend", "GB300Backend.cpp"),
           os.path.join(ROOT, "tests", "cpp", "adapter_runband.cpp")]


def _syntax(includes, src):
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", *["-I" + i for i in includes],
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "helios_gb300", "backend"), src]
    return subprocess.run(cmd, capture_output=True, text=True)


@pytest.mark.skipif(not HAVE_REF or not shutil.which("g++"), reason="reference tree or g++ not available")
@pytest.mark.parametrize("src", SOURCES, ids=["adapter", "runband_driver"])
def test_compiles_against_reference_headers(src):
    inc = [os.path.join(REF, "plugins", "radiation", "include"), os.path.join(REF, "core", "include"),
           os.path.join(REF, "core", "lib", "pugixml")]
    r = _syntax(inc, src)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.skipif(not shutil.which("g++"), reason="g++ not available")
@pytest.mark.parametrize("src", SOURCES, ids=["adapter", "runband_driver"])
def test_compiles_against_test_stand_in(src):
    r = _syntax([os.path.join(ROOT, "tests", "cpp", "helios_api")], src)
    assert r.returncode == 0, r.stderr[-2000:]
