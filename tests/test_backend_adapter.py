"""The C++ adapter (helios::RayTracingBackend over the C ABI) compiles against the
reference's own plugin headers -- the drop-in boundary.  Skipped where the
reference tree is not present."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("HELIOS_REFERENCE_TREE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "plugins", "radiation", "include")) or not shutil.which("g++"),
                    reason="reference tree or g++ not available")
def test_adapter_compiles_against_reference_headers():
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall",
           "-I" + os.path.join(REF, "plugins", "radiation", "include"), "-I" + os.path.join(REF, "core", "include"),
           "-I" + os.path.join(REF, "core", "lib", "pugixml"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "helios_gb300", "backend", "GB300Backend.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
