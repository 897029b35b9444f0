"""Ray-id decoding by multiplication (hrt_device.cuh FastDiv, used by the lean diffuse trace to
split a ray id into face, primitive, ray and stratum): the shipped header compiled for the host
and checked against plain division for every divisor up to 70,000, powers of two and their
neighbours and 20,000 pseudo-random divisors, each over edge and pseudo-random numerators."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


@pytest.mark.skipif(_nvcc() is None, reason="nvcc not available")
def test_fast_div_equals_division(tmp_path):
    exe = str(tmp_path / "fastdiv_check")
    src = os.path.join(ROOT, "tests", "cpp", "fastdiv_check.cu")
    r = subprocess.run([_nvcc(), "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "helios_gb300", "csrc"), src,
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
