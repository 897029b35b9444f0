"""The C-ABI library builds for sm_103a, loads, and exports every symbol include/hrt.h declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "hrt.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|size_t|int64_t|const char \*)\s*(hrt_\w+)\s*\(", src, re.M)))


def test_header_matches_binding():
    from helios_gb300 import _hrt
    assert declared() == sorted(_hrt.EXPORTS)


def test_library_exports_all(hrt_lib):
    for name in declared():
        assert hasattr(hrt_lib, name), name


def test_backend_name(hrt_lib):
    assert b"GB300" in hrt_lib.hrt_backend_name()


def test_no_cpu_fallback_path():
    """The product package never imports, loads or runs the oracle."""
    pkg = os.path.join(ROOT, "helios_gb300")
    pat = re.compile(r"(import\s+oracle|from\s+oracle|hrt_oracle|libhrt_oracle)")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dirpath, f)).read()
                assert not pat.search(txt), f
