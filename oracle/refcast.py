"""ctypes front end of the REFERENCE's own CPU ray caster (test infrastructure only).

oracle/ref.mk compiles Helios core and the CollisionDetection plug-in from the reference
tree, unchanged, into oracle/_ref/libref_raycast.so; ``ref_raycast.cpp`` loads a scene into a
helios::Context with the caller's transforms and casts rays with
``CollisionDetection::castRaysSoA`` (plugins/collisiondetection/src/
CollisionDetection_RayTracing.cpp:551-680).  Only tests and the golden-vector script use it.
The reference tree must be present to build it (REF, default /root/reference); where it
is not, ``available()`` is False and the tests that need it skip.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libref_raycast.so")
_lib = None


def reference_root() -> str:
    return os.environ.get("HELIOS_REFERENCE", "/root/reference")


def available() -> bool:
    return os.path.exists(_LIB_PATH) or os.path.isdir(os.path.join(reference_root(), "plugins", "collisiondetection"))


def build() -> str:
    """Compile the reference ray caster (make -f ref.mk); a no-op when it is up to date."""
    ref = reference_root()
    if os.path.isdir(ref):
        jobs = str(max(os.cpu_count() or 1, 1))
        subprocess.run(["make", "-s", "-f", "ref.mk", f"REF={ref}", "-j", jobs], cwd=_HERE, check=True)
    if not os.path.exists(_LIB_PATH):
        raise ImportError("the reference ray caster is not built and the reference tree is absent")
    return _LIB_PATH


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        lib.ref_scene_create.restype = C.c_void_p
        lib.ref_scene_create.argtypes = [C.c_int32, C.c_void_p, C.c_void_p]
        lib.ref_cast_rays.restype = C.c_int
        lib.ref_cast_rays.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                                      C.c_void_p, C.c_int]
        lib.ref_scene_free.argtypes = [C.c_void_p]
        lib.ref_last_error.restype = C.c_char_p
        _lib = lib
    return _lib


class RefScene:
    """Patches (type 0) and triangles (type 1) with row-major 4x4 transforms T [n, 16]."""

    def __init__(self, T, ptype):
        self.lib = load()
        self._T = np.ascontiguousarray(T, np.float32).reshape(-1, 16)
        self._ty = np.ascontiguousarray(ptype, np.uint32)
        self.h = self.lib.ref_scene_create(self._T.shape[0], self._T.ctypes.data, self._ty.ctypes.data)
        if not self.h:
            raise RuntimeError(self.lib.ref_last_error().decode())

    def cast(self, o, d, max_distance=-1.0, threads=0):
        """Closest hits: (index [n] int64, -1 = miss; t [n] float32)."""
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = o.shape[0]
        idx = np.zeros(n, np.int64)
        t = np.zeros(n, np.float32)
        if self.lib.ref_cast_rays(self.h, n, o.ctypes.data, d.ctypes.data, float(max_distance), idx.ctypes.data,
                                  t.ctypes.data, int(threads)):
            raise RuntimeError(self.lib.ref_last_error().decode())
        return idx, t

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_scene_free(self.h)
            self.h = None
