"""ctypes wrapper of the reference's own DamBreak kernels on the GPU
(oracle/_ref/ref_dambreak_sm103a.cubin, driven by oracle/_ref/libref_gpu.so).

TEST INFRASTRUCTURE ONLY: the GPU tests compare the library with the reference's
kernels on the same inputs, and bench.py times them beside the library.  The
product never imports it.
"""
import ctypes
import os

import numpy as np

from . import oracle as O

_lib = None


def available():
    return os.path.exists(O.REF_GPU_CUBIN) and os.path.exists(O.REF_GPU_LIB)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError("the reference's GPU kernels are not built (%s)" % O.REF_GPU_CUBIN)
        L = ctypes.CDLL(O.REF_GPU_LIB)
        vp = ctypes.c_void_p
        L.ref_gpu_error.restype = ctypes.c_char_p
        L.ref_gpu_create.argtypes = [ctypes.c_char_p, vp, ctypes.c_uint32, O.c_f32p, ctypes.POINTER(vp)]
        L.ref_gpu_remove_right_boundary.argtypes = [vp, vp]
        L.ref_gpu_steps.argtypes = [vp, ctypes.c_uint32, O.c_f32p, O.c_f32p]
        L.ref_gpu_get.argtypes = [vp, ctypes.c_int32, O.c_f32p]
        L.ref_gpu_get_index.argtypes = [vp, O.c_u32p]
        L.ref_gpu_set.argtypes = [vp, ctypes.c_int32, O.c_f32p]
        L.ref_gpu_destroy.argtypes = [vp]
        _lib = L
    return _lib


class RefGpu:
    """One DamBreak scene advanced by the reference's kernels on the current GPU
    (DamBreakSystem::update order).  p: parameter block with power-of-two grid
    sizes; pos: (n, 4) float32 initial positions."""

    def __init__(self, p, pos):
        self.p = p.copy()
        self.n = int(pos.shape[0])
        pos = np.ascontiguousarray(pos, np.float32)
        self._h = ctypes.c_void_p()
        self._chk(lib().ref_gpu_create(O.REF_GPU_CUBIN.encode(), ctypes.byref(self.p), self.n, O.fp(pos),
                                       ctypes.byref(self._h)))

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError("reference GPU kernels: " + lib().ref_gpu_error().decode(errors="replace"))

    def remove_right_boundary(self):
        """removeRightBoundary: rightBoundary = 0xffffffff as a float, gate parked."""
        self.p.right_boundary = np.float32(float(0xFFFFFFFF))
        self._chk(lib().ref_gpu_remove_right_boundary(self._h, ctypes.byref(self.p)))

    def steps(self, k):
        self._chk(lib().ref_gpu_steps(self._h, int(k), None, None))

    def timed_steps(self, k):
        """Device milliseconds of k updates (events around them)."""
        ms = ctypes.c_float()
        self._chk(lib().ref_gpu_steps(self._h, int(k), ctypes.byref(ms), None))
        return ms.value

    def stage_ms(self, k):
        """Milliseconds per stage summed over k updates: hash, sort, reorder (with
        the cellStart clear), density, force, integrate."""
        out = (ctypes.c_float * 6)()
        self._chk(lib().ref_gpu_steps(self._h, int(k), None, out))
        return list(out)

    def get(self, array):
        out = np.empty((self.n, 4), np.float32)
        self._chk(lib().ref_gpu_get(self._h, int(array), O.fp(out)))
        return out

    def set(self, array, data):
        data = np.ascontiguousarray(data, np.float32)
        assert data.shape == (self.n, 4)
        self._chk(lib().ref_gpu_set(self._h, int(array), O.fp(data)))

    def index(self):
        out = np.empty(self.n, np.uint32)
        self._chk(lib().ref_gpu_get_index(self._h, O.up(out)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().ref_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
