"""Batches of independent scenes over the C ABI (cmag_batch_*).

A batch advances many scenes of any families and sizes with one set of launches
per step; each scene follows exactly the arithmetic of a single-scene system with
the same parameters and lanes per particle.  Scenes are addressed by their index
in the constructor's list; arrays are scene-local (n, 4) float32 numpy arrays.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import BatchGroup, SphParams
from ._lib import c_f32p, c_u32p, check, lib


def _fp(a):
    return a.ctypes.data_as(c_f32p)


class Batch:
    def __init__(self, params, counts):
        params = list(params)
        counts = [int(c) for c in counts]
        if len(params) != len(counts):
            raise ValueError("one particle count per scene")
        arr = (SphParams * len(params))(*[_abi.as_params(p).copy() for p in params])
        cnt = (ctypes.c_uint32 * len(counts))(*counts)
        self._h = ctypes.c_void_p()
        check(lib().cmag_batch_create(arr, cnt, len(params), ctypes.byref(self._h)))
        self.counts = counts
        self.num_scenes = len(counts)

    # -- lifetime --
    def close(self):
        if getattr(self, "_h", None):
            lib().cmag_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, rc):
        return check(rc, batch=self._h)

    # -- state --
    @property
    def num_particles(self):
        v = ctypes.c_uint32()
        self._chk(lib().cmag_batch_num_particles(self._h, ctypes.byref(v)))
        return v.value

    def scene_range(self, scene):
        a, n = ctypes.c_uint32(), ctypes.c_uint32()
        self._chk(lib().cmag_batch_scene_range(self._h, int(scene), ctypes.byref(a), ctypes.byref(n)))
        return a.value, n.value

    def reset(self, scene=None):
        if scene is None:
            self._chk(lib().cmag_batch_reset(self._h))
        else:
            self._chk(lib().cmag_batch_reset_scene(self._h, int(scene)))

    def set_array(self, scene, array, data, start=0):
        a = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, 4)
        self._chk(lib().cmag_batch_set_array(self._h, int(scene), int(array), _fp(a), int(start), a.shape[0]))

    def get_array(self, scene, array, start=0, count=None, out=None):
        """Scene-local rows [start, start + count); into `out` (a C-contiguous
        (count, 4) float32 array) when given."""
        count = self.counts[scene] - start if count is None else int(count)
        if out is None:
            out = np.empty((count, 4), np.float32)
        elif out.dtype != np.float32 or out.shape != (count, 4) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous (%d, 4) float32 array" % count)
        self._chk(lib().cmag_batch_get_array(self._h, int(scene), int(array), _fp(out), int(start), count))
        return out

    def set_array_all(self, array, data):
        """Every scene's rows at once, scenes one after another in scene order
        ((num_particles, 4) float32)."""
        a = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, 4)
        if a.shape[0] != self.num_particles:
            raise ValueError("expected %d rows" % self.num_particles)
        self._chk(lib().cmag_batch_set_array_all(self._h, int(array), _fp(a)))

    def get_array_all(self, array, out=None):
        """Every scene's rows, scenes one after another in scene order; into `out`
        (a C-contiguous (num_particles, 4) float32 array) when given."""
        n = self.num_particles
        if out is None:
            out = np.empty((n, 4), np.float32)
        elif out.dtype != np.float32 or out.shape != (n, 4) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous (%d, 4) float32 array" % n)
        self._chk(lib().cmag_batch_get_array_all(self._h, int(array), _fp(out)))
        return out

    def get_uint_array(self, scene, array, start=0, count=None):
        if count is None:
            if array in (_abi.CELLSTART, _abi.CELLEND):
                count = self.params(scene).num_grid_cells - start
            elif array == _abi.CELLOFFSET:
                raise ValueError("give count for CELLOFFSET (scan window + 1 entries)")
            else:
                count = self.counts[scene] - start
        out = np.empty(int(count), np.uint32)
        self._chk(lib().cmag_batch_get_uint_array(self._h, int(scene), int(array),
                                                  out.ctypes.data_as(c_u32p), int(start), int(count)))
        return out

    def device_array(self, array):
        return lib().cmag_batch_device_array(self._h, int(array))

    def params(self, scene):
        p = SphParams()
        self._chk(lib().cmag_batch_get_params(self._h, int(scene), ctypes.byref(p)))
        return p

    def set_params(self, scene, p):
        self._chk(lib().cmag_batch_set_params(self._h, int(scene), ctypes.byref(_abi.as_params(p))))

    def elapsed_time(self, scene):
        t = ctypes.c_float()
        self._chk(lib().cmag_batch_elapsed_time(self._h, int(scene), ctypes.byref(t)))
        return t.value

    # -- stepping --
    def update(self):
        self._chk(lib().cmag_batch_update(self._h))

    def update_n(self, steps):
        self._chk(lib().cmag_batch_update_n(self._h, int(steps)))

    def timed_update(self, steps):
        ms = ctypes.c_float()
        self._chk(lib().cmag_batch_timed_update(self._h, int(steps), ctypes.byref(ms)))
        return ms.value

    def run_stages(self, last_stage):
        self._chk(lib().cmag_batch_run_stages(self._h, int(last_stage)))

    # -- per-scene scene controls (reference methods) --
    def dambreak_change_right_boundary(self, scene):
        self._chk(lib().cmag_batch_dambreak_change_right_boundary(self._h, int(scene)))

    def dambreak_remove_right_boundary(self, scene):
        self._chk(lib().cmag_batch_dambreak_remove_right_boundary(self._h, int(scene)))

    def poiseuille_change_gravity(self, scene):
        self._chk(lib().cmag_batch_poiseuille_change_gravity(self._h, int(scene)))

    def fluid_extents(self):
        """(lo, hi): (scenes, 3) fluid bounding boxes from one device reduction."""
        lo = np.empty((self.num_scenes, 3), np.float32)
        hi = np.empty((self.num_scenes, 3), np.float32)
        self._chk(lib().cmag_batch_fluid_extents(self._h, _fp(lo), _fp(hi)))
        return lo, hi

    # -- execution control --
    def set_stream(self, stream):
        self._chk(lib().cmag_batch_set_stream(self._h, stream))

    def set_graphs(self, enable, steps_per_graph=1):
        self._chk(lib().cmag_batch_set_graphs(self._h, int(bool(enable)), int(steps_per_graph)))

    def synchronize(self):
        self._chk(lib().cmag_batch_synchronize(self._h))

    def device_error_bits(self):
        b = ctypes.c_uint32()
        self._chk(lib().cmag_batch_device_error_bits(self._h, ctypes.byref(b)))
        return b.value

    def groups(self):
        n = ctypes.c_uint32()
        self._chk(lib().cmag_batch_num_groups(self._h, ctypes.byref(n)))
        out = []
        for g in range(n.value):
            info = BatchGroup()
            self._chk(lib().cmag_batch_group_info(self._h, g, ctypes.byref(info)))
            out.append({k: getattr(info, k) for k, _ in BatchGroup._fields_})
        return out

    def scene_group(self, scene):
        g = ctypes.c_uint32()
        self._chk(lib().cmag_batch_scene_group(self._h, int(scene), ctypes.byref(g)))
        return g.value

    def set_group_lanes(self, group, density_lanes, force_lanes):
        self._chk(lib().cmag_batch_set_group_lanes(self._h, int(group), int(density_lanes), int(force_lanes)))

    def set_group_lists(self, group, enable):
        """Interaction lists for launch group `group` (one lane per particle, the
        same results as the one-lane cell walk) or the cell walk."""
        self._chk(lib().cmag_batch_set_group_lists(self._h, int(group), int(bool(enable))))

    def autotune(self, reps=3):
        self._chk(lib().cmag_batch_autotune(self._h, int(reps)))

    def set_wall_cache(self, enable):
        """Kept densities of dam-break walls (same bits either way; on by default)."""
        self._chk(lib().cmag_batch_set_wall_cache(self._h, int(bool(enable))))

    def wall_cache(self):
        e = ctypes.c_int32()
        self._chk(lib().cmag_batch_get_wall_cache(self._h, ctypes.byref(e)))
        return bool(e.value)

    def set_stage_timing(self, enable):
        self._chk(lib().cmag_batch_set_stage_timing(self._h, int(bool(enable))))

    def stage_times(self):
        ms = (ctypes.c_float * 6)()
        steps = ctypes.c_uint32()
        self._chk(lib().cmag_batch_stage_times(self._h, ms, ctypes.byref(steps)))
        return list(ms), steps.value
