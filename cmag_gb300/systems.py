"""Python mirror of the reference solver classes over the C ABI.

DamBreakSystem       DamBreak.Core/fluidSystem.h:6-113
PoiseuilleFlowSystem Poiseuille.Core/poiseuilleFlowSystem.h:6-112
PeristalsisSystem    Peristalsis.Core/PeristalsisSystem.h:6-132

Same constructor arguments, method names and array meaning/order as the
reference; arrays are exchanged as (n, 4) float32 numpy arrays (float4 rows).
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import SphParams, f3, u3
from ._lib import c_f32p, c_u32p, check, lib


def _fp(a):
    return a.ctypes.data_as(c_f32p)


class _System:
    POSITION = _abi.POSITION
    VELOCITY = _abi.VELOCITY
    MEASURES = _abi.MEASURES
    ACCELERATION = _abi.ACCELERATION
    VELOCITYLEAPFROG = _abi.VELOCITYLEAPFROG
    VISCOUSFORCE = _abi.VISCOUSFORCE
    PRESSUREFORCE = _abi.PRESSUREFORCE
    PREDICTEDPOSITION = _abi.PREDICTEDPOSITION
    SORTEDPOSITION = _abi.SORTEDPOSITION
    SORTEDVELOCITY = _abi.SORTEDVELOCITY

    def __init__(self, params, num_particles=None):
        L = lib()
        self._p = _abi.as_params(params).copy()
        if num_particles is None:
            n = ctypes.c_uint32()
            check(L.cmag_reference_particle_count(ctypes.byref(self._p), ctypes.byref(n)))
            num_particles = n.value
        self._h = ctypes.c_void_p()
        check(L.cmag_system_create(ctypes.byref(self._p), int(num_particles), ctypes.byref(self._h)))
        self.numParticles = int(num_particles)

    # -- lifetime --
    def close(self):
        if getattr(self, "_h", None):
            lib().cmag_system_destroy(self._h)
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
        return check(rc, self._h)

    # -- reference API --
    def update(self, dt=None):
        """One step (update(), fluidSystem.cpp:257-319); with dt, a step of that
        length, kept in the parameter block for later steps."""
        if dt is None:
            self._chk(lib().cmag_system_update(self._h))
        else:
            self._chk(lib().cmag_system_update_dt(self._h, float(dt)))
            self._p.delta_time = float(dt)

    def update_n(self, steps):
        self._chk(lib().cmag_system_update_n(self._h, int(steps)))

    def timed_update(self, steps):
        """Run `steps` steps; device milliseconds between events on the solver stream."""
        ms = ctypes.c_float()
        self._chk(lib().cmag_system_timed_update(self._h, int(steps), ctypes.byref(ms)))
        return ms.value

    def reset(self):
        self._chk(lib().cmag_system_reset(self._h))

    def getNumParticles(self):
        return self.numParticles

    def getElapsedTime(self):
        t = ctypes.c_float()
        self._chk(lib().cmag_system_elapsed_time(self._h, ctypes.byref(t)))
        return t.value

    def setArray(self, array, data, start=0, count=None):
        a = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, 4)
        count = a.shape[0] if count is None else int(count)
        self._chk(lib().cmag_system_set_array(self._h, int(array), _fp(a), int(start), count))

    def getArray(self, array, start=0, count=None, out=None):
        """Copy of a float4 array; into `out` (a C-contiguous float32 (count, 4)
        array, e.g. pinned host memory) when given."""
        count = self.numParticles - start if count is None else int(count)
        if out is None:
            out = np.empty((count, 4), np.float32)
        elif out.dtype != np.float32 or out.shape != (count, 4) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float32 array of shape (%d, 4)" % count)
        self._chk(lib().cmag_system_get_array(self._h, int(array), _fp(out), int(start), count))
        return out

    def setArrays(self, arrays):
        """Whole float4 arrays {array id: (n, 4) float32} in one call (one
        synchronisation)."""
        ids = list(arrays)
        data = [np.ascontiguousarray(arrays[a], dtype=np.float32).reshape(-1, 4) for a in ids]
        for a in data:
            if a.shape[0] != self.numParticles:
                raise ValueError("setArrays takes whole arrays of %d rows" % self.numParticles)
        ids_c = (ctypes.c_int32 * len(ids))(*ids)
        ptrs = (c_f32p * len(ids))(*[_fp(a) for a in data])
        self._chk(lib().cmag_system_set_arrays(self._h, len(ids), ids_c, ptrs))

    def getArrays(self, arrays):
        """Whole float4 arrays in one call: {array id: out} with `out` None or a
        C-contiguous float32 (n, 4) array (e.g. pinned memory); returns the dict
        of filled arrays."""
        out = {}
        for a, buf in arrays.items():
            if buf is None:
                buf = np.empty((self.numParticles, 4), np.float32)
            elif buf.dtype != np.float32 or buf.shape != (self.numParticles, 4) or not buf.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float32 array of shape (%d, 4)" % self.numParticles)
            out[a] = buf
        ids = list(out)
        ids_c = (ctypes.c_int32 * len(ids))(*ids)
        ptrs = (c_f32p * len(ids))(*[_fp(out[a]) for a in ids])
        self._chk(lib().cmag_system_get_arrays(self._h, len(ids), ids_c, ptrs))
        return out

    def getUintArray(self, array, start=0, count=None):
        if count is None:
            if array in (_abi.CELLSTART, _abi.CELLEND):
                count = self.numGridCells - start
            elif array == _abi.CELLOFFSET:
                raise ValueError("give count for CELLOFFSET (scan window + 1 entries)")
            else:
                count = self.numParticles - start
        out = np.empty(int(count), np.uint32)
        self._chk(lib().cmag_system_get_uint_array(self._h, int(array), out.ctypes.data_as(c_u32p),
                                                   int(start), int(count)))
        return out

    def getCudaArray(self, array):
        """Borrowed device pointer (getCudaPosVBO, getCudaMeasures, ...)."""
        return lib().cmag_system_device_array(self._h, int(array))

    def getCudaPosVBO(self):
        return self.getCudaArray(_abi.POSITION)

    def getCudaVelVBO(self):
        return self.getCudaArray(_abi.VELOCITY)

    def getCudaHash(self):
        return self.getCudaArray(_abi.HASH)

    def getCudaIndex(self):
        return self.getCudaArray(_abi.INDEX)

    def getCudaSortedPosition(self):
        return self.getCudaArray(_abi.SORTEDPOSITION)

    def getLeapFrogVelocity(self):
        return self.getCudaArray(_abi.VELOCITYLEAPFROG)

    @property
    def params(self):
        p = SphParams()
        self._chk(lib().cmag_system_get_params(self._h, ctypes.byref(p)))
        return p

    def set_params(self, p):
        self._chk(lib().cmag_system_set_params(self._h, ctypes.byref(_abi.as_params(p))))

    @property
    def numGridCells(self):
        v = ctypes.c_uint64()
        self._chk(lib().cmag_system_num_grid_cells(self._h, ctypes.byref(v)))
        return v.value

    def getParticleRadius(self):
        return self.params.particle_radius

    def getGridSize(self):
        return tuple(self.params.grid_size)

    def getWorldOrigin(self):
        return tuple(self.params.world_origin)

    def getCellSize(self):
        return tuple(self.params.cell_size)

    def getGravity(self):
        return tuple(self.params.gravity)

    def getHalfWorldXSize(self):
        p = self.params
        return np.float32(p.grid_size[0]) * np.float32(p.particle_radius)

    def getHalfWorldYSize(self):
        p = self.params
        return np.float32(p.grid_size[1]) * np.float32(p.particle_radius)

    def getHalfWorldZSize(self):
        p = self.params
        return np.float32(p.grid_size[2]) * np.float32(p.particle_radius)

    # -- extras: stages, streams, graphs, diagnostics --
    def run_stages(self, last_stage):
        self._chk(lib().cmag_system_run_stages(self._h, int(last_stage)))

    def synchronize(self):
        self._chk(lib().cmag_system_synchronize(self._h))

    def device_error_bits(self):
        b = ctypes.c_uint32()
        self._chk(lib().cmag_system_device_error_bits(self._h, ctypes.byref(b)))
        return b.value

    def set_graphs(self, enable):
        self._chk(lib().cmag_system_set_graphs(self._h, int(bool(enable))))

    def set_groups(self, density_lanes, force_lanes):
        self._chk(lib().cmag_system_set_groups(self._h, int(density_lanes), int(force_lanes)))

    def groups(self):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        self._chk(lib().cmag_system_get_groups(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def autotune(self, reps=3):
        """Pick lanes per particle and interaction lists by timing; returns
        (density lanes, force lanes, lists on)."""
        self._chk(lib().cmag_system_autotune(self._h, int(reps)))
        return self.groups() + (self.neighbor_lists()[0],)

    def set_verlet(self, skin):
        """Neighbour lists kept over several steps with this skin (in particle
        spacings; 0: the reference's per-step sort and walk)."""
        self._chk(lib().cmag_system_set_verlet(self._h, float(skin)))

    def verlet(self):
        """(skin, rebuilds so far)."""
        sk, nb = ctypes.c_float(), ctypes.c_uint32()
        self._chk(lib().cmag_system_get_verlet(self._h, ctypes.byref(sk), ctypes.byref(nb)))
        return sk.value, nb.value

    def set_neighbor_lists(self, enable, cap=None):
        """Interaction lists on/off; cap: entries per particle (default automatic)."""
        v = (int(cap) if cap else 1) if enable else 0
        self._chk(lib().cmag_system_set_neighbor_lists(self._h, v))

    def neighbor_lists(self):
        """(enabled, entries per particle)."""
        e, c = ctypes.c_int32(), ctypes.c_uint32()
        self._chk(lib().cmag_system_get_neighbor_lists(self._h, ctypes.byref(e), ctypes.byref(c)))
        return bool(e.value), c.value

    def set_wall_cache(self, enable):
        """DamBreak: keep the densities of non-fluid particles far from the fluid
        over steps (on by default; the results are the same bits either way)."""
        self._chk(lib().cmag_system_set_wall_cache(self._h, int(bool(enable))))

    def wall_cache(self):
        e = ctypes.c_int32()
        self._chk(lib().cmag_system_get_wall_cache(self._h, ctypes.byref(e)))
        return bool(e.value)

    def set_stage_timing(self, enable):
        self._chk(lib().cmag_system_set_stage_timing(self._h, int(bool(enable))))

    def stage_times(self):
        ms = (ctypes.c_float * 6)()
        steps = ctypes.c_uint32()
        self._chk(lib().cmag_system_stage_times(self._h, ms, ctypes.byref(steps)))
        return list(ms), steps.value

    def fluid_extent(self):
        """(min xyz, max xyz) over fluid particles, reduced on the device."""
        lo, hi = (ctypes.c_float * 3)(), (ctypes.c_float * 3)()
        self._chk(lib().cmag_system_fluid_extent(self._h, lo, hi))
        return tuple(lo), tuple(hi)

    def fluid_sum(self, array):
        """(sum of the float4 components over fluid particles, fluid count)."""
        s = (ctypes.c_double * 4)()
        c = ctypes.c_uint32()
        self._chk(lib().cmag_system_fluid_sum(self._h, int(array), s, ctypes.byref(c)))
        return tuple(s), c.value

    # -- headless colours and point view (the Demo programs' VBOs) --
    def colors(self):
        out = np.empty((self.numParticles, 4), np.float32)
        self._chk(lib().cmag_system_colors(self._h, _fp(out)))
        return out

    def render_ppm(self, path, width=512, height=0):
        self._chk(lib().cmag_system_render_ppm(self._h, str(path).encode(), int(width), int(height)))

    # -- learned closure (DamBreak) --
    def set_closure(self, closure):
        """Attach a cmag_gb300.closure.Closure (None detaches); it must outlive the
        attachment."""
        self._closure = closure
        self._chk(lib().cmag_system_set_closure(self._h, closure._h if closure is not None else None))

    def closure_features(self, dev_ptr):
        """Raw closure features of the last run_stages(FORCE) state into the device
        array at dev_ptr (num_particles x 16 floats, original order)."""
        self._chk(lib().cmag_system_closure_features(self._h, ctypes.c_void_p(int(dev_ptr))))

    def interpolate(self, array, points_ptr, n, out_ptr):
        """SPH interpolation of `array` over the fluid at n device points (n x 4
        floats at points_ptr) into out_ptr (n x 4: value, Shepard sum)."""
        self._chk(lib().cmag_system_interpolate(self._h, int(array), ctypes.c_void_p(int(points_ptr)),
                                                int(n), ctypes.c_void_p(int(out_ptr))))

    def set_elapsed_time(self, t):
        self._chk(lib().cmag_system_set_elapsed_time(self._h, float(t)))

    def load_state(self, st):
        """Restore arrays and time from a dict like state() returns, or from an
        oracle state object (attributes pos, vel, vlf, meas, acc[, vforce, pforce],
        phase = [elapsed, time_shift, time_relax, wave_height], p)."""
        get = (lambda k: st[k]) if isinstance(st, dict) else (lambda k: getattr(st, k))
        for k, a in (("pos", _abi.POSITION), ("vel", _abi.VELOCITY), ("vlf", _abi.VELOCITYLEAPFROG),
                     ("meas", _abi.MEASURES), ("acc", _abi.ACCELERATION)):
            self.setArray(a, get(k))
        if self._p.system == _abi.PERISTALSIS:
            self.setArray(_abi.VISCOUSFORCE, get("vforce"))
            self.setArray(_abi.PRESSUREFORCE, get("pforce"))
        if not isinstance(st, dict):
            p = self.params
            src = st.p
            p.right_boundary = src.right_boundary
            p.is_boundary_configuration = src.is_boundary_configuration
            p.particle_mass = src.particle_mass
            p.gravity[0], p.gravity[1], p.gravity[2] = src.gravity[0], src.gravity[1], src.gravity[2]
            self.set_params(p)
            ph = st.phase
            self.set_elapsed_time(float(ph[0]))
            if self._p.system == _abi.PERISTALSIS:
                self._chk(lib().cmag_peristalsis_set_phase(self._h, float(ph[3]), float(ph[2]),
                                                           float(ph[1]),
                                                           int(src.is_boundary_configuration)))

    def set_stream(self, stream_ptr):
        self._chk(lib().cmag_system_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def state(self):
        """All float4 arrays and the sorted integer arrays, as numpy."""
        out = {}
        names = {"pos": _abi.POSITION, "vel": _abi.VELOCITY, "vlf": _abi.VELOCITYLEAPFROG,
                 "meas": _abi.MEASURES, "acc": _abi.ACCELERATION,
                 "spos": _abi.SORTEDPOSITION, "svel": _abi.SORTEDVELOCITY}
        if self._p.system == _abi.PERISTALSIS:
            names.update(vforce=_abi.VISCOUSFORCE, pforce=_abi.PRESSUREFORCE)
        for k, a in names.items():
            out[k] = self.getArray(a)
        out["hash"] = self.getUintArray(_abi.HASH)
        out["idx"] = self.getUintArray(_abi.INDEX)
        return out


class DamBreakSystem(_System):
    """DamBreakSystem(uint3 fluidParticlesSize, int boundaryOffset, uint3 gridSize,
    float particleRadius, bool bUseOpenGL) -- fluidSystem.h:9-14.  `params` (an
    SphParams) replaces the reference derivation when given."""

    def __init__(self, fluidParticlesSize=None, boundaryOffset=None, gridSize=None,
                 particleRadius=None, bUseOpenGL=False, params=None, num_particles=None):
        if params is None:
            params = SphParams()
            check(lib().cmag_dambreak_default_params(u3(fluidParticlesSize), int(boundaryOffset),
                                                     u3(gridSize), float(particleRadius),
                                                     ctypes.byref(params)))
        super().__init__(params, num_particles)

    def changeRightBoundary(self):
        self._chk(lib().cmag_dambreak_change_right_boundary(self._h))

    def removeRightBoundary(self):
        self._chk(lib().cmag_dambreak_remove_right_boundary(self._h))

    def getCudaMeasures(self):
        return self.getCudaArray(_abi.MEASURES)

    def getCudaAcceleration(self):
        return self.getCudaArray(_abi.ACCELERATION)

    def scene3d(self, tank_cells, layers=3, jitter_frac=0.01, seed=1973):
        self._chk(lib().cmag_dambreak3d_scene(self._h, u3(tank_cells), int(layers),
                                              float(jitter_frac), int(seed)))


class PoiseuilleFlowSystem(_System):
    """PoiseuilleFlowSystem(fluidParticlesSize, boundaryOffset, gridSize, particleRadius,
    bUseOpenGL) -- poiseuilleFlowSystem.h:9-14."""

    def __init__(self, fluidParticlesSize=None, boundaryOffset=None, gridSize=None,
                 particleRadius=None, bUseOpenGL=False, params=None, num_particles=None):
        if params is None:
            params = SphParams()
            check(lib().cmag_poiseuille_default_params(u3(fluidParticlesSize), int(boundaryOffset),
                                                       u3(gridSize), float(particleRadius),
                                                       ctypes.byref(params)))
        super().__init__(params, num_particles)

    def changeGravity(self):
        self._chk(lib().cmag_poiseuille_change_gravity(self._h))

    def getCudaMeasures(self):
        return self.getCudaArray(_abi.MEASURES)

    def getCudaAcceleration(self):
        return self.getCudaArray(_abi.ACCELERATION)


class PeristalsisSystem(_System):
    """PeristalsisSystem(deltaTime, fluid_size, amplitude, wave_speed, soundspeed,
    gravity, boundaryOffset, gridSize, radius, bUseOpenGL) -- PeristalsisSystem.h:9-19."""

    def __init__(self, deltaTime=None, fluid_size=None, amplitude=None, wave_speed=None,
                 soundspeed=None, gravity=None, boundaryOffset=None, gridSize=None, radius=None,
                 bUseOpenGL=False, params=None, num_particles=None):
        if params is None:
            params = SphParams()
            check(lib().cmag_peristalsis_default_params(
                float(deltaTime), u3(fluid_size), float(amplitude), float(wave_speed),
                float(soundspeed), f3(gravity), int(boundaryOffset), u3(gridSize), float(radius),
                ctypes.byref(params)))
        super().__init__(params, num_particles)

    def Update(self, dt=None):
        self.update(dt)

    def Reset(self):
        self.reset()

    def GetElapsedTime(self):
        return self.getElapsedTime()

    def getradius(self):
        return self.getParticleRadius()

    def getMeasures(self):
        return self.getCudaArray(_abi.MEASURES)

    def viscous_force(self):
        return self.getCudaArray(_abi.VISCOUSFORCE)

    def pressure_force(self):
        return self.getCudaArray(_abi.PRESSUREFORCE)

    def getPredictedPos(self):
        return self.getCudaArray(_abi.PREDICTEDPOSITION)

    def getSortedVelocity(self):
        return self.getCudaArray(_abi.SORTEDVELOCITY)

    def phase(self):
        wh, tr, ts = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        bc = ctypes.c_int32()
        self._chk(lib().cmag_peristalsis_phase(self._h, ctypes.byref(wh), ctypes.byref(tr),
                                               ctypes.byref(ts), ctypes.byref(bc)))
        return {"current_wave_height": wh.value, "time_relax": tr.value, "time_shift": ts.value,
                "is_boundary_configuration": bc.value}


def sort_particles(d_hash, d_index, n, key_bits, stream=None):
    """sortParticles: stable in-place sort of device (hash, index) arrays."""
    check(lib().cmag_sort_particles(ctypes.cast(d_hash, c_u32p), ctypes.cast(d_index, c_u32p),
                                    int(n), int(key_bits), ctypes.c_void_p(stream or 0)))
