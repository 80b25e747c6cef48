"""ctypes wrapper of the CPU oracle and of the reference-on-CPU libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

* ``OracleState``: the C restatement (oracle/cmag_oracle.c) of one solver's
  state and update().
* ``RefState``: the reference's own kernel sources compiled for the CPU
  (oracle/_ref, built by oracle/ref/Makefile where the reference tree exists),
  driven in the order of the reference update()/Update().
"""
import ctypes
import os
import subprocess

import numpy as np

from .params import DAMBREAK, PERISTALSIS, POISEUILLE, STAGE_INTEGRATE, SphParams, f3, u3

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None
_ref = {}

P = ctypes.POINTER
c_u32p = P(ctypes.c_uint32)
c_f32p = P(ctypes.c_float)


def build(quiet=True):
    """Compile the oracle (gcc; used on every host, including the GPU machine)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _ref_make_args(ref_root):
    # the tree: the argument, else what oracle/ref/Makefile resolves (REF=,
    # CMAG_REFERENCE)
    return ["make", "-s", "-C", os.path.join(HERE, "ref")] + (["REF=" + ref_root] if ref_root else [])


def have_ref(ref_root=None):
    """Whether the reference tree the recipe reads is present on this host."""
    return subprocess.run(_ref_make_args(ref_root) + ["have-ref"], capture_output=True).returncode == 0


def build_ref(ref_root=None):
    """Compile oracle/_ref from the reference sources, where the tree exists."""
    if not have_ref(ref_root):
        return False
    out = subprocess.run(_ref_make_args(ref_root), capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle/_ref build failed:\n" + out.stdout + out.stderr)
    return True


REF_GPU_CUBIN = os.path.join(REF_DIR, "ref_dambreak_sm103a.cubin")
REF_GPU_LIB = os.path.join(REF_DIR, "libref_gpu.so")


def build_ref_gpu(ref_root=None):
    """The reference's DamBreak kernels for the GPU: the cubin where the reference
    tree exists, and the launcher wherever the cubin exists.  Returns whether
    the launcher is ready."""
    if have_ref(ref_root):
        out = subprocess.run(_ref_make_args(ref_root) + ["gpu-cubin"], capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("reference cubin build failed:\n" + out.stdout + out.stderr)
    if not os.path.exists(REF_GPU_CUBIN):
        return False
    out = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "gpu-launcher"], capture_output=True,
                         text=True)
    if out.returncode != 0:
        raise RuntimeError("reference GPU launcher build failed:\n" + out.stdout + out.stderr)
    return True


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        # parameter blocks by address: the oracle's SphParams or the product's
        # mirror of the same struct
        sp = ctypes.c_void_p
        L.orc_dambreak_params.argtypes = [c_u32p, ctypes.c_int32, c_u32p, ctypes.c_float, sp]
        L.orc_poiseuille_params.argtypes = [c_u32p, ctypes.c_int32, c_u32p, ctypes.c_float, sp]
        L.orc_peristalsis_params.argtypes = [ctypes.c_float, c_u32p, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_float, c_f32p, ctypes.c_int32, c_u32p,
                                             ctypes.c_float, sp]
        L.orc_particle_count.argtypes = [sp]
        L.orc_particle_count.restype = ctypes.c_uint32
        L.orc_scene.argtypes = [sp, c_f32p, ctypes.c_uint32]
        L.orc_peristalsis_mass_sum.argtypes = [sp, c_f32p, ctypes.c_uint32]
        L.orc_peristalsis_mass_sum.restype = ctypes.c_float
        L.orc_dambreak3d_count.argtypes = [c_u32p, c_u32p, ctypes.c_uint32]
        L.orc_dambreak3d_count.restype = ctypes.c_uint32
        L.orc_dambreak3d_scene.argtypes = [sp, c_u32p, ctypes.c_uint32, ctypes.c_float,
                                           ctypes.c_uint64, c_f32p, ctypes.c_uint32]
        L.orc_calc_hash.argtypes = [sp, c_f32p, c_u32p, c_u32p, ctypes.c_uint32]
        L.orc_sort_pairs.argtypes = [c_u32p, c_u32p, ctypes.c_uint32]
        L.orc_reorder.argtypes = [c_u32p, c_u32p, c_f32p, c_f32p, c_u32p, c_u32p, c_f32p, c_f32p,
                                  ctypes.c_uint32, ctypes.c_uint64]
        L.orc_density.argtypes = [sp, c_f32p, c_f32p, c_u32p, c_u32p, ctypes.c_uint32, ctypes.c_int]
        L.orc_force.argtypes = [sp, c_f32p, c_f32p, c_f32p, c_u32p, c_u32p, c_u32p, c_f32p, c_f32p,
                                ctypes.c_uint32, ctypes.c_int]
        L.orc_force_scale.argtypes = [sp, c_f32p, c_f32p, c_f32p, c_u32p, c_u32p, c_u32p, c_f32p,
                                      c_f32p, ctypes.c_uint32, ctypes.c_int]
        L.orc_set_wall_state.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int32]
        L.orc_density_at.argtypes = [sp, c_f32p, c_u32p, c_u32p, ctypes.c_uint32]
        L.orc_density_at.restype = ctypes.c_float
        L.orc_force_at.argtypes = [sp, c_f32p, c_f32p, c_f32p, c_u32p, c_u32p, ctypes.c_uint32,
                                   c_f32p, c_f32p, P(ctypes.c_int32)]
        L.orc_integrate.argtypes = [sp, c_f32p, c_f32p, c_f32p, c_f32p, c_f32p, c_f32p,
                                    ctypes.c_float, ctypes.c_uint32]
        L.orc_configure_boundary.argtypes = [sp, c_f32p, ctypes.c_float, ctypes.c_uint32]
        L.orc_shift_right_boundary.argtypes = [sp, c_f32p, ctypes.c_uint32]
        L.orc_remove_right_boundary.argtypes = [sp, c_f32p, ctypes.c_uint32]
        L.orc_step.argtypes = [sp, ctypes.c_uint32, ctypes.c_uint64] + [c_f32p] * 9 + \
            [c_u32p] * 4 + [c_f32p, ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def fp(a):
    return a.ctypes.data_as(c_f32p)


def up(a):
    return a.ctypes.data_as(c_u32p)


# ---------------------------------------------------------------------------
# parameter blocks and scenes
# ---------------------------------------------------------------------------

def dambreak_params(fluid_size, boundary_offset, grid_size, radius):
    p = SphParams()
    lib().orc_dambreak_params(u3(fluid_size), boundary_offset, u3(grid_size), radius,
                              ctypes.byref(p))
    return p


def poiseuille_params(fluid_size, boundary_offset, grid_size, radius):
    p = SphParams()
    lib().orc_poiseuille_params(u3(fluid_size), boundary_offset, u3(grid_size), radius,
                                ctypes.byref(p))
    return p


def peristalsis_params(dt, fluid_size, amplitude, wave_speed, soundspeed, gravity,
                       boundary_offset, grid_size, radius):
    p = SphParams()
    lib().orc_peristalsis_params(dt, u3(fluid_size), amplitude, wave_speed, soundspeed,
                                 f3(gravity), boundary_offset, u3(grid_size), radius,
                                 ctypes.byref(p))
    return p


def particle_count(p):
    return int(lib().orc_particle_count(ctypes.byref(p)))


def scene(p, n=None):
    n = particle_count(p) if n is None else n
    pos = np.zeros((n, 4), np.float32)
    lib().orc_scene(ctypes.byref(p), fp(pos), n)
    return pos


def dambreak3d_count(fluid_size, tank_cells, layers):
    return int(lib().orc_dambreak3d_count(u3(fluid_size), u3(tank_cells), layers))


def dambreak3d_scene(p, tank_cells, layers, jitter_frac, seed):
    n = dambreak3d_count(p.fluid_size, tank_cells, layers)
    pos = np.zeros((n, 4), np.float32)
    lib().orc_dambreak3d_scene(ctypes.byref(p), u3(tank_cells), layers, jitter_frac, seed,
                               fp(pos), n)
    return pos


# ---------------------------------------------------------------------------
# solver state
# ---------------------------------------------------------------------------

class _StateBase:
    """Arrays of one solver (float4 AoS as (n, 4) float32, like the reference)."""

    def __init__(self, params, n):
        self.p = params.copy()
        self.n = int(n)
        self.ncells = self.p.num_grid_cells
        z4 = lambda: np.zeros((self.n, 4), np.float32)
        self.pos, self.vel, self.vlf, self.meas = z4(), z4(), z4(), z4()
        self.acc, self.vforce, self.pforce = z4(), z4(), z4()
        self.spos, self.svel = z4(), z4()
        self.hash = np.zeros(self.n, np.uint32)
        self.idx = np.zeros(self.n, np.uint32)
        self.cell_start = np.full(self.ncells, 0xFFFFFFFF, np.uint32)
        self.cell_end = np.zeros(self.ncells, np.uint32)
        # elapsed, time_shift, time_relax, current_wave_height, t of the last integration
        self.phase = np.zeros(5, np.float32)

    def reset_reference(self):
        """reset()/Reset(): reference scene and initial arrays."""
        self.pos[:] = scene(self.p, self.n)
        for a in (self.vel, self.vlf, self.acc, self.vforce, self.pforce, self.meas):
            a[:] = 0
        self.phase[:] = 0
        if self.p.system in (DAMBREAK, POISEUILLE):
            self.meas[:, 0] = self.p.rest_density  # fluidSystem.cpp:131-132
        if self.p.system == DAMBREAK:               # fluidSystem.cpp:378-379
            self.p.right_boundary = dambreak_params(self.p.fluid_size, self.p.boundary_offset,
                                                    self.p.grid_size,
                                                    self.p.particle_radius).right_boundary
        if self.p.system == PERISTALSIS:            # PeristalsisSystem.cpp:213-236
            self.phase[2] = np.float32(1000) * np.float32(self.p.delta_time)
            self.p.is_boundary_configuration = 1
            s = lib().orc_peristalsis_mass_sum(ctypes.byref(self.p), fp(self.pos), self.n)
            self.p.particle_mass = np.float32(np.float32(self.p.rest_density) / np.float32(s))
        return self

    def set_state(self, other):
        """Copy every array and the phase from another state."""
        for name in ("pos", "vel", "vlf", "meas", "acc", "vforce", "pforce"):
            getattr(self, name)[:] = getattr(other, name)
        self.phase[:] = other.phase
        self.p = other.p.copy()
        return self

    @property
    def elapsed(self):
        return float(self.phase[0])


def integrate_from(pre, post, acc, vforce, pforce):
    """The integration of the step pre -> post recomputed from given forces:
    pre's arrays (walls placed by configureBoundary first when that step ran it),
    post's parameters and time.  Returns (pos, vel, vlf)."""
    pos, vel, vlf = pre.pos.copy(), pre.vel.copy(), pre.vlf.copy()
    p = post.p
    if (p.system == PERISTALSIS and pre.p.is_boundary_configuration
            and pre.phase[3] < np.float32(pre.p.amplitude)):
        lib().orc_configure_boundary(ctypes.byref(pre.p), fp(pos), float(pre.phase[3]), pre.n)
    acc = np.ascontiguousarray(acc, np.float32)
    vforce = np.ascontiguousarray(vforce, np.float32)
    pforce = np.ascontiguousarray(pforce, np.float32)
    lib().orc_integrate(ctypes.byref(p), fp(pos), fp(vel), fp(vlf), fp(acc), fp(vforce), fp(pforce),
                        float(post.phase[4]), pre.n)
    return pos, vel, vlf


class OracleState(_StateBase):
    """One solver advanced by the C restatement."""

    def step(self, stop_after=STAGE_INTEGRATE, threads=1):
        lib().orc_step(ctypes.byref(self.p), self.n, self.ncells, fp(self.pos), fp(self.vel),
                       fp(self.vlf), fp(self.meas), fp(self.acc), fp(self.vforce),
                       fp(self.pforce), fp(self.spos), fp(self.svel), up(self.hash), up(self.idx),
                       up(self.cell_start), up(self.cell_end), fp(self.phase), threads,
                       stop_after)
        return self

    def force_scale(self, threads=1):
        """Per particle (original order) sum of |pair term| of this step's forces,
        evaluated on the current sorted arrays: (scale_a, scale_b) as (n, 4)."""
        sa = np.zeros((self.n, 4), np.float32)
        sb = np.zeros((self.n, 4), np.float32)
        lib().orc_force_scale(ctypes.byref(self.p), fp(self.spos), fp(self.svel), fp(self.meas),
                              up(self.idx), up(self.cell_start), up(self.cell_end), fp(sa), fp(sb),
                              self.n, threads)
        return sa, sb

    def forces_on(self, meas, spos=None, svel=None, threads=1, wall=None):
        """This step's forces recomputed on given sorted inputs (e.g. another
        implementation's measures), with this state's sort and cell ranges.
        wall: (amplitude, time, moving) of the Peristalsis wall law for the
        no-slip option.  Returns (out_a, out_b, scale_a, scale_b), original order."""
        if wall is not None:
            lib().orc_set_wall_state(float(wall[0]), float(wall[1]), int(wall[2]))
        meas = np.ascontiguousarray(meas, np.float32)
        spos = self.spos if spos is None else np.ascontiguousarray(spos, np.float32)
        svel = self.svel if svel is None else np.ascontiguousarray(svel, np.float32)
        a = self.acc.copy() if self.p.system != PERISTALSIS else self.vforce.copy()
        b = self.pforce.copy()
        lib().orc_force(ctypes.byref(self.p), fp(spos), fp(svel), fp(meas), up(self.idx),
                        up(self.cell_start), up(self.cell_end), fp(a), fp(b), self.n, threads)
        sa = np.zeros((self.n, 4), np.float32)
        sb = np.zeros((self.n, 4), np.float32)
        lib().orc_force_scale(ctypes.byref(self.p), fp(spos), fp(svel), fp(meas), up(self.idx),
                              up(self.cell_start), up(self.cell_end), fp(sa), fp(sb), self.n, threads)
        return a, b, sa, sb

    def density_at(self, i):
        return float(lib().orc_density_at(ctypes.byref(self.p), fp(self.spos),
                                          up(self.cell_start), up(self.cell_end), int(i)))


# ---------------------------------------------------------------------------
# the reference's own kernels, compiled for the CPU
# ---------------------------------------------------------------------------

_REF_PREFIX = {DAMBREAK: ("dambreak", "db"), POISEUILLE: ("poiseuille", "pf"),
               PERISTALSIS: ("peristalsis", "ps")}


def ref_available():
    return all(os.path.exists(os.path.join(REF_DIR, "libref_%s.so" % v[0]))
               for v in _REF_PREFIX.values())


def ref_lib(system):
    if system not in _ref:
        name, _ = _REF_PREFIX[system]
        path = os.path.join(REF_DIR, "libref_%s.so" % name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        _ref[system] = ctypes.CDLL(path)
    return _ref[system]


_libm = ctypes.CDLL("libm.so.6")
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]
_libm.powf.restype = ctypes.c_float
F32 = np.float32


class RefState(_StateBase):
    """One solver advanced by the reference's kernels on the CPU.  The host-side
    stage order (and Peristalsis phase logic) restates the reference update()
    functions, whose sources cannot be compiled here (OpenGL/cutil headers)."""

    def _call(self, fn, *args):
        L = ref_lib(self.p.system)
        tag = _REF_PREFIX[self.p.system][1]
        return getattr(L, "ref_%s_%s" % (tag, fn))(*args)

    def step(self, stop_after=STAGE_INTEGRATE, threads=1):
        p = self.p
        n = ctypes.c_uint(self.n)
        dt = F32(p.delta_time)
        sys = p.system
        if sys == PERISTALSIS and p.is_boundary_configuration:  # PeristalsisSystem.cpp:330-343
            self.phase[1] = F32(self.phase[1] + dt)
            if self.phase[3] < F32(p.amplitude):
                self._call("set_params", ctypes.byref(p))
                self._call("configure_boundary", fp(self.pos), ctypes.c_float(self.phase[3]), n)
                self.phase[3] = F32(self.phase[3] + F32(dt * F32(_libm.powf(10.0, -3.0))))
            else:
                self.phase[2] = F32(self.phase[2] - dt)
                if self.phase[2] < 0:
                    p.is_boundary_configuration = 0
        self._call("set_params", ctypes.byref(p))
        self._call("calc_hash", fp(self.pos), up(self.hash), up(self.idx), n)
        if stop_after == 0:
            return self
        self._call("sort", up(self.hash), up(self.idx), n)
        if stop_after == 1:
            return self
        self._call("reorder", up(self.cell_start), up(self.cell_end), fp(self.spos), fp(self.svel),
                   up(self.hash), up(self.idx), fp(self.pos), fp(self.vlf), n,
                   ctypes.c_uint(self.ncells))
        if stop_after == 2:
            return self
        self._call("density", fp(self.meas), fp(self.spos), fp(self.svel), up(self.idx),
                   up(self.cell_start), up(self.cell_end), n)
        if stop_after == 3:
            return self
        t = F32(0.0)
        if sys == PERISTALSIS and not p.is_boundary_configuration:
            t = F32(self.phase[0] - self.phase[1])
        if sys == PERISTALSIS:
            self._call("force", fp(self.vforce), fp(self.pforce), fp(self.meas), fp(self.spos),
                       fp(self.svel), up(self.idx), up(self.cell_start), up(self.cell_end), n,
                       ctypes.c_float(t))
        else:
            self._call("force", fp(self.acc), fp(self.meas), fp(self.spos), fp(self.svel),
                       up(self.idx), up(self.cell_start), up(self.cell_end), n)
        if stop_after == 4:
            return self
        if sys == PERISTALSIS:
            self._call("integrate", fp(self.pos), fp(self.vel), fp(self.vlf), fp(self.vforce),
                       fp(self.pforce), ctypes.c_float(t), n)
        else:
            self._call("integrate", fp(self.pos), fp(self.vel), fp(self.vlf), fp(self.acc), n)
        self.phase[0] = F32(self.phase[0] + dt)
        return self

    def remove_right_boundary(self):
        self.p.right_boundary = F32(float(0xFFFFFFFF))
        self._call("set_params", ctypes.byref(self.p))
        self._call("remove_right_boundary", fp(self.pos), ctypes.c_uint(self.n))
        self.phase[0] = 0

    def shift_right_boundary(self):
        self._call("set_params", ctypes.byref(self.p))
        self._call("shift_right_boundary", fp(self.pos), ctypes.c_uint(self.n))
