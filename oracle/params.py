"""The parameter block of include/cmag_sph.h (struct cmag_sph_params) and the
constants the oracle needs, mirrored for ctypes.

TEST INFRASTRUCTURE ONLY: the oracle's own copy, so that the oracle, the tests'
checkers and the CPU reference arm of bench.py never import the product package.
tests/test_oracle_golden.py checks that it matches the product's mirror field
for field."""
import ctypes

DAMBREAK, POISEUILLE, PERISTALSIS = 0, 1, 2
KERNEL_WENDLAND, KERNEL_CUBIC_SPLINE = 0, 1
EOS_REFERENCE, EOS_TAIT = 0, 1
STAGE_HASH, STAGE_SORT, STAGE_REORDER, STAGE_DENSITY, STAGE_FORCE, STAGE_INTEGRATE = range(6)

u32x3 = ctypes.c_uint32 * 3
f32x3 = ctypes.c_float * 3


class SphParams(ctypes.Structure):
    """struct cmag_sph_params (include/cmag_sph.h)."""

    _fields_ = [
        ("system", ctypes.c_int32),
        ("grid_size", u32x3),
        ("world_origin", f32x3),
        ("cell_size", f32x3),
        ("fluid_size", u32x3),
        ("cell_count", ctypes.c_int32),
        ("world_size", f32x3),
        ("gravity", f32x3),
        ("particle_radius", ctypes.c_float),
        ("smoothing_radius", ctypes.c_float),
        ("particle_mass", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("soundspeed", ctypes.c_float),
        ("B", ctypes.c_float),
        ("gamma", ctypes.c_float),
        ("delta_time", ctypes.c_float),
        ("boundary_damping", ctypes.c_float),
        ("mu", ctypes.c_float),
        ("boundary_offset", ctypes.c_int32),
        ("right_boundary", ctypes.c_float),
        ("lj_D", ctypes.c_float),
        ("lj_a", ctypes.c_float),
        ("amplitude", ctypes.c_float),
        ("wave_speed", ctypes.c_float),
        ("wave_count", ctypes.c_float),
        ("is_boundary_configuration", ctypes.c_int32),
        ("dims", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("eos", ctypes.c_int32),
        ("av_alpha", ctypes.c_float),
        ("lj_cutoff", ctypes.c_int32),
        ("clamp_z", ctypes.c_int32),
        ("z_min_border", ctypes.c_float),
        ("z_max_border", ctypes.c_float),
        ("wall_noslip", ctypes.c_int32),
        ("wall_beta_max", ctypes.c_float),
        ("reserved", ctypes.c_int32 * 3),
    ]

    def copy(self):
        out = SphParams()
        ctypes.memmove(ctypes.byref(out), ctypes.byref(self), ctypes.sizeof(SphParams))
        return out

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "__len__"):
                v = list(v)
            d[name] = v
        return d

    def __eq__(self, other):
        return bytes(self) == bytes(other)

    @property
    def num_grid_cells(self):
        g = self.grid_size
        return int(g[0]) * int(g[1]) * int(g[2])


def u3(v):
    return u32x3(*[int(x) for x in v])


def f3(v):
    return f32x3(*[float(x) for x in v])
