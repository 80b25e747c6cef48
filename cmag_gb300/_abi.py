"""ctypes mirror of include/cmag_sph.h (types and constants only, no library)."""
import ctypes

CMAG_OK = 0
CMAG_ERR_INVALID = 1
CMAG_ERR_CUDA = 2
CMAG_ERR_NOMEM = 3
CMAG_ERR_DEVICE = 4
CMAG_ERR_STATE = 5

# device-side check bits (enum cmag_device_error)
CMAG_DEVERR_LOOKBACK_TIMEOUT = 1
CMAG_DEVERR_RANGE = 2

DAMBREAK, POISEUILLE, PERISTALSIS = 0, 1, 2
KERNEL_WENDLAND, KERNEL_CUBIC_SPLINE = 0, 1
EOS_REFERENCE, EOS_TAIT = 0, 1

# DamBreak particle types (DamBreak.Core/fluid_kernel.cuh:16-23)
RIGHT_FIRST_TYPE, FIRST_TYPE, RIGHT_SECOND_TYPE, SECOND_TYPE, FLUID = 0, 1, 2, 3, 4

# particle arrays
POSITION = 0
VELOCITY = 1
MEASURES = 2
ACCELERATION = 3
VELOCITYLEAPFROG = 4
VISCOUSFORCE = 5
PRESSUREFORCE = 6
PREDICTEDPOSITION = 7
SORTEDPOSITION = 8
SORTEDVELOCITY = 9
HASH = 16
INDEX = 17
CELLSTART = 18
CELLEND = 19
CELLOFFSET = 20

# stages
STAGE_HASH, STAGE_SORT, STAGE_REORDER, STAGE_DENSITY, STAGE_FORCE, STAGE_INTEGRATE = range(6)
STAGE_NAMES = ("hash", "sort", "reorder", "density", "force", "integrate")

u32x3 = ctypes.c_uint32 * 3
f32x3 = ctypes.c_float * 3


class SphParams(ctypes.Structure):
    """struct cmag_sph_params."""

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


def as_params(p):
    """p as a SphParams: p itself, or a copy of any object with the struct's bytes
    (another ctypes mirror of cmag_sph_params)."""
    if isinstance(p, SphParams):
        return p
    b = bytes(p)
    if len(b) != ctypes.sizeof(SphParams):
        raise TypeError("not a cmag_sph_params block (%d bytes)" % len(b))
    return SphParams.from_buffer_copy(b)


def u3(v):
    return u32x3(*[int(x) for x in v])


def f3(v):
    return f32x3(*[float(x) for x in v])


class BatchGroup(ctypes.Structure):
    """cmag_batch_group: one launch group of a batch."""
    _fields_ = [
        ("system", ctypes.c_int32),
        ("planar", ctypes.c_int32),
        ("trim", ctypes.c_int32),
        ("size_bucket", ctypes.c_uint32),
        ("scenes", ctypes.c_uint32),
        ("particles", ctypes.c_uint32),
        ("density_lanes", ctypes.c_int32),
        ("force_lanes", ctypes.c_int32),
        ("lists", ctypes.c_int32),
    ]
