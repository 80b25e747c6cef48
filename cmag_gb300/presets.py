"""Parameter blocks for the reference scenes and for the benchmark workloads.

Reference scenes (exact reference constructors, via the C ABI):
  * dambreak_xfront():   DamBreak.Report/XFrontTest.h:17-23 (128x256 column)
  * poiseuille_dump():   Poiseuille.Report/dump.h:17-27 (16x58 channel)
  * peristalsis_report(): Peristalsis.Report/density.h:14-35 (256x58 channel)

Benchmark workloads (synthetic, seeded):
  * poiseuille_c1():   2-D Poiseuille, 64x64 fluid, 3 wall rows, periodic x
  * dambreak3d():      3-D dam break, 64x128x64 = 524,288 fluid, 3 wall layers
  * peristalsis_c3():  2-D peristaltic channel, 2048x512 = 1,048,576 fluid, 4 waves
  * batched_scenes():  256 independent 2-D scenes (128 Poiseuille, 128 dam breaks),
                       fluid counts log-uniform in [4096, 262144]
"""
import ctypes
import math

import numpy as np

from . import _abi
from ._abi import SphParams, f3, u3
from ._lib import check, lib

F32 = np.float32


def _next_pow2(v):
    p = 1
    while p < v:
        p <<= 1
    return p


def dambreak_params(fluid_size, boundary_offset, grid_size, radius):
    p = SphParams()
    check(lib().cmag_dambreak_default_params(u3(fluid_size), int(boundary_offset), u3(grid_size),
                                             float(radius), ctypes.byref(p)))
    return p


def poiseuille_params(fluid_size, boundary_offset, grid_size, radius):
    p = SphParams()
    check(lib().cmag_poiseuille_default_params(u3(fluid_size), int(boundary_offset), u3(grid_size),
                                               float(radius), ctypes.byref(p)))
    return p


def peristalsis_params(dt, fluid_size, amplitude, wave_speed, soundspeed, gravity,
                       boundary_offset, grid_size, radius):
    p = SphParams()
    check(lib().cmag_peristalsis_default_params(float(dt), u3(fluid_size), float(amplitude),
                                                float(wave_speed), float(soundspeed), f3(gravity),
                                                int(boundary_offset), u3(grid_size), float(radius),
                                                ctypes.byref(p)))
    return p


def reference_count(p):
    n = ctypes.c_uint32()
    check(lib().cmag_reference_particle_count(ctypes.byref(_abi.as_params(p)), ctypes.byref(n)))
    return n.value


# ---- reference report scenes -------------------------------------------------

def dambreak_xfront(num=128):
    """XFrontTest/YFrontTest: column num x 2num in a 4num x 2num x 4 grid."""
    return dict(fluid_size=(num, 2 * num, 1), boundary_offset=1, grid_size=(512 * num // 128, 256 * num // 128, 4),
                radius=1.0 / (2 * num))


def poiseuille_dump(grid_x=16, grid_y=64, boundary_offset=3):
    """Poiseuille.Report/dump.h: channel 1 mm wide with grid_y - 2*offset fluid rows."""
    fy = grid_y - 2 * boundary_offset
    return dict(fluid_size=(grid_x, fy, 1), boundary_offset=boundary_offset,
                grid_size=(grid_x, grid_y, 4), radius=1.0 / (2 * fy * 1000))


def peristalsis_report():
    """Peristalsis.Report/density.h, forces.h, velocityfield.h."""
    off = 3
    r = 1.0 / (2 * (64 - 6) * 1000)
    c = 1e-4
    return dict(dt=1e-4, fluid_size=(256, 64 - 2 * off, 1), amplitude=0.6 * 35 * r,
                wave_speed=100 * c, soundspeed=c, gravity=(0.0, 0.0, 0.0), boundary_offset=off,
                grid_size=(256, 128, 4), radius=r)


# ---- benchmark workloads -------------------------------------------------------

def poiseuille_c1(reference_physics=True):
    """2-D Poiseuille: 64x64 fluid at dx = 1/64 of a 1 mm channel, 3 wall rows top and
    bottom, periodic x, body force 1e-4 (4,096 + 384 particles).  With
    reference_physics=False: cubic spline, h = 1.3 dx, Tait gamma 7 with
    c0 = 10 u_max (u_max = F l^2 / (8 nu)), mass from the lattice kernel sum."""
    off = 3
    fx, fy = 64, 64
    r = 1.0 / (2 * fy * 1000)
    p = poiseuille_params((fx, fy, 1), off, (64, _next_pow2(fy + 2 * off), 4), r)
    if not reference_physics:
        dx = 2 * r
        nu = 1e-6
        umax = 1e-4 * (1e-3) ** 2 / (8 * nu)
        c0 = 10 * umax
        p.kernel = _abi.KERNEL_CUBIC_SPLINE
        p.smoothing_radius = F32(1.3 * dx)
        p.cell_count = int(math.ceil(2 * 1.3))
        p.eos = _abi.EOS_TAIT
        p.gamma = 7.0
        p.soundspeed = F32(c0)
        p.B = F32(c0 * c0 * 1000.0 / 7.0)
        p.particle_mass = F32(1000.0 * dx * dx)
    return p


def dambreak3d(fluid=(64, 128, 64), tank=(256, 192, 64), layers=3, h_over_dx=1.3, alpha=0.01,
               kernel=_abi.KERNEL_WENDLAND, dt=5e-5, column_width=0.5):
    """3-D dam break (extension of the reference's 2-D DamBreak): water column
    fluid = 64x128x64 lattice (0.5 x 1.0 x 0.5 m at dx = 1/128) in a 2.0 x 1.5 x 0.5 m
    tank of `tank` cells, `layers` wall layers on the floor and four sides, gravity
    -9.81, Tait gamma 7 with c0 = 10 sqrt(2 g H), h = 1.3 dx, Monaghan alpha 0.01,
    Lennard-Jones walls cut off at 2h, clamps on all tank faces.
    Returns (params, particle count, tank, layers)."""
    dx = column_width / fluid[0]
    r = dx / 2
    L = int(layers)
    # a tight grid around the tank (+1 cell each side, a quarter tank height of
    # headroom); sizes need not be powers of two (cells wrap by residue)
    gx = tank[0] + 2 * L + 2
    gy = tank[1] + L + 2 + tank[1] // 4
    gz = tank[2] + 2 * L + 2
    p = dambreak_params(fluid, L + 1, (gx, gy, gz), r)
    o = -(L + 1) * dx
    p.world_origin[0] = p.world_origin[1] = p.world_origin[2] = F32(o)
    p.world_size[0], p.world_size[1], p.world_size[2] = gx * dx, gy * dx, gz * dx
    H = fluid[1] * dx
    g = 9.81
    c0 = 10.0 * math.sqrt(2.0 * g * H)
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, -g, 0.0
    p.dims = 3
    p.kernel = kernel
    p.smoothing_radius = F32(h_over_dx * dx)
    p.cell_count = int(math.ceil(2 * h_over_dx - 1e-9))
    p.particle_mass = F32(1000.0 * dx ** 3)
    p.soundspeed = F32(c0)
    p.gamma = 7.0
    p.B = F32(c0 * c0 * 1000.0 / 7.0)
    p.lj_D = F32(10.0 * -g * H)
    p.lj_a = F32(r)
    p.lj_cutoff = 1
    p.av_alpha = F32(alpha)
    p.right_boundary = F32(tank[0] * dx)
    p.clamp_z = 1
    p.z_min_border = 0.0
    p.z_max_border = F32(tank[2] * dx)
    p.delta_time = F32(dt)
    n = ctypes.c_uint32()
    check(lib().cmag_dambreak3d_particle_count(u3(fluid), u3(tank), L, ctypes.byref(n)))
    return p, n.value, tuple(tank), L


def peristalsis_c3(fluid=(2048, 512), amplitude_frac=0.3, waves=4, reynolds=10.0,
                   channel_width=1e-3):
    """2-D peristaltic channel: fluid[0] x fluid[1] lattice filling a channel of
    half-width R = fluid[1]/2 dx and length 4 wavelengths (lambda = 2R), walls
    y = +-R(1 - 0.3 sin(2 pi (x - c t)/lambda)) (the reference's wall law, a half
    period from +-R(1 + 0.3 sin)), Re = c R / nu = 10 with nu = 1e-6."""
    off = 3
    fx, fy = fluid
    dx = channel_width / fy
    r = dx / 2
    R = channel_width / 2
    nu = 1e-6
    c = reynolds * nu / R
    soundspeed = (10 * c) ** 2 / 50.0  # p = 50 c_s rho: effective c^2 = 50 c_s
    gx = _next_pow2(fx)
    gy = _next_pow2(int(fy * (1 + 2 * amplitude_frac)) + 2 * off + 8)
    h = 3 * r
    dt = min(0.125 * h * h / nu, 0.25 * h / (10 * c))
    p = peristalsis_params(dt, (fx, fy, 1), amplitude_frac * R, c, soundspeed, (0.0, 0.0, 0.0),
                           off, (gx, gy, 4), r)
    p.wave_count = float(waves)
    return p


def batched_scenes(scenes=256, seed=1973, lo=4096, hi=262144, nu_lo=1e-6, nu_hi=1e-4):
    """Batch of independent 2-D scenes: the first half Poiseuille channels, the
    second half dam breaks.  Fluid particle counts are drawn log-uniform in
    [lo, hi] and the kinematic viscosity of each channel log-uniform in
    [nu_lo, nu_hi] from `seed`.

    Poiseuille (the reference channel, Poiseuille.Report/dump.h): fy rows across a
    1 mm channel (fy = sqrt(count)), fx = count / fy columns along the periodic x
    axis, 3 wall rows each side, grid (fx, fy + 12, 4); the reference particle mass
    scaled with the particle area, (58 / fy)^2, for the reference's rest density;
    mu = 1000 nu and the body
    force 1e-4 nu / 1e-6, so every channel has the reference's u_max = F l^2 / (8 nu)
    = 1.25e-5 m/s; dt = min(1e-4, 0.125 h^2 / nu).
    Dam break (the reference column, DamBreak.Report/XFrontTest.h:17-23): a num x
    2num column (num = sqrt(count / 2)) in a 4num x 2num x 4 grid at radius
    1/(2 num), gravity -9.8, reference walls, artificial viscosity coefficient
    0.38 sqrt(nu / 1e-5) from the drawn nu (gravity stays: every column is 1 x 2 m,
    so scaling g would only rescale time).  The
    reference's particle mass and dt (1e-4) belong to its num = 128 column
    (fluidSystem.cpp:17-77); here the mass scales with the particle area,
    (128 / num)^2, so every column has the reference's rest density, and dt with
    the spacing at half the reference's CFL number, 1e-4 * 64 / num: the columns
    are released at t = 0 without the reference's 1.5 s of settling.

    Returns (params list, particle counts, fluid counts, per-scene description)."""
    rng = np.random.default_rng(seed)
    half = scenes // 2
    out_p, out_n, out_f, desc = [], [], [], []
    for k in range(scenes):
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        nu = float(np.exp(rng.uniform(np.log(nu_lo), np.log(nu_hi))))
        if k < half:
            off = 3
            fy = max(16, int(round(math.sqrt(target))))
            fx = max(16, int(round(target / fy)))
            r = 1.0 / (2 * fy * 1000)
            p = poiseuille_params((fx, fy, 1), off, (fx, fy + 2 * off + 6, 4), r)
            # the reference's particle mass belongs to its 58-row channel
            # (poiseuilleFlowSystem.cpp:48-49); it scales with the particle area
            # so every channel has the reference's rest density
            p.particle_mass = F32(float(p.particle_mass) * (58.0 / fy) ** 2)
            p.mu = F32(1000.0 * nu)
            p.gravity[0] = F32(1e-4 * nu / 1e-6)
            h = float(p.smoothing_radius)
            p.delta_time = F32(min(1e-4, 0.125 * h * h / nu))
            fluid = fx * fy
            desc.append(("poiseuille", fx, fy, nu))
        else:
            num = max(16, int(round(math.sqrt(target / 2))))
            p = dambreak_params((num, 2 * num, 1), 1, (4 * num, 2 * num, 4), 1.0 / (2 * num))
            p.particle_mass = F32(float(p.particle_mass) * (128.0 / num) ** 2)
            p.delta_time = F32(1e-4 * 64 / num)
            # Monaghan's artificial viscosity is the dam break's only viscosity: its
            # coefficient follows the drawn nu, log-uniform over [0.12, 1.2] around
            # the reference's 0.38 (fluid_kernel.cu:229-233) at nu = 1e-5
            p.av_alpha = F32(0.38 * math.sqrt(nu / 1e-5))
            fluid = 2 * num * num
            desc.append(("dambreak", num, 2 * num, nu))
        out_p.append(p)
        out_n.append(reference_count(p))
        out_f.append(fluid)
    return out_p, out_n, out_f, desc
