"""The benchmark workloads' parameter blocks and scenes, derived on the oracle.

TEST INFRASTRUCTURE ONLY: what bench.py's CPU arms (the cpu_baseline leg and
--impl reference) and the tests use to build a workload without the product
library.  Each function restates the matching one of cmag_gb300/presets.py on
the oracle's own parameter derivation (the reference constructors restated in
oracle/cmag_oracle.c: DamBreak.Core/fluidSystem.cpp:17-77,
Poiseuille.Core/poiseuilleFlowSystem.cpp:21-67, PeristalsisSystem.cpp:17-80);
tests/test_oracle_golden.py checks that both give the same bytes.
"""
import math

import numpy as np

from . import oracle as O
from .params import EOS_TAIT, KERNEL_CUBIC_SPLINE, KERNEL_WENDLAND

F32 = np.float32


def _next_pow2(v):
    p = 1
    while p < v:
        p <<= 1
    return p


def poiseuille_c1(reference_physics=True):
    """2-D Poiseuille, 64x64 fluid at dx = 1/64 of a 1 mm channel, 3 wall rows each
    side, periodic x; reference_physics=False: cubic spline, h = 1.3 dx, Tait
    gamma 7 with c0 = 10 u_max, mass rho0 dx^2."""
    off = 3
    fx, fy = 64, 64
    r = 1.0 / (2 * fy * 1000)
    p = O.poiseuille_params((fx, fy, 1), off, (64, _next_pow2(fy + 2 * off), 4), r)
    if not reference_physics:
        dx = 2 * r
        nu = 1e-6
        umax = 1e-4 * (1e-3) ** 2 / (8 * nu)
        c0 = 10 * umax
        p.kernel = KERNEL_CUBIC_SPLINE
        p.smoothing_radius = F32(1.3 * dx)
        p.cell_count = int(math.ceil(2 * 1.3))
        p.eos = EOS_TAIT
        p.gamma = 7.0
        p.soundspeed = F32(c0)
        p.B = F32(c0 * c0 * 1000.0 / 7.0)
        p.particle_mass = F32(1000.0 * dx * dx)
    return p


def dambreak3d(fluid=(64, 128, 64), tank=(256, 192, 64), layers=3, h_over_dx=1.3, alpha=0.01,
               kernel=KERNEL_WENDLAND, dt=5e-5, column_width=0.5):
    """3-D dam break: 64x128x64 column (0.5 x 1.0 x 0.5 m) in a 2.0 x 1.5 x 0.5 m tank
    with 3 wall layers, Tait gamma 7, c0 = 10 sqrt(2 g H), h = 1.3 dx, alpha 0.01,
    wall force cut off at 2h, tight grid.  Returns (params, particles, tank, layers)."""
    dx = column_width / fluid[0]
    r = dx / 2
    L = int(layers)
    gx = tank[0] + 2 * L + 2
    gy = tank[1] + L + 2 + tank[1] // 4
    gz = tank[2] + 2 * L + 2
    p = O.dambreak_params(fluid, L + 1, (gx, gy, gz), r)
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
    return p, O.dambreak3d_count(fluid, tank, L), tuple(tank), L


def peristalsis_c3(fluid=(2048, 512), amplitude_frac=0.3, waves=4, reynolds=10.0, channel_width=1e-3):
    """2-D peristaltic channel: 2048x512 fluid, 4 wavelengths (lambda = 2R), wall
    amplitude 0.3 R, Re = c R / nu = 10 with nu = 1e-6."""
    off = 3
    fx, fy = fluid
    dx = channel_width / fy
    r = dx / 2
    R = channel_width / 2
    nu = 1e-6
    c = reynolds * nu / R
    soundspeed = (10 * c) ** 2 / 50.0
    gx = _next_pow2(fx)
    gy = _next_pow2(int(fy * (1 + 2 * amplitude_frac)) + 2 * off + 8)
    h = 3 * r
    dt = min(0.125 * h * h / nu, 0.25 * h / (10 * c))
    p = O.peristalsis_params(dt, (fx, fy, 1), amplitude_frac * R, c, soundspeed, (0.0, 0.0, 0.0),
                             off, (gx, gy, 4), r)
    p.wave_count = float(waves)
    return p


def workload(name):
    """(params, particles, fluid particles, initial oracle state) of a bench workload."""
    if name == "dambreak3d":
        p, n, tank, L = dambreak3d()
        st = O.OracleState(p, n)
        st.pos[:] = O.dambreak3d_scene(p, tank, L, 0.01, 1973)
        st.meas[:, 0] = p.rest_density
        return p, n, int(np.prod(p.fluid_size)), st
    if name == "peristalsis":
        p = peristalsis_c3()
    elif name == "poiseuille":
        p = poiseuille_c1(reference_physics=False)
    else:
        raise ValueError("no single-scene workload %r" % name)
    n = O.particle_count(p)
    st = O.OracleState(p, n).reset_reference()
    return p, n, int(p.fluid_size[0]) * int(p.fluid_size[1]), st


def batched_scenes(scenes=256, seed=1973, lo=4096, hi=262144, nu_lo=1e-6, nu_hi=1e-4):
    """The 256-scene batch (cmag_gb300/presets.py batched_scenes): Poiseuille
    channels then dam breaks, fluid counts log-uniform in [lo, hi], viscosity
    log-uniform in [nu_lo, nu_hi], body force / gravity scaled per scene.
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
            p = O.poiseuille_params((fx, fy, 1), off, (fx, fy + 2 * off + 6, 4), r)
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
            p = O.dambreak_params((num, 2 * num, 1), 1, (4 * num, 2 * num, 4), 1.0 / (2 * num))
            p.particle_mass = F32(float(p.particle_mass) * (128.0 / num) ** 2)
            p.delta_time = F32(1e-4 * 64 / num)
            # Monaghan's artificial viscosity is the dam break's only viscosity: its
            # coefficient follows the drawn nu, log-uniform over [0.12, 1.2] around
            # the reference's 0.38 (fluid_kernel.cu:229-233) at nu = 1e-5
            p.av_alpha = F32(0.38 * math.sqrt(nu / 1e-5))
            fluid = 2 * num * num
            desc.append(("dambreak", num, 2 * num, nu))
        out_p.append(p)
        out_n.append(O.particle_count(p))
        out_f.append(fluid)
    return out_p, out_n, out_f, desc
