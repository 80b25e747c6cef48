// host_scenes.cpp -- parameter blocks and scenes of the reference constructors
// and reset() functions, plus the 3-D dam-break scene.
//
// Compiled with -ffp-contract=off: every float operation is rounded separately
// and in the order of the reference expression, so positions and parameters are
// the reference's bit for bit on any host.
#include <cmath>
#include <cstring>

#include "host_scenes.h"

namespace cmag {

namespace {

void set_defaults(cmag_sph_params &p)
{
    std::memset(&p, 0, sizeof(p));
    p.dims = 2;
    p.kernel = CMAG_KERNEL_WENDLAND;
    p.eos = CMAG_EOS_REFERENCE;
    p.av_alpha = 0.38f;   // hard-coded in fluid_kernel.cu:229
    p.lj_cutoff = 0;
    p.wave_count = 1.0f;
    p.gamma = 7.0f;
}

// the geometry every reference constructor derives the same way
void set_grid(cmag_sph_params &p, const uint32_t fs[3], const uint32_t gs[3], float r)
{
    for (int k = 0; k < 3; ++k) {
        p.fluid_size[k] = fs[k];
        p.grid_size[k] = gs[k];
    }
    p.particle_radius = r;
    p.smoothing_radius = 3.0f * r;
    p.rest_density = 1000.0f;
    p.cell_count = 3;
    // worldOrigin = -(getHalfWorld{X,Y,Z}Size() = gridSize * radius)
    p.world_origin[0] = -(gs[0] * r);
    p.world_origin[1] = -(gs[1] * r);
    p.world_origin[2] = -(gs[2] * r);
    const float cell = r * 2.0f;
    p.cell_size[0] = p.cell_size[1] = p.cell_size[2] = cell;
    for (int k = 0; k < 3; ++k) p.world_size[k] = gs[k] * 2.0f * r;
    p.boundary_damping = -1.0f;
}

inline void put(float *pos, uint32_t i, uint32_t n, float x, float y, float z, float w)
{
    if (i >= n) return;
    float *q = pos + 4 * (size_t)i;
    q[0] = x; q[1] = y; q[2] = z; q[3] = w;
}

}  // namespace

// DamBreakSystem::DamBreakSystem, DamBreak.Core/fluidSystem.cpp:17-77
void dambreak_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                     cmag_sph_params &p)
{
    set_defaults(p);
    p.system = CMAG_DAMBREAK;
    set_grid(p, fs, gs, r);
    p.boundary_offset = off;
    p.particle_mass = (float)(p.rest_density / 16327.6);
    const uint32_t gate_cells = (uint32_t)(off + (int32_t)fs[0]) * 2u;
    p.right_boundary = p.world_origin[0] + gate_cells * r;
    p.gravity[1] = -9.8f;
    const float column = 2 * r * fs[1];
    p.B = 200 * p.rest_density * std::fabs(p.gravity[1]) * column / p.gamma;
    p.lj_D = 10 * p.gravity[1] * 2 * r * fs[1];
    p.lj_a = 1 * r;
    p.soundspeed = std::sqrt(p.B * p.gamma / p.rest_density);
    p.delta_time = std::pow(10.0f, -4.0f);
}

// PoiseuilleFlowSystem::PoiseuilleFlowSystem, Poiseuille.Core/poiseuilleFlowSystem.cpp:21-67
void poiseuille_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                       cmag_sph_params &p)
{
    set_defaults(p);
    p.system = CMAG_POISEUILLE;
    set_grid(p, fs, gs, r);
    p.boundary_offset = off;
    p.particle_mass = (float)(1000.0f / 3381320880.551724);
    p.gravity[0] = std::pow(10.0f, -4.0f);
    p.soundspeed = std::pow(10.0f, -4.0f);
    p.mu = std::pow(10.0f, -3.0f);
    p.delta_time = std::pow(10.0f, -4.0f);
}

// PeristalsisSystem::PeristalsisSystem, Peristalsis.Core/PeristalsisSystem.cpp:17-80
void peristalsis_params(float dt, const uint32_t fs[3], float amplitude, float wave_speed,
                        float soundspeed, const float g[3], int32_t off, const uint32_t gs[3],
                        float r, cmag_sph_params &p)
{
    set_defaults(p);
    p.system = CMAG_PERISTALSIS;
    set_grid(p, fs, gs, r);
    p.boundary_offset = off;
    p.amplitude = amplitude;
    p.wave_speed = wave_speed;
    p.particle_mass = 0.0f;  // Reset() derives it from the lattice
    for (int k = 0; k < 3; ++k) p.gravity[k] = g[k];
    p.soundspeed = soundspeed;
    p.mu = std::pow(10.0f, -3.0f);
    p.delta_time = dt;
    p.is_boundary_configuration = 1;
}

uint32_t reference_particle_count(const cmag_sph_params &p)
{
    const uint32_t fluid = p.fluid_size[0] * p.fluid_size[1] * p.fluid_size[2];
    const uint32_t off = (uint32_t)p.boundary_offset;
    if (p.system == CMAG_DAMBREAK)  // fluidSystem.cpp:34-37
        return fluid + p.grid_size[0] * off + 2u * (p.grid_size[1] - off) * off;
    return fluid + 2u * p.grid_size[0] * off;
}

// DamBreakSystem::initFluid + initBoundaryParticles (fluidSystem.cpp:382-523)
static void dambreak_scene(const cmag_sph_params &p, float *pos, uint32_t n)
{
    const float r = p.particle_radius, s = r * 2.0f;
    const float hx = p.grid_size[0] * r, hy = p.grid_size[1] * r, hz = p.grid_size[2] * r;
    const int off = p.boundary_offset;
    const uint32_t fx = p.fluid_size[0], fy = p.fluid_size[1], fz = p.fluid_size[2];
    const uint32_t gx = p.grid_size[0], gy = p.grid_size[1];
    const float ox = p.world_origin[0], oy = p.world_origin[1], oz = p.world_origin[2];
    for (uint32_t z = 0; z < fz; ++z)
        for (uint32_t y = 0; y < fy; ++y)
            for (uint32_t x = 0; x < fx; ++x)
                put(pos, z * fy * fx + y * fx + x, n, s * x + r - hx + off * 2 * r,
                    s * y + r - hy + off * 2 * r, s * z + r - hz, (float)CMAG_FLUID);
    if (off <= 0) return;
    const float lo = (off - 1) * 2 * r;  // one layer inside the outer wall
    const float z0 = s * 0u + r + oz;
    uint32_t base = fx * fy * fz;
    const uint32_t bottom = gx - (uint32_t)(off - 1), side = gy - (uint32_t)off;
    for (uint32_t x = 0; x < bottom; ++x)  // bottom row, FirstType
        put(pos, base + x, n, s * x + r + ox + lo, s * 0u + r + oy + lo, z0, (float)CMAG_FIRST_TYPE);
    base += bottom;
    for (uint32_t y = 0; y < side; ++y)  // left column, FirstType
        put(pos, base + y, n, s * 0u + r + ox + lo, s * y + r + oy + (off + 0) * 2 * r, z0,
            (float)CMAG_FIRST_TYPE);
    base += side;
    const float gate = (fx + (uint32_t)off) * 2 * r;
    for (uint32_t y = 0; y < side; ++y)  // right gate column, RightFirstType
        put(pos, base + y, n, s * 0u + r + ox + gate, s * y + r + oy + off * 2 * r, z0,
            (float)CMAG_RIGHT_FIRST_TYPE);
    base += side;
    const uint32_t outer = (uint32_t)(off - 1);
    for (uint32_t y = 0; y < outer; ++y)  // outer bottom rows, SecondType
        for (uint32_t x = 0; x < gx; ++x)
            put(pos, base + y * gx + x, n, s * x + r + ox, s * y + r + oy, z0, (float)CMAG_SECOND_TYPE);
    base += gx * outer;
    const uint32_t lrows = gy - (uint32_t)(off - 1);
    for (uint32_t y = 0; y < lrows; ++y)  // outer left columns, SecondType
        for (uint32_t x = 0; x < outer; ++x)
            put(pos, base + y * outer + x, n, s * x + r + ox, s * y + r + oy + lo, z0,
                (float)CMAG_SECOND_TYPE);
    base += outer * lrows;
    const float gate2 = (fx + (uint32_t)off + 1u) * 2 * r;
    for (uint32_t y = 0; y < side; ++y)  // outer gate columns, RightSecondType
        for (uint32_t x = 0; x < outer; ++x)
            put(pos, base + y * outer + x, n, s * x + r + ox + gate2, s * y + r + oy + off * 2 * r,
                z0, (float)CMAG_RIGHT_SECOND_TYPE);
}

// PoiseuilleFlowSystem::initFluid + initBoundaryParticles (poiseuilleFlowSystem.cpp:325-383)
static void poiseuille_scene(const cmag_sph_params &p, float *pos, uint32_t n)
{
    const float r = p.particle_radius, s = r * 2.0f;
    const float hx = p.grid_size[0] * r, hy = p.grid_size[1] * r, hz = p.grid_size[2] * r;
    const int off = p.boundary_offset;
    const uint32_t fx = p.fluid_size[0], fy = p.fluid_size[1], fz = p.fluid_size[2];
    const uint32_t gx = p.grid_size[0];
    const float ox = p.world_origin[0], oy = p.world_origin[1], oz = p.world_origin[2];
    for (uint32_t z = 0; z < fz; ++z)
        for (uint32_t y = 0; y < fy; ++y)
            for (uint32_t x = 0; x < fx; ++x)
                put(pos, z * fy * fx + y * fx + x, n, s * x + r - hx, s * y + r - hy + off * 2 * r,
                    s * z + r - hz, 0.0f);
    uint32_t base = fx * fy * fz;
    const uint32_t rows = (uint32_t)off;
    const float z0 = s * 0u + r + oz;
    for (uint32_t y = 0; y < rows; ++y)  // bottom wall
        for (uint32_t x = 0; x < gx; ++x)
            put(pos, base + y * gx + x, n, s * x + r + ox, s * y + r + oy, z0, 1.0f);
    base += gx * rows;
    for (uint32_t y = 0; y < rows; ++y)  // top wall
        for (uint32_t x = 0; x < gx; ++x)
            put(pos, base + y * gx + x, n, s * x + r + ox,
                s * y + r + oy + off * 2 * r + fy * 2.0f * r, z0, 1.0f);
}

// PeristalsisSystem::initFluid + initBoundaryParticles (PeristalsisSystem.cpp:255-317)
static void peristalsis_scene(const cmag_sph_params &p, float *pos, uint32_t n)
{
    const float r = p.particle_radius, s = r * 2.0f;
    const float hx = p.grid_size[0] * r, hz = p.grid_size[2] * r;
    const int fx = (int)p.fluid_size[0], fy = (int)p.fluid_size[1], fz = (int)p.fluid_size[2];
    const float ox = p.world_origin[0], oz = p.world_origin[2];
    const uint32_t ufy = p.fluid_size[1];
    for (int z = 0; z < fz; ++z)
        for (int y = 0; y < fy; ++y)
            for (int x = 0; x < fx; ++x)
                put(pos, (uint32_t)(z * fy * fx + y * fx + x), n, s * x + r - hx,
                    -1.0f * ufy * r + s * y + r, s * z + r - hz, 0.0f);
    uint32_t base = p.fluid_size[0] * p.fluid_size[1] * p.fluid_size[2];
    const uint32_t cols = p.fluid_size[0], rows = (uint32_t)p.boundary_offset;
    const float z0 = s * 0u + r + oz;
    for (uint32_t y = 0; y < rows; ++y)  // bottom layers, type 2,4,6
        for (uint32_t x = 0; x < cols; ++x)
            put(pos, base + y * cols + x, n, r * (2 * x + 1) + ox, -1.0f * ufy * r - s * y - r, z0,
                2.0f * (1.0f + y));
    base += cols * rows;
    for (uint32_t y = 0; y < rows; ++y)  // top layers, type -2,-4,-6
        for (uint32_t x = 0; x < cols; ++x)
            put(pos, base + y * cols + x, n, r * (2 * x + 1) + ox, ufy * r + s * y + r, z0,
                -2.0f * (1.0f + y));
}

void reference_scene(const cmag_sph_params &p, float *pos, uint32_t n)
{
    std::memset(pos, 0, sizeof(float) * 4 * (size_t)n);
    if (p.system == CMAG_DAMBREAK) dambreak_scene(p, pos, n);
    else if (p.system == CMAG_POISEUILLE) poiseuille_scene(p, pos, n);
    else peristalsis_scene(p, pos, n);
}

// PeristalsisSystem::CalculateMass (PeristalsisSystem.cpp:238-253): kernel sum at
// particle gridSize.x / 2 over all particles, in 2-D
float peristalsis_mass_sum(const cmag_sph_params &p, const float *pos, uint32_t n)
{
    const uint32_t probe = p.grid_size[0] / 2;
    const float tx = pos[probe * 4], ty = pos[probe * 4 + 1];
    const float h = p.smoothing_radius;
    const float coeff = 7.0f / 4 / 3.141592654f / std::pow(h, 2.0f);
    float sum = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const float dx = tx - pos[4 * (size_t)i], dy = ty - pos[4 * (size_t)i + 1];
        const float q = std::sqrt(dx * dx + dy * dy) / h;
        if (q < 2) sum += coeff * (std::pow(1 - 0.5f * q, 4.0f) * (2 * q + 1));
    }
    return sum;
}

// ---------------------------------------------------------------- 3-D scene --

uint32_t dambreak3d_count(const uint32_t fs[3], const uint32_t tank[3], uint32_t L)
{
    const uint64_t box = (uint64_t)(tank[0] + 2 * L) * (tank[1] + L) * (tank[2] + 2 * L);
    const uint64_t inner = (uint64_t)tank[0] * tank[1] * tank[2];
    return (uint32_t)((uint64_t)fs[0] * fs[1] * fs[2] + box - inner);
}

namespace {
uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
// uniform in [-1, 1) from 24 hash bits of (seed, particle, axis)
float jitter(uint64_t seed, uint64_t i, int axis)
{
    const uint64_t r = mix64(seed * 0x100000001B3ull + i * 3u + (uint64_t)axis);
    return (float)(int32_t)((uint32_t)(r >> 40) - (1u << 23)) * (1.0f / 8388608.0f);
}
}  // namespace

// Fluid block on tank cells [0,fx)x[0,fy)x[0,fz) (cell k centred at (k + 0.5) dx)
// with +-jitter_frac*dx seeded jitter, then L wall layers on the floor and the four
// sides (open top), each wall particle at a cell centre.
void dambreak3d_scene(const cmag_sph_params &p, const uint32_t tank[3], uint32_t L,
                      float jitter_frac, uint64_t seed, float *pos, uint32_t n)
{
    const float dx = p.particle_radius * 2.0f;
    const float amp = jitter_frac * dx;
    const uint32_t *fs = p.fluid_size;
    uint32_t i = 0;
    for (uint32_t z = 0; z < fs[2]; ++z)
        for (uint32_t y = 0; y < fs[1]; ++y)
            for (uint32_t x = 0; x < fs[0]; ++x, ++i)
                put(pos, i, n, ((float)x + 0.5f) * dx + amp * jitter(seed, i, 0),
                    ((float)y + 0.5f) * dx + amp * jitter(seed, i, 1),
                    ((float)z + 0.5f) * dx + amp * jitter(seed, i, 2), (float)CMAG_FLUID);
    const int l = (int)L, tx = (int)tank[0], ty = (int)tank[1], tz = (int)tank[2];
    for (int z = -l; z < tz + l; ++z)
        for (int y = -l; y < ty; ++y)
            for (int x = -l; x < tx + l; ++x) {
                if (x >= 0 && x < tx && y >= 0 && z >= 0 && z < tz) continue;
                put(pos, i++, n, ((float)x + 0.5f) * dx, ((float)y + 0.5f) * dx,
                    ((float)z + 0.5f) * dx, (float)CMAG_FIRST_TYPE);
            }
}

}  // namespace cmag
