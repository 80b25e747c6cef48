/*
 * cmag_oracle.c -- CPU restatement of cmag's WCSPH time step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA path; never part of the
 * product).  Every function cites the reference lines it restates.  Floating-
 * point expressions keep the reference's evaluation order and types (float
 * arithmetic, powf/sqrtf), and the file is compiled with -ffp-contract=off so
 * that no multiply-add is fused; the integer stages (hash, sort, cell ranges)
 * are therefore exactly the reference's, and the floating-point stages differ
 * from the reference GPU kernels only by the GPU's own rounding (FMA
 * contraction, powf/rsqrtf accuracy).
 */
#include "cmag_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI_F 3.141592654f /* CUDART_PI_F, PeristalsisKernel.cuh:10-12 */
#define ORC_EMPTY 0xffffffffu

typedef struct { float x, y, z; } f3;
typedef struct { int x, y, z; } i3;

static f3 mk3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static f3 muls3(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }  /* float3 * float */
static f3 smul3(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }  /* float * float3 */
static f3 divs3(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
static float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float len3(f3 v) { return sqrtf(dot3(v, v)); }
/* helper_math.h normalize with the host rsqrtf (1/sqrtf) */
static f3 normalize3(f3 v) { float inv = 1.0f / sqrtf(dot3(v, v)); return muls3(v, inv); }
static f3 ld3(const float *a, uint32_t i) { return mk3(a[4 * (size_t)i], a[4 * (size_t)i + 1], a[4 * (size_t)i + 2]); }

/* float -> int as the GPU's cvt.rzi.s32.f32 (saturating, NaN -> 0) */
static int sat_f2i(float f)
{
    if (f != f) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (-2147483647 - 1);
    return (int)f;
}

static uint32_t umul24(uint32_t a, uint32_t b) { return (a & 0xffffffu) * (b & 0xffffffu); }

/* ------------------------------------------------------------------------ */
/* reference constructors                                                   */
/* ------------------------------------------------------------------------ */

static void common_defaults(cmag_sph_params *p)
{
    memset(p, 0, sizeof(*p));
    p->dims = 2;
    p->kernel = CMAG_KERNEL_WENDLAND;
    p->eos = CMAG_EOS_REFERENCE;
    p->av_alpha = 0.38f;      /* fluid_kernel.cu:229 (hard-coded) */
    p->lj_cutoff = 0;
    p->wave_count = 1.0f;
}

/* DamBreakSystem ctor, DamBreak.Core/fluidSystem.cpp:17-77 */
int orc_dambreak_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                        cmag_sph_params *p)
{
    common_defaults(p);
    p->system = CMAG_DAMBREAK;
    for (int k = 0; k < 3; ++k) { p->fluid_size[k] = fs[k]; p->grid_size[k] = gs[k]; }
    p->boundary_offset = off;
    p->particle_radius = r;
    p->smoothing_radius = 3.0f * r;                       /* :46 */
    p->rest_density = 1000.0f;
    p->particle_mass = (float)(p->rest_density / 16327.6); /* :49 (double division) */
    p->cell_count = 3;
    float hx = gs[0] * r, hy = gs[1] * r, hz = gs[2] * r;  /* getHalfWorld*Size */
    p->world_origin[0] = -hx; p->world_origin[1] = -hy; p->world_origin[2] = -hz;
    p->right_boundary = p->world_origin[0] + (float)((uint32_t)(off + fs[0]) * 2u) * r; /* :56-57 */
    float cs = r * 2.0f;
    p->cell_size[0] = p->cell_size[1] = p->cell_size[2] = cs;
    p->boundary_damping = -1.0f;
    p->gravity[0] = 0.0f; p->gravity[1] = -9.8f; p->gravity[2] = 0.0f;
    p->gamma = 7;
    /* B = 200 * rho0 * |g.y| * (2 r fy) / gamma, :67-68 */
    p->B = 200 * p->rest_density * fabsf(p->gravity[1]) * (2 * r * (float)fs[1]) / p->gamma;
    p->lj_D = 10 * p->gravity[1] * 2 * r * (float)fs[1];  /* :70 */
    p->lj_a = 1 * r;
    p->soundspeed = sqrtf(p->B * p->gamma / p->rest_density); /* :73 */
    p->delta_time = powf(10.0f, -4.0f);                   /* :75 */
    p->world_size[0] = gs[0] * 2.0f * r; p->world_size[1] = gs[1] * 2.0f * r;
    p->world_size[2] = gs[2] * 2.0f * r;
    return 0;
}

/* PoiseuilleFlowSystem ctor, Poiseuille.Core/poiseuilleFlowSystem.cpp:21-67 */
int orc_poiseuille_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                          cmag_sph_params *p)
{
    common_defaults(p);
    p->system = CMAG_POISEUILLE;
    for (int k = 0; k < 3; ++k) { p->fluid_size[k] = fs[k]; p->grid_size[k] = gs[k]; }
    p->boundary_offset = off;
    p->particle_radius = r;
    p->smoothing_radius = 3.0f * r;
    p->rest_density = 1000.0f;
    p->particle_mass = (float)(1000.0f / 3381320880.551724); /* :48-49 */
    p->cell_count = 3;
    float hx = gs[0] * r, hy = gs[1] * r, hz = gs[2] * r;
    p->world_origin[0] = -hx; p->world_origin[1] = -hy; p->world_origin[2] = -hz;
    float cs = r * 2.0f;
    p->cell_size[0] = p->cell_size[1] = p->cell_size[2] = cs;
    p->boundary_damping = -1.0f;
    p->gravity[0] = powf(10.0f, -4.0f); p->gravity[1] = 0.0f; p->gravity[2] = 0.0f; /* :60 */
    p->soundspeed = powf(10.0f, -4.0f);                   /* :62 */
    p->mu = powf(10.0f, -3.0f);                           /* :63 */
    p->delta_time = powf(10.0f, -4.0f);
    p->gamma = 7.0f;
    p->world_size[0] = gs[0] * 2.0f * r; p->world_size[1] = gs[1] * 2.0f * r;
    p->world_size[2] = gs[2] * 2.0f * r;
    return 0;
}

/* PeristalsisSystem ctor, Peristalsis.Core/PeristalsisSystem.cpp:17-80 */
int orc_peristalsis_params(float dt, const uint32_t fs[3], float amplitude, float wave_speed,
                           float soundspeed, const float g[3], int32_t off,
                           const uint32_t gs[3], float r, cmag_sph_params *p)
{
    common_defaults(p);
    p->system = CMAG_PERISTALSIS;
    for (int k = 0; k < 3; ++k) { p->fluid_size[k] = fs[k]; p->grid_size[k] = gs[k]; }
    p->boundary_offset = off;
    p->amplitude = amplitude;
    p->wave_speed = wave_speed;
    p->particle_radius = r;
    p->smoothing_radius = 3.0f * r;
    p->rest_density = 1000.0f;
    p->particle_mass = 0.0f;                               /* set by Reset */
    p->cell_count = 3;
    float hx = gs[0] * r, hy = gs[1] * r, hz = gs[2] * r;
    p->world_origin[0] = -hx; p->world_origin[1] = -hy; p->world_origin[2] = -hz;
    float cs = r * 2.0f;
    p->cell_size[0] = p->cell_size[1] = p->cell_size[2] = cs;
    p->world_size[0] = gs[0] * 2.0f * r;                   /* :38-41 */
    p->world_size[1] = gs[1] * 2.0f * r;
    p->world_size[2] = gs[2] * 2.0f * r;
    p->boundary_damping = -1.0f;
    for (int k = 0; k < 3; ++k) p->gravity[k] = g[k];
    p->soundspeed = soundspeed;
    p->mu = powf(10.0f, -3.0f);
    p->delta_time = dt;
    p->gamma = 7.0f;
    p->is_boundary_configuration = 1;                      /* :56 */
    return 0;
}

uint32_t orc_particle_count(const cmag_sph_params *p)
{
    uint32_t fx = p->fluid_size[0], fy = p->fluid_size[1], fz = p->fluid_size[2];
    uint32_t gx = p->grid_size[0], gy = p->grid_size[1];
    uint32_t off = (uint32_t)p->boundary_offset;
    if (p->system == CMAG_DAMBREAK) /* fluidSystem.cpp:34-37 */
        return fx * fy * fz + gx * off + 2u * (gy - off) * off;
    return fx * fy * fz + 2u * gx * off; /* poiseuilleFlowSystem.cpp:35-36, PeristalsisSystem.cpp:23-24 */
}

/* ------------------------------------------------------------------------ */
/* scene generators                                                         */
/* ------------------------------------------------------------------------ */

static void put4(float *pos, uint32_t i, uint32_t n, float x, float y, float z, float w)
{
    if (i >= n) return;
    pos[4 * (size_t)i] = x; pos[4 * (size_t)i + 1] = y; pos[4 * (size_t)i + 2] = z;
    pos[4 * (size_t)i + 3] = w;
}

/* DamBreakSystem::initFluid + initBoundaryParticles, fluidSystem.cpp:382-523 */
static void dambreak_scene(const cmag_sph_params *p, float *pos, uint32_t n)
{
    float r = p->particle_radius, spacing = r * 2.0f;
    float hx = p->grid_size[0] * r, hy = p->grid_size[1] * r, hz = p->grid_size[2] * r;
    int off = p->boundary_offset;
    uint32_t fx = p->fluid_size[0], fy = p->fluid_size[1], fz = p->fluid_size[2];
    uint32_t gx = p->grid_size[0], gy = p->grid_size[1];
    const float *o = p->world_origin;
    for (uint32_t z = 0; z < fz; z++)
        for (uint32_t y = 0; y < fy; y++)
            for (uint32_t x = 0; x < fx; x++) {
                uint32_t i = (z * fy * fx) + y * fx + x;
                put4(pos, i, n, (spacing * x) + r - hx + off * 2 * r,
                     (spacing * y) + r - hy + off * 2 * r, (spacing * z) + r - hz, CMAG_FLUID);
            }
    if (off <= 0) return; /* reset: if(params.boundaryOffset > 0) */
    uint32_t na = fx * fy * fz, s0, s1;
    /* bottom, FirstType */
    s0 = gx - (uint32_t)(off - 1);
    for (uint32_t x = 0; x < s0; x++)
        put4(pos, na + x, n, (spacing * x) + r + o[0] + (off - 1) * 2 * r,
             (spacing * 0u) + r + o[1] + (off - 1) * 2 * r, (spacing * 0u) + r + o[2], CMAG_FIRST_TYPE);
    na += s0;
    /* left, FirstType */
    s1 = gy - (uint32_t)off;
    for (uint32_t y = 0; y < s1; y++)
        put4(pos, na + y, n, (spacing * 0u) + r + o[0] + (off - 1) * 2 * r,
             (spacing * y) + r + o[1] + (off + 0) * 2 * r, (spacing * 0u) + r + o[2], CMAG_FIRST_TYPE);
    na += s1;
    /* right gate, RightFirstType */
    for (uint32_t y = 0; y < s1; y++)
        put4(pos, na + y, n, (spacing * 0u) + r + o[0] + (fx + (uint32_t)off) * 2 * r,
             (spacing * y) + r + o[1] + off * 2 * r, (spacing * 0u) + r + o[2], CMAG_RIGHT_FIRST_TYPE);
    na += s1;
    /* bottom, SecondType */
    s0 = gx; s1 = (uint32_t)(off - 1);
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++)
            put4(pos, na + y * s0 + x, n, (spacing * x) + r + o[0], (spacing * y) + r + o[1],
                 (spacing * 0u) + r + o[2], CMAG_SECOND_TYPE);
    na += s0 * s1;
    /* left, SecondType */
    s0 = (uint32_t)(off - 1); s1 = gy - (uint32_t)(off - 1);
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++)
            put4(pos, na + y * s0 + x, n, (spacing * x) + r + o[0],
                 (spacing * y) + r + o[1] + (off - 1) * 2 * r, (spacing * 0u) + r + o[2], CMAG_SECOND_TYPE);
    na += s0 * s1;
    /* right gate, RightSecondType */
    s0 = (uint32_t)(off - 1); s1 = gy - (uint32_t)off;
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++)
            put4(pos, na + y * s0 + x, n,
                 (spacing * x) + r + o[0] + (fx + (uint32_t)off + 1u) * 2 * r,
                 (spacing * y) + r + o[1] + (off) * 2 * r, (spacing * 0u) + r + o[2], CMAG_RIGHT_SECOND_TYPE);
}

/* PoiseuilleFlowSystem::initFluid + initBoundaryParticles, poiseuilleFlowSystem.cpp:325-383 */
static void poiseuille_scene(const cmag_sph_params *p, float *pos, uint32_t n)
{
    float r = p->particle_radius, spacing = r * 2.0f;
    float hx = p->grid_size[0] * r, hy = p->grid_size[1] * r, hz = p->grid_size[2] * r;
    int off = p->boundary_offset;
    uint32_t fx = p->fluid_size[0], fy = p->fluid_size[1], fz = p->fluid_size[2];
    uint32_t gx = p->grid_size[0];
    const float *o = p->world_origin;
    for (uint32_t z = 0; z < fz; z++)
        for (uint32_t y = 0; y < fy; y++)
            for (uint32_t x = 0; x < fx; x++) {
                uint32_t i = (z * fy * fx) + y * fx + x;
                put4(pos, i, n, (spacing * x) + r - hx, (spacing * y) + r - hy + off * 2 * r,
                     (spacing * z) + r - hz, 0.0f);
            }
    uint32_t na = fx * fy * fz, s0 = gx, s1 = (uint32_t)off;
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++)
            put4(pos, na + y * s0 + x, n, (spacing * x) + r + o[0], (spacing * y) + r + o[1],
                 (spacing * 0u) + r + o[2], 1.0f);
    na += s0 * s1;
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++)
            put4(pos, na + y * s0 + x, n, (spacing * x) + r + o[0],
                 (spacing * y) + r + o[1] + off * 2 * r + fy * 2.0f * r,
                 (spacing * 0u) + r + o[2], 1.0f);
}

/* PeristalsisSystem::initFluid + initBoundaryParticles, PeristalsisSystem.cpp:255-317 */
static void peristalsis_scene(const cmag_sph_params *p, float *pos, uint32_t n)
{
    float r = p->particle_radius, spacing = r * 2.0f;
    float hx = p->grid_size[0] * r, hz = p->grid_size[2] * r;
    int off = p->boundary_offset;
    uint32_t fx = p->fluid_size[0], fy = p->fluid_size[1], fz = p->fluid_size[2];
    const float *o = p->world_origin;
    for (int z = 0; z < (int)fz; z++)
        for (int y = 0; y < (int)fy; y++)
            for (int x = 0; x < (int)fx; x++) {
                uint32_t i = (uint32_t)((z * (int)fy * (int)fx) + y * (int)fx + x);
                put4(pos, i, n, (spacing * x) + r - hx, -1.0f * fy * r + (spacing * y) + r,
                     (spacing * z) + r - hz, 0.0f);
            }
    uint32_t na = fx * fy * fz, s0 = fx, s1 = (uint32_t)off;
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++) {
            float j = r * (2 * x + 1);
            put4(pos, na + y * s0 + x, n, j + o[0], -1.0f * fy * r - (spacing * y) - r,
                 (spacing * 0u) + r + o[2], 2.0f * (1.0f + y));
        }
    na += s0 * s1;
    for (uint32_t y = 0; y < s1; y++)
        for (uint32_t x = 0; x < s0; x++) {
            float j = r * (2 * x + 1);
            put4(pos, na + y * s0 + x, n, j + o[0], fy * r + (spacing * y) + r,
                 (spacing * 0u) + r + o[2], -2.0f * (1.0f + y));
        }
}

void orc_scene(const cmag_sph_params *p, float *pos, uint32_t n)
{
    memset(pos, 0, sizeof(float) * 4 * (size_t)n);
    if (p->system == CMAG_DAMBREAK) dambreak_scene(p, pos, n);
    else if (p->system == CMAG_POISEUILLE) poiseuille_scene(p, pos, n);
    else peristalsis_scene(p, pos, n);
}

/* PeristalsisSystem::CalculateMass, PeristalsisSystem.cpp:238-253 */
float orc_peristalsis_mass_sum(const cmag_sph_params *p, const float *pos, uint32_t n)
{
    uint32_t t = p->grid_size[0] / 2;
    float tx = pos[t * 4 + 0], ty = pos[t * 4 + 1];
    float h = p->smoothing_radius, sum = 0.0f;
    for (uint32_t i = 0; i < n; i++) {
        float rx = tx - pos[4 * (size_t)i], ry = ty - pos[4 * (size_t)i + 1];
        float dist = sqrtf(rx * rx + ry * ry);
        float q = dist / h;
        float coeff = 7.0f / 4 / ORC_PI_F / powf(h, 2);
        if (q < 2) sum += coeff * (powf(1 - 0.5f * q, 4) * (2 * q + 1));
    }
    return sum;
}

/* ---- 3-D dam break (extension) ---- */
uint32_t orc_dambreak3d_count(const uint32_t fs[3], const uint32_t tank[3], uint32_t L)
{
    uint64_t shell = (uint64_t)(tank[0] + 2 * L) * (tank[1] + L) * (tank[2] + 2 * L) -
                     (uint64_t)tank[0] * tank[1] * tank[2];
    return (uint32_t)((uint64_t)fs[0] * fs[1] * fs[2] + shell);
}

static uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

/* uniform in [-1, 1): 24 random bits */
static float jitter_unit(uint64_t seed, uint64_t i, int axis)
{
    uint64_t r = splitmix64(seed * 0x100000001B3ull + i * 3u + (uint64_t)axis);
    return (float)(int32_t)((uint32_t)(r >> 40) - (1u << 23)) * (1.0f / 8388608.0f);
}

/* Fluid block on cells [0,fx)x[0,fy)x[0,fz) of the tank interior (cell k centred
 * at (k+0.5)*spacing) with jitter; walls are every cell of
 * [-L,tx+L)x[-L,ty)x[-L,tz+L) outside the interior (floor and four sides, open
 * top).  Order: fluid (x fastest, then y, z), then walls (x fastest). */
void orc_dambreak3d_scene(const cmag_sph_params *p, const uint32_t tank[3], uint32_t L,
                          float jitter_frac, uint64_t seed, float *pos, uint32_t n)
{
    float spacing = p->particle_radius * 2.0f;
    float jit = jitter_frac * spacing;
    const uint32_t *fs = p->fluid_size;
    uint32_t i = 0;
    for (uint32_t z = 0; z < fs[2]; z++)
        for (uint32_t y = 0; y < fs[1]; y++)
            for (uint32_t x = 0; x < fs[0]; x++, i++) {
                float px = ((float)x + 0.5f) * spacing + jit * jitter_unit(seed, i, 0);
                float py = ((float)y + 0.5f) * spacing + jit * jitter_unit(seed, i, 1);
                float pz = ((float)z + 0.5f) * spacing + jit * jitter_unit(seed, i, 2);
                put4(pos, i, n, px, py, pz, CMAG_FLUID);
            }
    int iL = (int)L;
    for (int z = -iL; z < (int)tank[2] + iL; z++)
        for (int y = -iL; y < (int)tank[1]; y++)
            for (int x = -iL; x < (int)tank[0] + iL; x++) {
                int inside = x >= 0 && x < (int)tank[0] && y >= 0 && z >= 0 && z < (int)tank[2];
                if (inside) continue;
                put4(pos, i, n, ((float)x + 0.5f) * spacing, ((float)y + 0.5f) * spacing,
                     ((float)z + 0.5f) * spacing, CMAG_FIRST_TYPE);
                i++;
            }
}

/* ------------------------------------------------------------------------ */
/* hash, sort, reorder                                                      */
/* ------------------------------------------------------------------------ */

/* calcGridPos: fluid_kernel.cu:19-25 divides by cellSize; poiseuilleFlowKernel.cu:18-24
 * and PeristalsisKernel.cu:18-24 multiply by 0.5f and divide by the radius. */
static i3 grid_pos(const cmag_sph_params *p, float x, float y, float z)
{
    i3 g;
    if (p->system == CMAG_DAMBREAK) {
        g.x = sat_f2i(floorf((x - p->world_origin[0]) / p->cell_size[0]));
        g.y = sat_f2i(floorf((y - p->world_origin[1]) / p->cell_size[1]));
        g.z = sat_f2i(floorf((z - p->world_origin[2]) / p->cell_size[2]));
    } else {
        float r = p->particle_radius;
        g.x = sat_f2i(floorf((x - p->world_origin[0]) * 0.5f / r));
        g.y = sat_f2i(floorf((y - p->world_origin[1]) * 0.5f / r));
        g.z = sat_f2i(floorf((z - p->world_origin[2]) * 0.5f / r));
    }
    return g;
}

static int is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

/* periodic wrap onto [0, n): the reference's mask (fluid_kernel.cu:28-30) for
 * power-of-two grids; the same residue for other sizes (extension) */
static uint32_t wrap_cell(int v, uint32_t n, int pow2)
{
    if (pow2) return (uint32_t)v & (n - 1);
    long long m = (long long)v % (long long)n;
    return (uint32_t)(m < 0 ? m + (long long)n : m);
}

/* calcGridHash, fluid_kernel.cu:27-32: z*Y*X + y*X + x of the wrapped cell */
static uint32_t grid_hash(const cmag_sph_params *p, i3 g)
{
    uint32_t X = p->grid_size[0], Y = p->grid_size[1], Z = p->grid_size[2];
    int pow2 = is_pow2(X) && is_pow2(Y) && is_pow2(Z);
    uint32_t x = wrap_cell(g.x, X, pow2), y = wrap_cell(g.y, Y, pow2), z = wrap_cell(g.z, Z, pow2);
    return umul24(umul24(z, Y), X) + umul24(y, X) + x;
}

/* calcHashD, fluid_kernel.cu:34-48 (and the Poiseuille/Peristalsis copies) */
void orc_calc_hash(const cmag_sph_params *p, const float *pos, uint32_t *hash, uint32_t *idx,
                   uint32_t n)
{
    for (uint32_t i = 0; i < n; i++) {
        i3 g = grid_pos(p, pos[4 * (size_t)i], pos[4 * (size_t)i + 1], pos[4 * (size_t)i + 2]);
        hash[i] = grid_hash(p, g);
        idx[i] = i;
    }
}

/* thrust::sort_by_key (fluidSystem.cu:94-99): stable ascending key sort; an LSD
 * counting sort on 16-bit digits is stable by construction. */
void orc_sort_pairs(uint32_t *hash, uint32_t *idx, uint32_t n)
{
    uint32_t *kt = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t *vt = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t *cnt = (uint32_t *)malloc(sizeof(uint32_t) * 65537);
    uint32_t *ka = hash, *va = idx, *kb = kt, *vb = vt;
    for (int shift = 0; shift < 32; shift += 16) {
        memset(cnt, 0, sizeof(uint32_t) * 65537);
        for (uint32_t i = 0; i < n; i++) cnt[((ka[i] >> shift) & 0xffffu) + 1]++;
        for (uint32_t d = 0; d < 65536; d++) cnt[d + 1] += cnt[d];
        for (uint32_t i = 0; i < n; i++) {
            uint32_t d = (ka[i] >> shift) & 0xffffu;
            uint32_t o = cnt[d]++;
            kb[o] = ka[i]; vb[o] = va[i];
        }
        uint32_t *t = ka; ka = kb; kb = t; t = va; va = vb; vb = t;
    }
    /* two passes: result is back in hash/idx */
    free(kt); free(vt); free(cnt);
}

/* reorderDataAndFindCellStartD + cudaMemset(cellStart, 0xff), fluid_kernel.cu:50-97,
 * fluidSystem.cu:150-188.  cellEnd is not cleared (as in the reference). */
void orc_reorder(const uint32_t *hash, const uint32_t *idx, const float *pos, const float *vel,
                 uint32_t *cell_start, uint32_t *cell_end, float *spos, float *svel, uint32_t n,
                 uint64_t ncells)
{
    for (uint64_t c = 0; c < ncells; c++) cell_start[c] = ORC_EMPTY;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t h = hash[i];
        if (i == 0 || h != hash[i - 1]) {
            cell_start[h] = i;
            if (i > 0) cell_end[hash[i - 1]] = i;
        }
        if (i == n - 1) cell_end[h] = i + 1;
        memcpy(spos + 4 * (size_t)i, pos + 4 * (size_t)idx[i], 16);
        memcpy(svel + 4 * (size_t)i, vel + 4 * (size_t)idx[i], 16);
    }
}

/* ------------------------------------------------------------------------ */
/* smoothing kernel and equation of state                                    */
/* ------------------------------------------------------------------------ */

/* kernel value W(q), q < 2.  Wendland/2-D is the reference expression
 * (fluid_kernel.cu:121-124); the rest are the documented extensions. */
static float kernel_w(const cmag_sph_params *p, float q)
{
    float h = p->smoothing_radius;
    if (p->kernel == CMAG_KERNEL_WENDLAND) {
        float coeff = (p->dims == 2) ? 7.0f / 4 / ORC_PI_F / powf(h, 2)
                                     : 21.0f / 16 / ORC_PI_F / powf(h, 3);
        return coeff * (powf(1 - 0.5f * q, 4) * (2 * q + 1));
    }
    float sigma = (p->dims == 2) ? 10.0f / 7 / ORC_PI_F / powf(h, 2) : 1.0f / ORC_PI_F / powf(h, 3);
    if (q < 1.0f) return sigma * (1.0f - 1.5f * q * q + 0.75f * q * q * q);
    float t = 2.0f - q;
    return sigma * (0.25f * t * t * t);
}

/* kernel radial derivative dW/dr, q < 2.  Wendland/2-D: DamBreak and Poiseuille
 * use 7/2/pi/h^3 (fluid_kernel.cu:222-224), Peristalsis 7/(2 pi h^3)
 * (PeristalsisPressureForce.cu:36-38, PeristalsisViscousForce.cu:201-205). */
static float kernel_dw(const cmag_sph_params *p, float q)
{
    float h = p->smoothing_radius;
    if (p->kernel == CMAG_KERNEL_WENDLAND) {
        float coeff;
        if (p->dims == 2)
            coeff = (p->system == CMAG_PERISTALSIS) ? 7.0f / (2 * ORC_PI_F * powf(h, 3))
                                                    : 7.0f / 2 / ORC_PI_F / powf(h, 3);
        else
            coeff = 21.0f / 8 / ORC_PI_F / powf(h, 4);
        return coeff * (-powf(1 - 0.5f * q, 3) * (2 * q + 1) + powf(1 - 0.5f * q, 4));
    }
    float sigma = (p->dims == 2) ? 10.0f / 7 / ORC_PI_F / powf(h, 2) : 1.0f / ORC_PI_F / powf(h, 3);
    float s = sigma / h;
    if (q < 1.0f) return s * (-3.0f * q + 2.25f * q * q);
    float t = 2.0f - q;
    return s * (-0.75f * t * t);
}

/* 1 + |d ln(dW/dr) / d ln q|: how much a relative rounding of the distance is
 * amplified in the kernel derivative (large near q = 2, where dW/dr -> 0) */
static float kernel_dw_cond(const cmag_sph_params *p, float q)
{
    if (p->kernel == CMAG_KERNEL_WENDLAND) {
        float t = 1.0f - 0.5f * q;
        return 1.0f + fabsf(1.0f - 1.5f * q / fmaxf(t, 1e-6f));
    }
    if (q < 1.0f) return 1.0f + fabsf((-3.0f + 4.5f * q) / (-3.0f + 2.25f * q));
    return 1.0f + 2.0f * q / fmaxf(2.0f - q, 1e-6f);
}

static float eos_pressure(const cmag_sph_params *p, float dens)
{
    if (p->eos == CMAG_EOS_TAIT || p->system == CMAG_DAMBREAK)
        return p->B * (powf(dens / p->rest_density, p->gamma) - 1.0f); /* fluid_kernel.cu:168 */
    if (p->system == CMAG_POISEUILLE)
        return powf(p->soundspeed, 2) * dens;                          /* poiseuilleFlowKernel.cu:181 */
    return 50 * powf(p->soundspeed, 1) * dens;                         /* PeristalsisDensity.cu:75 */
}

/* EvaluateShift, PeristalsisUtil.cu:4-11 */
static int eval_shift(int pos, uint32_t size)
{
    if (pos < 0) return -1;
    if (pos > (int)size - 1) return 1;
    return 0;
}

/* relative position of j as seen from i through the neighbour cell g:
 * DamBreak plain; Poiseuille x image (poiseuilleFlowKernel.cu:121-127);
 * Peristalsis image in every axis (PeristalsisDensity.cu:16-22). */
static f3 rel_pos(const cmag_sph_params *p, f3 pi, f3 pj, i3 g)
{
    if (p->system == CMAG_POISEUILLE) {
        float wxs = p->grid_size[0] * 2.0f * p->particle_radius;
        if (g.x < 0) return mk3(pi.x - (pj.x - wxs), pi.y - pj.y, pi.z - pj.z);
        if ((uint32_t)g.x > p->grid_size[0] - 1) return mk3(pi.x - (pj.x + wxs), pi.y - pj.y, pi.z - pj.z);
        return sub3(pi, pj);
    }
    if (p->system == CMAG_PERISTALSIS) {
        int sx = eval_shift(g.x, p->grid_size[0]), sy = eval_shift(g.y, p->grid_size[1]),
            sz = eval_shift(g.z, p->grid_size[2]);
        return mk3(pi.x - (pj.x + sx * p->world_size[0]), pi.y - (pj.y + sy * p->world_size[1]),
                   pi.z - (pj.z + sz * p->world_size[2]));
    }
    return sub3(pi, pj);
}

/* ------------------------------------------------------------------------ */
/* density                                                                  */
/* ------------------------------------------------------------------------ */

/* sumDensity over the (2c+1)^3 cell box: fluid_kernel.cu:99-128/130-166,
 * poiseuilleFlowKernel.cu:99-139/141-179, PeristalsisDensity.cu:3-37/39-68 */
static float density_sum(const cmag_sph_params *p, const float *spos, const uint32_t *cs,
                         const uint32_t *ce, uint32_t i)
{
    f3 pi = ld3(spos, i);
    i3 g = grid_pos(p, pi.x, pi.y, pi.z);
    int c = p->cell_count;
    float h = p->smoothing_radius, sum = 0.0f;
    for (int z = -c; z <= c; z++)
        for (int y = -c; y <= c; y++)
            for (int x = -c; x <= c; x++) {
                i3 nb = {g.x + x, g.y + y, g.z + z};
                uint32_t gh = grid_hash(p, nb);
                uint32_t start = cs[gh];
                float csum = 0.0f;
                if (start != ORC_EMPTY) {
                    uint32_t end = ce[gh];
                    for (uint32_t j = start; j < end; j++) {
                        f3 rp = rel_pos(p, pi, ld3(spos, j), nb);
                        float dist = len3(rp);
                        float q = dist / h;
                        if (q < 2) csum += kernel_w(p, q);
                    }
                }
                sum += csum;
            }
    return sum;
}

float orc_density_at(const cmag_sph_params *p, const float *spos, const uint32_t *cs,
                     const uint32_t *ce, uint32_t i)
{
    return density_sum(p, spos, cs, ce, i) * p->particle_mass;
}

void orc_density(const cmag_sph_params *p, const float *spos, float *meas, const uint32_t *cs,
                 const uint32_t *ce, uint32_t n, int threads)
{
    (void)threads;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : 1)
    for (long li = 0; li < (long)n; li++) {
        uint32_t i = (uint32_t)li;
        float *m = meas + 4 * (size_t)i;
        float w = spos[4 * (size_t)i + 3];
        if (p->system == CMAG_POISEUILLE && w == 1.0f) { /* poiseuilleFlowKernel.cu:154-158 */
            m[0] = p->rest_density;
            m[1] = eos_pressure(p, p->rest_density);
            continue;
        }
        float dens = density_sum(p, spos, cs, ce, i) * p->particle_mass;
        m[0] = dens;
        m[1] = eos_pressure(p, dens);
        if (p->system == CMAG_PERISTALSIS) { m[2] = 0; m[3] = w; } /* PeristalsisDensity.cu:72-77 */
    }
}

/* ------------------------------------------------------------------------ */
/* forces                                                                   */
/* ------------------------------------------------------------------------ */

/* getVelocityDiff with wall velocity extrapolation, poiseuilleFlowKernel.cu:184-208 */
static f3 poiseuille_vab(const cmag_sph_params *p, f3 vi, f3 pi, f3 vj, f3 pj, float wj)
{
    float bottom = p->world_origin[1] + p->boundary_offset * 2.0f * p->particle_radius;
    float top = bottom + p->fluid_size[1] * 2.0f * p->particle_radius;
    if (wj == 1.0f && pj.y > top) {
        float da = top - pi.y, db = pj.y - top;
        float beta = fminf(1000.0f, 1 + db / da);
        return smul3(beta, vi);
    }
    if (wj == 1.0f && pj.y < bottom) {
        float da = pi.y - bottom, db = bottom - pj.y;
        float beta = fminf(1000.0f, 1 + db / da);
        return smul3(beta, vi);
    }
    return sub3(vi, vj);
}

/* Peristalsis no-slip extrapolation into the moving walls (an option of this
 * build; the reference keeps it commented out, PeristalsisViscousForce.cu:4-138):
 * the wall interfaces y = +-half height +- A sin(K((x - ox) - c t)), their closest
 * point to a fluid particle by Newton's method, and the wall velocity there.  The
 * wall state (amplitude, time, moving) is set by orc_set_wall_state or orc_step. */
static float g_wall_amp = 0.0f, g_wall_t = 0.0f;
static int g_wall_moving = 0;

void orc_set_wall_state(float amp, float t, int32_t moving)
{
    g_wall_amp = amp;
    g_wall_t = t;
    g_wall_moving = moving;
}

typedef struct { float xa, ya, slope, inv_norm, inv_da, vw; } wall_side_t;

static wall_side_t wall_side(const cmag_sph_params *p, float sgn, float base, float x0, float y0)
{
    const float K = 3.141592654f * p->wave_count / (p->fluid_size[0] * p->particle_radius);
    const float ox = p->world_origin[0], c = p->wave_speed, amp = g_wall_amp, t = g_wall_t;
    const float r = p->particle_radius, h = p->smoothing_radius;
    float x = x0;
    for (int it = 0; it < 8; ++it) {
        float ph = K * ((x - ox) - c * t);
        float s = sinf(ph), cs = cosf(ph);
        float yw = base + sgn * amp * s;
        float d1 = sgn * amp * K * cs, d2 = -sgn * amp * K * K * s;
        float f = (x0 - x) + (y0 - yw) * d1;
        float df = -1.0f - d1 * d1 + (y0 - yw) * d2;
        float dx = f / df;
        x -= dx;
        if (!(fabsf(dx) >= 1e-3f * r)) break;
    }
    if (!(fabsf(x - x0) < 4.0f * h)) x = x0;
    float ph = K * ((x - ox) - c * t);
    float s = sinf(ph), cs = cosf(ph);
    wall_side_t w;
    w.xa = x;
    w.ya = base + sgn * amp * s;
    w.slope = sgn * amp * K * cs;
    w.inv_norm = 1.0f / sqrtf(1.0f + w.slope * w.slope);
    float da = sqrtf((x0 - x) * (x0 - x) + (y0 - w.ya) * (y0 - w.ya));
    w.inv_da = 1.0f / fmaxf(da, 1e-6f * r);
    w.vw = g_wall_moving ? -sgn * amp * K * c * cs : 0.0f;
    return w;
}

/* Force on sorted particle i.  Returns 0 when the reference writes nothing for i
 * (DamBreak non-fluid particles, fluid_kernel.cu:258). */
/* |t| summed component-wise over the pair terms: the scale of the rounding error
 * of any summation order of those terms */
static f3 abs3(f3 a) { return mk3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }

static int force_one(const cmag_sph_params *p, const float *spos, const float *svel,
                     const float *meas, const uint32_t *cs, const uint32_t *ce, uint32_t i,
                     f3 *fa, f3 *fb, f3 *sa, f3 *sb)
{
    f3 scA = mk3(0, 0, 0), scB = mk3(0, 0, 0);
    f3 pi = ld3(spos, i);
    float wi = spos[4 * (size_t)i + 3];
    if (p->system == CMAG_DAMBREAK && wi != (float)CMAG_FLUID) return 0;
    f3 vi = ld3(svel, i);
    float rho = meas[4 * (size_t)i], pr = meas[4 * (size_t)i + 1];
    i3 g = grid_pos(p, pi.x, pi.y, pi.z);
    int c = p->cell_count;
    float h = p->smoothing_radius, m = p->particle_mass;
    f3 fA = mk3(0, 0, 0), fB = mk3(0, 0, 0);
    const int noslip = p->system == CMAG_PERISTALSIS && p->wall_noslip && wi == 0.0f;
    wall_side_t wb = {0, 0, 0, 0, 0, 0}, wt = wb;
    if (noslip) {
        const float hf = p->fluid_size[1] * p->particle_radius;
        wb = wall_side(p, 1.0f, -hf, pi.x, pi.y);
        wt = wall_side(p, -1.0f, hf, pi.x, pi.y);
    }
    for (int z = -c; z <= c; z++)
        for (int y = -c; y <= c; y++)
            for (int x = -c; x <= c; x++) {
                i3 nb = {g.x + x, g.y + y, g.z + z};
                uint32_t gh = grid_hash(p, nb);
                uint32_t start = cs[gh];
                f3 tA = mk3(0, 0, 0), tB = mk3(0, 0, 0);
                if (start != ORC_EMPTY) {
                    uint32_t end = ce[gh];
                    for (uint32_t j = start; j < end; j++) {
                        if (j == i) continue;
                        f3 pj = ld3(spos, j);
                        float wj = spos[4 * (size_t)j + 3];
                        f3 rp = rel_pos(p, pi, pj, nb);
                        float dist = len3(rp);
                        float q = dist / h;
                        if (p->system == CMAG_DAMBREAK) {
                            if (wj != (float)CMAG_FLUID) { /* Lennard-Jones wall, fluid_kernel.cu:199-207 */
                                if (p->lj_cutoff && !(q < 2)) continue;
                                float s = p->lj_D * (powf(p->lj_a / dist, 12) - powf(p->lj_a / dist, 6));
                                f3 term = divs3(smul3(s, rp), powf(dist, 2));
                                tA = add3(tA, term);
                                float smag = fabsf(p->lj_D) * (powf(p->lj_a / dist, 12) + powf(p->lj_a / dist, 6));
                                /* (a/r)^12 amplifies a relative rounding of r twelve times */
                                scA = add3(scA, divs3(smul3(13.0f * smag, abs3(rp)), powf(dist, 2)));
                                continue;
                            }
                            if (q < 2) { /* fluid_kernel.cu:221-237 */
                                f3 vj = ld3(svel, j);
                                float rho2 = meas[4 * (size_t)j], pr2 = meas[4 * (size_t)j + 1];
                                float temp = kernel_dw(p, q);
                                float art = 0.0f;
                                float vij_pij = dot3(sub3(vi, vj), rp);
                                if (vij_pij < 0) {
                                    float nu = 2.0f * p->av_alpha * h * p->soundspeed / (rho + rho2);
                                    art = -1.0f * nu * vij_pij / (dot3(rp, rp) + 0.001f * powf(h, 2));
                                }
                                float s = -1.0f * m * (pr / powf(rho, 2) + pr2 / powf(rho2, 2) + art);
                                f3 term = muls3(smul3(s, normalize3(rp)), temp);
                                tA = add3(tA, term);
                                /* conditioning: the sizes of the factors, with every
                                 * difference (v_i - v_j, p_i + p_j terms) taken as a sum
                                 * of magnitudes */
                                float art_mag = 0.0f;
                                if (vij_pij < 0) {
                                    f3 vs = add3(abs3(vi), abs3(vj));
                                    art_mag = 2.0f * p->av_alpha * h * p->soundspeed / (rho + rho2) *
                                              dot3(vs, abs3(rp)) / (dot3(rp, rp) + 0.001f * powf(h, 2));
                                }
                                float smag = m * (fabsf(pr) / powf(rho, 2) + fabsf(pr2) / powf(rho2, 2) + art_mag);
                                scA = add3(scA, muls3(abs3(rp), smag * fabsf(temp) * kernel_dw_cond(p, q) / dist));
                            }
                        } else if (p->system == CMAG_POISEUILLE) {
                            if (q < 2) { /* poiseuilleFlowKernel.cu:236-245 */
                                f3 vj = ld3(svel, j);
                                float rho2 = meas[4 * (size_t)j], pr2 = meas[4 * (size_t)j + 1];
                                float temp = kernel_dw(p, q);
                                f3 vab = poiseuille_vab(p, vi, pi, vj, pj, wj);
                                float s1 = -1.0f * m * (pr / powf(rho, 2) + pr2 / powf(rho2, 2));
                                f3 t1 = muls3(smul3(s1, normalize3(rp)), temp);
                                float s2 = m * (p->mu + p->mu);
                                f3 t2 = muls3(divs3(muls3(divs3(smul3(s2, vab), rho * rho2), 1.0f), dist), temp);
                                tA = add3(tA, add3(t1, t2));
                                float m1 = m * (fabsf(pr) / powf(rho, 2) + fabsf(pr2) / powf(rho2, 2));
                                f3 vin = (wj == 1.0f && (pj.y > p->world_origin[1] + p->boundary_offset * 2.0f * p->particle_radius +
                                                                   p->fluid_size[1] * 2.0f * p->particle_radius ||
                                                         pj.y < p->world_origin[1] + p->boundary_offset * 2.0f * p->particle_radius))
                                             ? abs3(vab) : add3(abs3(vi), abs3(vj));
                                float ct = fabsf(temp) * kernel_dw_cond(p, q);
                                scA = add3(scA, add3(muls3(abs3(rp), m1 * ct / dist),
                                                     muls3(vin, s2 * ct / (rho * rho2 * dist))));
                            }
                        } else {
                            if (q < 2) {
                                f3 vj = ld3(svel, j);
                                float rho2 = meas[4 * (size_t)j], pr2 = meas[4 * (size_t)j + 1];
                                float temp = kernel_dw(p, q);
                                /* viscous, PeristalsisViscousForce.cu:206-213 */
                                f3 vab = sub3(vi, vj);
                                f3 vmag = add3(abs3(vi), abs3(vj));
                                if (noslip && wj != 0.0f) {
                                    const wall_side_t *w = wj > 0.0f ? &wb : &wt;
                                    const f3 pjs = sub3(pi, rp);  /* j through its image shift */
                                    float db = fabsf(w->slope * (pjs.x - w->xa) - (pjs.y - w->ya)) * w->inv_norm;
                                    float bmax = p->wall_beta_max > 0.0f ? p->wall_beta_max : 1000.0f;
                                    float beta = fminf(bmax, 1.0f + db * w->inv_da);
                                    vab = mk3(beta * vi.x, beta * (vi.y - w->vw), beta * vi.z);
                                    vmag = add3(abs3(vab), smul3(beta, abs3(mk3(0, w->vw, 0))));
                                }
                                float sv = m * temp * (p->mu + p->mu);
                                f3 tv = divs3(smul3(sv, vab), rho * rho2 * dist);
                                tA = add3(tA, tv);
                                scA = add3(scA, muls3(vmag, fabsf(sv) * kernel_dw_cond(p, q) / (rho * rho2 * dist)));
                                /* pressure, PeristalsisPressureForce.cu:39-43 */
                                float sp = -1.0f * m * temp * (pr / powf(rho, 2) + pr2 / powf(rho2, 2));
                                f3 tp = smul3(sp, normalize3(rp));
                                tB = add3(tB, tp);
                                float pm = m * fabsf(temp) * kernel_dw_cond(p, q) *
                                           (fabsf(pr) / powf(rho, 2) + fabsf(pr2) / powf(rho2, 2));
                                scB = add3(scB, muls3(abs3(rp), pm / dist));
                            }
                        }
                    }
                }
                fA = add3(fA, tA);
                fB = add3(fB, tB);
            }
    *fa = fA;
    *fb = fB;
    if (sa) *sa = scA;
    if (sb) *sb = scB;
    return 1;
}

void orc_force_at(const cmag_sph_params *p, const float *spos, const float *svel,
                  const float *meas, const uint32_t *cs, const uint32_t *ce, uint32_t i,
                  float out_a[3], float out_b[3], int32_t *written)
{
    f3 a, b;
    *written = force_one(p, spos, svel, meas, cs, ce, i, &a, &b, NULL, NULL);
    if (!*written) { a = mk3(0, 0, 0); b = a; }
    out_a[0] = a.x; out_a[1] = a.y; out_a[2] = a.z;
    out_b[0] = b.x; out_b[1] = b.y; out_b[2] = b.z;
}

/* calcAndApplyAccelerationD (fluid_kernel.cu:245-292), calculatePoiseuilleAccelerationD
 * (poiseuilleFlowKernel.cu:267-309), computeViscousForceD + computePressureForceD
 * (PeristalsisViscousForce.cu:198-242, PeristalsisPressureForce.cu:51-91):
 * results scattered to original order through the sorted index. */
void orc_force(const cmag_sph_params *p, const float *spos, const float *svel, const float *meas,
               const uint32_t *idx, const uint32_t *cs, const uint32_t *ce, float *out_a,
               float *out_b, uint32_t n, int threads)
{
    (void)threads;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : 1)
    for (long li = 0; li < (long)n; li++) {
        uint32_t i = (uint32_t)li;
        f3 a, b;
        if (!force_one(p, spos, svel, meas, cs, ce, i, &a, &b, NULL, NULL)) continue;
        size_t o = 4 * (size_t)idx[i];
        out_a[o] = a.x; out_a[o + 1] = a.y; out_a[o + 2] = a.z; out_a[o + 3] = 0.0f;
        if (p->system == CMAG_PERISTALSIS && out_b) {
            out_b[o] = b.x; out_b[o + 1] = b.y; out_b[o + 2] = b.z; out_b[o + 3] = 0.0f;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* integration and wall motion                                              */
/* ------------------------------------------------------------------------ */

/* GetWave, PeristalsisKernel.cuh:59-62 (wave_count wavelengths per domain) */
static float get_wave(const cmag_sph_params *p, float x, float t)
{
    return sinf(ORC_PI_F * p->wave_count / (p->fluid_size[0] * p->particle_radius) *
                ((x - p->world_origin[0]) - p->wave_speed * t));
}

void orc_integrate(const cmag_sph_params *p, float *pos, float *vel, float *vlf, const float *acc,
                   const float *vforce, const float *pforce, float t, uint32_t n)
{
    float dt = p->delta_time, r = p->particle_radius;
    f3 g = mk3(p->gravity[0], p->gravity[1], p->gravity[2]);
    for (uint32_t i = 0; i < n; i++) {
        float *P = pos + 4 * (size_t)i, *V = vel + 4 * (size_t)i, *L = vlf + 4 * (size_t)i;
        float w = P[3];
        f3 ps = mk3(P[0], P[1], P[2]), v = mk3(V[0], V[1], V[2]), a;
        if (p->system == CMAG_DAMBREAK) {           /* integrate, fluid_kernel.cu:323-366 */
            if (w != (float)CMAG_FLUID) continue;
            a = ld3(acc, i);
        } else if (p->system == CMAG_POISEUILLE) {  /* integratePoiseuilleSystemD, :311-348 */
            if (w == 1.0f) continue;
            a = ld3(acc, i);
        } else {                                    /* computeCoordinatesD, PeristalsisIntegrate.cu:1-66 */
            if (w != 0.0f && p->is_boundary_configuration) continue;
            if (w > 0.0f) {
                P[1] = -1.0f * p->fluid_size[1] * r + p->amplitude * get_wave(p, P[0], t) - r * (w - 1.0f);
                continue;
            }
            if (w < 0.0f) {
                P[1] = p->fluid_size[1] * r - p->amplitude * get_wave(p, P[0], t) + r * (-w - 1.0f);
                continue;
            }
            a = add3(ld3(vforce, i), ld3(pforce, i));
        }
        f3 nv;
        if (p->system == CMAG_PERISTALSIS) {
            f3 vis = ld3(vforce, i), pres = ld3(pforce, i);
            nv = add3(v, muls3(add3(add3(g, vis), pres), dt));
        } else {
            nv = add3(v, muls3(add3(g, a), dt));
        }
        f3 lf = muls3(add3(v, nv), 0.5f);
        v = nv;
        ps = add3(ps, muls3(v, dt));
        if (p->system == CMAG_DAMBREAK) {
            float left = p->world_origin[0] + p->boundary_offset * 2 * r;
            float bottom = p->world_origin[1] + p->boundary_offset * 2 * r;
            if (ps.x < left) { ps.x = left; v.x *= p->boundary_damping; }
            if (ps.x > p->right_boundary) { ps.x = p->right_boundary; v.x *= p->boundary_damping; }
            if (ps.y < bottom) { ps.y = bottom; v.y *= p->boundary_damping; }
            if (p->clamp_z) { /* extension: the same clamp on the z walls of a 3-D tank */
                if (ps.z < p->z_min_border) { ps.z = p->z_min_border; v.z *= p->boundary_damping; }
                if (ps.z > p->z_max_border) { ps.z = p->z_max_border; v.z *= p->boundary_damping; }
            }
        } else {
            float hx = p->grid_size[0] * r;
            if (ps.x > hx) ps.x -= 2 * hx;
            if (p->system == CMAG_PERISTALSIS && ps.x < -hx) ps.x += 2 * hx;
        }
        P[0] = ps.x; P[1] = ps.y; P[2] = ps.z;
        V[0] = v.x; V[1] = v.y; V[2] = v.z;
        L[0] = lf.x; L[1] = lf.y; L[2] = lf.z;
    }
}

/* configureBoundaryD, PeristalsisKernel.cu:144-171 */
void orc_configure_boundary(const cmag_sph_params *p, float *pos, float wh, uint32_t n)
{
    float r = p->particle_radius;
    for (uint32_t i = 0; i < n; i++) {
        float *P = pos + 4 * (size_t)i;
        float w = P[3];
        if (w > 0.0f) P[1] = -1.0f * p->fluid_size[1] * r + wh * get_wave(p, P[0], 0) - r * (w - 1.0f);
        if (w < 0.0f) P[1] = p->fluid_size[1] * r - wh * get_wave(p, P[0], 0) + r * (-w - 1.0f);
    }
}

/* shiftRightBoundaryD, fluid_kernel.cu:294-306 */
void orc_shift_right_boundary(const cmag_sph_params *p, float *pos, uint32_t n)
{
    for (uint32_t i = 0; i < n; i++) {
        float *P = pos + 4 * (size_t)i;
        if (P[3] != (float)CMAG_RIGHT_FIRST_TYPE && P[3] != (float)CMAG_RIGHT_SECOND_TYPE) continue;
        P[0] = P[0] + p->fluid_size[0] * 2 * p->particle_radius;
    }
}

/* DamBreakSystem::removeRightBoundary + removeRightBoundaryD,
 * fluidSystem.cpp:222-237, fluid_kernel.cu:308-321 */
void orc_remove_right_boundary(cmag_sph_params *p, float *pos, uint32_t n)
{
    p->right_boundary = (float)0xffffffffu;
    float fw = p->fluid_size[0] * 2 * p->particle_radius;
    float ht = p->grid_size[1] * 2 * p->particle_radius;
    for (uint32_t i = 0; i < n; i++) {
        float *P = pos + 4 * (size_t)i;
        if (P[3] != (float)CMAG_RIGHT_FIRST_TYPE && P[3] != (float)CMAG_RIGHT_SECOND_TYPE) continue;
        P[0] = fw;
        P[1] = ht;
    }
}

/* ------------------------------------------------------------------------ */
/* update() orchestration                                                   */
/* ------------------------------------------------------------------------ */

/* DamBreakSystem::update fluidSystem.cpp:257-319, PoiseuilleFlowSystem::update
 * poiseuilleFlowSystem.cpp:212-270, PeristalsisSystem::Update PeristalsisSystem.cpp:320-407 */
void orc_step(cmag_sph_params *p, uint32_t n, uint64_t ncells, float *pos, float *vel, float *vlf,
              float *meas, float *acc, float *vforce, float *pforce, float *spos, float *svel,
              uint32_t *hash, uint32_t *idx, uint32_t *cs, uint32_t *ce, float phase[5],
              int threads, int stop_after)
{
    float dt = p->delta_time;
    static float last_configured = 0.0f;
    if (p->system == CMAG_PERISTALSIS && p->is_boundary_configuration) { /* :330-343 */
        phase[1] += dt;
        if (phase[3] < p->amplitude) {
            orc_configure_boundary(p, pos, phase[3], n);
            last_configured = phase[3];
            phase[3] += dt * powf(10.0f, -3.0f);
        } else {
            phase[2] -= dt;
            if (phase[2] < 0) p->is_boundary_configuration = !p->is_boundary_configuration;
        }
    }
    orc_calc_hash(p, pos, hash, idx, n);
    if (stop_after == CMAG_STAGE_HASH) return;
    orc_sort_pairs(hash, idx, n);
    if (stop_after == CMAG_STAGE_SORT) return;
    orc_reorder(hash, idx, pos, vlf, cs, ce, spos, svel, n, ncells);
    if (stop_after == CMAG_STAGE_REORDER) return;
    orc_density(p, spos, meas, cs, ce, n, threads);
    if (stop_after == CMAG_STAGE_DENSITY) return;
    if (p->system == CMAG_PERISTALSIS && p->wall_noslip) {
        if (p->is_boundary_configuration) orc_set_wall_state(last_configured, 0.0f, 0);
        else orc_set_wall_state(p->amplitude, phase[0] - phase[1], 1);
    }
    if (p->system == CMAG_PERISTALSIS)
        orc_force(p, spos, svel, meas, idx, cs, ce, vforce, pforce, n, threads);
    else
        orc_force(p, spos, svel, meas, idx, cs, ce, acc, NULL, n, threads);
    if (stop_after == CMAG_STAGE_FORCE) return;
    float t = 0.0f;
    if (p->system == CMAG_PERISTALSIS) t = p->is_boundary_configuration ? 0 : phase[0] - phase[1];
    phase[4] = t;
    orc_integrate(p, pos, vel, vlf, acc, vforce, pforce, t, n);
    phase[0] += dt;
}

void orc_force_scale(const cmag_sph_params *p, const float *spos, const float *svel,
                     const float *meas, const uint32_t *idx, const uint32_t *cs,
                     const uint32_t *ce, float *scale_a, float *scale_b, uint32_t n, int threads)
{
    (void)threads;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : 1)
    for (long li = 0; li < (long)n; li++) {
        uint32_t i = (uint32_t)li;
        f3 a, b, sa, sb;
        size_t o = 4 * (size_t)idx[i];
        if (!force_one(p, spos, svel, meas, cs, ce, i, &a, &b, &sa, &sb)) {
            sa = mk3(0, 0, 0);
            sb = sa;
        }
        scale_a[o] = sa.x; scale_a[o + 1] = sa.y; scale_a[o + 2] = sa.z; scale_a[o + 3] = 0;
        if (scale_b) { scale_b[o] = sb.x; scale_b[o + 1] = sb.y; scale_b[o + 2] = sb.z; scale_b[o + 3] = 0; }
    }
}
