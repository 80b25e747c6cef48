/*
 * cmag_sph.h -- C ABI of the GB300-native weakly-compressible SPH time step.
 *
 * This is the drop-in boundary for cmag's three 2-D particle solvers (DamBreak,
 * Poiseuille, Peristalsis).  In the reference each solver is a C++ class over an
 * extern "C" launcher layer that keeps its parameters in one global __constant__
 * block per library:
 *
 *   DamBreak     DamBreak.Core/fluidSystem.h:6-113     launchers fluidSystem.cuh:4-71
 *   Poiseuille   Poiseuille.Core/poiseuilleFlowSystem.h:6-112
 *                                                      launchers poiseuilleFlowSystem.cuh:4-67
 *   Peristalsis  Peristalsis.Core/PeristalsisSystem.h:6-132
 *                                                      launchers PeristalsisSystem.cuh:4-95
 *
 * Here every solver instance is an opaque handle with its own parameter block,
 * device buffers and CUDA stream, so any number of instances of any system can
 * live in one process (the reference's three libraries export clashing names and
 * one parameter block each).  All entry points take plain pointers and sizes,
 * return an int status (CMAG_OK == 0) and never exit the process; the text of the
 * last failure is available from cmag_system_last_error() / cmag_last_error().
 *
 * Array meaning and order follow the reference exactly: positions, velocities,
 * leap-frog velocities, accelerations and forces are in ORIGINAL particle order;
 * measures (x = density, y = pressure), the sorted hash/index pair and the
 * sorted position/velocity copies are in SORTED (cell) order.
 *
 * The C++ classes in include/cmag/systems.hpp mirror the reference class API on
 * top of these entry points.
 */
#ifndef CMAG_SPH_H
#define CMAG_SPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
enum cmag_status {
    CMAG_OK = 0,
    CMAG_ERR_INVALID = 1,  /* bad argument or parameter block                  */
    CMAG_ERR_CUDA = 2,     /* a CUDA runtime call failed (message has the name) */
    CMAG_ERR_NOMEM = 3,    /* device or host allocation failed                  */
    CMAG_ERR_DEVICE = 4,   /* a kernel reported a failed device-side check      */
    CMAG_ERR_STATE = 5     /* call not valid in the current state               */
};

/* device-side check bits, reported by cmag_system_synchronize() */
enum cmag_device_error {
    CMAG_DEVERR_LOOKBACK_TIMEOUT = 1, /* a look-back wait of the radix sort (cmag_sort_particles) hit its spin limit */
    CMAG_DEVERR_RANGE = 2             /* an index left its buffer; access skipped       */
};

/* ---- solver families ---------------------------------------------------- */
enum cmag_system_kind {
    CMAG_DAMBREAK = 0,    /* DamBreak.Core/fluid_kernel.cu                     */
    CMAG_POISEUILLE = 1,  /* Poiseuille.Core/poiseuilleFlowKernel.cu           */
    CMAG_PERISTALSIS = 2  /* Peristalsis.Core/Peristalsis{Density,...}.cu      */
};

/* smoothing kernel; the reference uses the Wendland C2 function everywhere
 * (fluid_kernel.cu:121,222) with the 2-D normalisation 7/(4 pi h^2) */
enum cmag_kernel_fn {
    CMAG_KERNEL_WENDLAND = 0,
    CMAG_KERNEL_CUBIC_SPLINE = 1
};

/* equation of state */
enum cmag_eos {
    CMAG_EOS_REFERENCE = 0, /* per family: DamBreak Tait (fluid_kernel.cu:168),
                               Poiseuille p = c^2 rho (poiseuilleFlowKernel.cu:181),
                               Peristalsis p = 50 c rho (PeristalsisDensity.cu:75)  */
    CMAG_EOS_TAIT = 1       /* p = B((rho/rho0)^gamma - 1) for any family        */
};

/* DamBreak particle types, DamBreak.Core/fluid_kernel.cuh:16-23 */
enum cmag_dambreak_type {
    CMAG_RIGHT_FIRST_TYPE = 0,
    CMAG_FIRST_TYPE = 1,
    CMAG_RIGHT_SECOND_TYPE = 2,
    CMAG_SECOND_TYPE = 3,
    CMAG_FLUID = 4
};

/* ---- particle arrays (setArray / getArray selectors) -------------------- */
enum cmag_array {
    /* float4 arrays */
    CMAG_POSITION = 0,          /* original order; .w = particle type           */
    CMAG_VELOCITY = 1,          /* original order                               */
    CMAG_MEASURES = 2,          /* SORTED order: x density, y pressure          */
    CMAG_ACCELERATION = 3,      /* original order (DamBreak, Poiseuille)        */
    CMAG_VELOCITYLEAPFROG = 4,  /* original order: 0.5 (v_n + v_n+1)            */
    CMAG_VISCOUSFORCE = 5,      /* original order (Peristalsis)                 */
    CMAG_PRESSUREFORCE = 6,     /* original order (Peristalsis)                 */
    CMAG_PREDICTEDPOSITION = 7, /* Peristalsis; allocated, never advanced (the
                                   reference's predictor is dead code)          */
    CMAG_SORTEDPOSITION = 8,    /* sorted order                                 */
    CMAG_SORTEDVELOCITY = 9,    /* sorted order (copy of leap-frog velocity)    */
    /* uint32 arrays (cmag_system_get_uint_array only) */
    CMAG_HASH = 16,             /* sorted cell hash                             */
    CMAG_INDEX = 17,            /* sorted -> original particle index            */
    CMAG_CELLSTART = 18,        /* numGridCells; 0xffffffff for empty cells     */
    CMAG_CELLEND = 19,          /* numGridCells; defined for occupied cells     */
    CMAG_CELLOFFSET = 20        /* numGridCells + 1: first sorted particle with
                                   hash >= cell (dense form used by the kernels) */
};

/* ---- parameter block ---------------------------------------------------- */
/* Superset of SimParams (DamBreak.Core/fluid_kernel.cuh:25-51), PoiseuilleParams
 * (Poiseuille.Core/poiseuilleFlowKernel.cuh:16-35) and Peristalsiscfg
 * (Peristalsis.Core/PeristalsisKernel.cuh:22-63), plus the options that the
 * reference hard-codes.  The *_default_params() functions fill it exactly as the
 * reference constructors do. */
typedef struct cmag_sph_params {
    int32_t system;              /* enum cmag_system_kind                           */
    uint32_t grid_size[3];       /* cells per axis, each a power of two             */
    float world_origin[3];
    float cell_size[3];
    uint32_t fluid_size[3];      /* fluid lattice dimensions                        */
    int32_t cell_count;          /* neighbour cells searched each side (3)          */
    float world_size[3];         /* periodic image shift (Peristalsis)              */

    float gravity[3];
    float particle_radius;
    float smoothing_radius;      /* h */
    float particle_mass;
    float rest_density;
    float soundspeed;
    float B;                     /* Tait coefficient                                */
    float gamma;                 /* Tait exponent                                   */
    float delta_time;
    float boundary_damping;
    float mu;                    /* dynamic viscosity (Poiseuille, Peristalsis)     */
    int32_t boundary_offset;
    float right_boundary;        /* DamBreak gate clamp                             */
    float lj_D;                  /* DamBreak wall force strength D                  */
    float lj_a;                  /* DamBreak wall force length a                    */

    float amplitude;             /* Peristalsis wall wave amplitude                 */
    float wave_speed;
    float wave_count;            /* wavelengths per domain length (reference: 1)    */
    int32_t is_boundary_configuration;

    /* options the reference hard-codes; defaults reproduce the reference */
    int32_t dims;                /* 2: kernel normalised in 2-D (reference); 3: 3-D  */
    int32_t kernel;              /* enum cmag_kernel_fn                              */
    int32_t eos;                 /* enum cmag_eos                                    */
    float av_alpha;              /* DamBreak artificial viscosity (reference 0.38)   */
    int32_t lj_cutoff;           /* 0: wall force from every wall particle in the
                                    searched cell box (reference); 1: only q < 2     */
    int32_t clamp_z;             /* DamBreak: 1 also clamps z to [z_min_border,
                                    z_max_border] like the x/y clamps (3-D tanks)   */
    float z_min_border;
    float z_max_border;
    int32_t wall_noslip;         /* Peristalsis: 1 = no-slip extrapolation of the fluid
                                    velocity into the moving walls (wall distance by
                                    Newton's method, as the reference's commented-out
                                    PeristalsisViscousForce.cu:4-138); 0 = reference   */
    float wall_beta_max;         /* cap of that extrapolation factor (0: 1000)        */
    int32_t reserved[3];
} cmag_sph_params;

/* Reference-constructor parameter derivations.
 * DamBreakSystem::DamBreakSystem        DamBreak.Core/fluidSystem.cpp:17-77
 * PoiseuilleFlowSystem::PoiseuilleFlowSystem  Poiseuille.Core/poiseuilleFlowSystem.cpp:21-67
 * PeristalsisSystem::PeristalsisSystem  Peristalsis.Core/PeristalsisSystem.cpp:17-80 */
int cmag_dambreak_default_params(const uint32_t fluid_size[3], int32_t boundary_offset,
                                 const uint32_t grid_size[3], float particle_radius,
                                 cmag_sph_params *out);
int cmag_poiseuille_default_params(const uint32_t fluid_size[3], int32_t boundary_offset,
                                   const uint32_t grid_size[3], float particle_radius,
                                   cmag_sph_params *out);
int cmag_peristalsis_default_params(float delta_time, const uint32_t fluid_size[3],
                                    float amplitude, float wave_speed, float soundspeed,
                                    const float gravity[3], int32_t boundary_offset,
                                    const uint32_t grid_size[3], float radius,
                                    cmag_sph_params *out);

/* Number of particles a family's reference scene generator creates
 * (fluidSystem.cpp:34-37, poiseuilleFlowSystem.cpp:35-36, PeristalsisSystem.cpp:23-24). */
int cmag_reference_particle_count(const cmag_sph_params *p, uint32_t *out);

/* Host-side scene generators (no device needed): fill pos[4*n] with the
 * reference scene of p (initFluid + initBoundaryParticles, fluidSystem.cpp:382-523,
 * poiseuilleFlowSystem.cpp:325-383, PeristalsisSystem.cpp:255-317), and the
 * Peristalsis lattice kernel sum whose inverse sets the particle mass
 * (CalculateMass, PeristalsisSystem.cpp:238-253). */
int cmag_reference_scene(const cmag_sph_params *p, float *pos, uint32_t n);
int cmag_peristalsis_mass_sum(const cmag_sph_params *p, const float *pos, uint32_t n,
                              float *out);
int cmag_dambreak3d_scene_host(const cmag_sph_params *p, const uint32_t tank_cells[3],
                               uint32_t layers, float jitter_frac, uint64_t seed, float *pos,
                               uint32_t n);

/* ---- solver instances --------------------------------------------------- */
typedef struct cmag_system cmag_system;

/* Allocate a solver for num_particles particles on the current CUDA device
 * (replaces the constructors' _initialize, fluidSystem.cpp:116-190). */
int cmag_system_create(const cmag_sph_params *params, uint32_t num_particles,
                       cmag_system **out);
int cmag_system_destroy(cmag_system *s);

/* Fill the reference scene (reset/Reset: fluidSystem.cpp:361-380,
 * poiseuilleFlowSystem.cpp:311-323, PeristalsisSystem.cpp:213-236).  For
 * Peristalsis this also sets the particle mass from the lattice sum
 * (PeristalsisSystem.cpp:238-253). */
int cmag_system_reset(cmag_system *s);

/* Build a 3-D dam break: fluid block fx*fy*fz on a lattice of spacing
 * 2*particle_radius with uniform jitter of +-jitter_frac*spacing (seeded), in a
 * tank of tank_cells[3] lattice cells with `layers` wall layers on the floor and
 * the four sides.  Particle mass = rest_density * spacing^3.  Extension beyond the
 * reference (which is 2-D only). */
int cmag_dambreak3d_scene(cmag_system *s, const uint32_t tank_cells[3], uint32_t layers,
                          float jitter_frac, uint64_t seed);
/* particles cmag_dambreak3d_scene creates for the given sizes */
int cmag_dambreak3d_particle_count(const uint32_t fluid_size[3], const uint32_t tank_cells[3],
                                   uint32_t layers, uint32_t *out);

/* One time step (update/Update: fluidSystem.cpp:257-319,
 * poiseuilleFlowSystem.cpp:212-270, PeristalsisSystem.cpp:320-407). */
int cmag_system_update(cmag_system *s);
/* One time step of length dt: sets the parameter block's delta_time to dt (it
 * stays for later update() calls, as the reference's params.dt does,
 * fluidSystem.cpp:257,268) and steps.  A dt that differs from the previous one
 * re-captures the step's CUDA graph on this call. */
int cmag_system_update_dt(cmag_system *s, float dt);
/* Run `steps` time steps back to back (replayed as one captured CUDA graph per
 * step when graphs are enabled). */
int cmag_system_update_n(cmag_system *s, uint32_t steps);

/* Run `steps` steps between two CUDA events recorded on the instance's stream,
 * synchronize, and return the elapsed device time in milliseconds (benchmarks). */
int cmag_system_timed_update(cmag_system *s, uint32_t steps, float *ms_out);

/* Stage-by-stage execution for parity tests: run the stages of one step up to
 * and including `last_stage` without advancing time (CMAG_STAGE_INTEGRATE runs
 * a full step and does advance time). */
enum cmag_stage {
    CMAG_STAGE_HASH = 0,
    CMAG_STAGE_SORT = 1,
    CMAG_STAGE_REORDER = 2,
    CMAG_STAGE_DENSITY = 3,
    CMAG_STAGE_FORCE = 4,
    CMAG_STAGE_INTEGRATE = 5
};
int cmag_system_run_stages(cmag_system *s, int32_t last_stage);

/* setArray (fluidSystem.cpp:321-355): copy `count` float4 elements starting at
 * element `start` from host memory.  getArray is its inverse. */
int cmag_system_set_array(cmag_system *s, int32_t array, const float *host, uint32_t start,
                          uint32_t count);
int cmag_system_get_array(cmag_system *s, int32_t array, float *host, uint32_t start,
                          uint32_t count);
int cmag_system_get_uint_array(cmag_system *s, int32_t array, uint32_t *host, uint32_t start,
                               uint32_t count);
/* Several whole float4 arrays (num_particles x 4 floats each) in one call: host[k]
 * is array arrays[k]; one copy per array and one synchronisation for all (at most
 * 8 arrays).  No reference counterpart (its setArray moves one array per call,
 * fluidSystem.cpp:321-355, and reading goes through getCuda* pointers). */
int cmag_system_set_arrays(cmag_system *s, uint32_t count, const int32_t *arrays, const float *const *host);
int cmag_system_get_arrays(cmag_system *s, uint32_t count, const int32_t *arrays, float *const *host);
/* Borrowed device pointer of an array (getCudaPosVBO, getCudaMeasures, ...);
 * valid until destroy.  NULL for unknown arrays. */
void *cmag_system_device_array(cmag_system *s, int32_t array);

int cmag_system_num_particles(const cmag_system *s, uint32_t *out);
int cmag_system_num_grid_cells(const cmag_system *s, uint64_t *out);
int cmag_system_elapsed_time(const cmag_system *s, float *out);
int cmag_system_get_params(const cmag_system *s, cmag_sph_params *out);
/* Replace the parameter block (system kind and grid must not change). */
int cmag_system_set_params(cmag_system *s, const cmag_sph_params *p);

/* DamBreakSystem::changeRightBoundary / removeRightBoundary
 * (fluidSystem.cpp:222-255). */
int cmag_dambreak_change_right_boundary(cmag_system *s);
int cmag_dambreak_remove_right_boundary(cmag_system *s);
/* PoiseuilleFlowSystem::changeGravity (poiseuilleFlowSystem.cpp:207-210). */
int cmag_poiseuille_change_gravity(cmag_system *s);
/* Peristalsis host-side phase state: current wave height, relax time left,
 * time shift and the boundary-configuration flag (PeristalsisSystem.cpp:330-343). */
int cmag_peristalsis_phase(const cmag_system *s, float *current_wave_height,
                           float *time_relax, float *time_shift, int32_t *is_boundary_configuration);
/* Restore the host-side time state (checkpoint/resume; no reference counterpart:
 * the reference keeps elapsedTime and the phase private). */
int cmag_system_set_elapsed_time(cmag_system *s, float elapsed);
int cmag_peristalsis_set_phase(cmag_system *s, float current_wave_height, float time_relax,
                               float time_shift, int32_t is_boundary_configuration);

/* Device reductions over the fluid particles (DamBreak type CMAG_FLUID, the other
 * families type 0), replacing the Report harnesses' host-side sorts and loops:
 * the surge front and column height (XFrontTest.h:75-86, YFrontTest.h:79-90) are
 * hi[0] and hi[1] of cmag_system_fluid_extent; the per-step averages of density.h
 * (:51-67) and forces.h (:56-82) are cmag_system_fluid_sum / count.
 * fluid_sum accepts any float4 array; sorted-order arrays (MEASURES, SORTED*)
 * take the particle type from the sorted positions, the others from POSITION. */
int cmag_system_fluid_extent(cmag_system *s, float lo[3], float hi[3]);
int cmag_system_fluid_sum(cmag_system *s, int32_t array, double sum[4], uint32_t *count);

/* Use a caller-owned cudaStream_t (NULL = the instance's own stream). */
int cmag_system_set_stream(cmag_system *s, void *cuda_stream);
void *cmag_system_stream(const cmag_system *s);
/* 1: capture each step as a CUDA graph and replay it (default); 0: plain launches. */
int cmag_system_set_graphs(cmag_system *s, int32_t enable);
/* Wait for the instance's stream and report device-side check failures
 * (CMAG_ERR_DEVICE with the cmag_device_error bits in the message). */
int cmag_system_synchronize(cmag_system *s);
int cmag_system_device_error_bits(cmag_system *s, uint32_t *bits);

/* Lanes per particle in the density and force loops (1, 2 or 4; the rows of a
 * particle's cell box are split between its lanes). */
int cmag_system_set_groups(cmag_system *s, int32_t density_lanes, int32_t force_lanes);
int cmag_system_get_groups(const cmag_system *s, int32_t *density_lanes, int32_t *force_lanes);
/* Interaction lists: the density pass records each particle's interacting
 * neighbours (sorted indices, in the order the force loop would visit them) and
 * the force pass reads them instead of walking the cells again; the forces are
 * bit-identical to the one-lane walk.  Memory: num_particles x cap x 4 bytes (cap
 * about 1.5 times the lattice neighbour count + 32; enable > 1 sets cap instead;
 * a particle with more neighbours walks the cells).  Fewer than 2^26 particles. */
int cmag_system_set_neighbor_lists(cmag_system *s, int32_t enable);
int cmag_system_get_neighbor_lists(const cmag_system *s, int32_t *enabled, uint32_t *cap);
/* DamBreak systems: the density of a non-fluid particle with no fluid particle in
 * its searched cell box is kept over steps and reused (its walk would visit the
 * same non-fluid particles in the same order, so the reused value has the bits
 * the walk would give).  A non-fluid particle that moves or changes type, and any
 * change of parameters, lanes or lists, starts over.  On by default for DamBreak
 * (memory: num_particles x 32 bytes + 4 bytes per 4x4x4 cells; an instance whose
 * creation could not have that memory is made without it); other families have
 * nothing to keep.  enable = 1 without kept wall densities: CMAG_ERR_STATE. */
int cmag_system_set_wall_cache(cmag_system *s, int32_t enable);
int cmag_system_get_wall_cache(const cmag_system *s, int32_t *enabled);
/* Neighbour lists kept over several steps.  No counterpart in the reference,
 * which hashes, sorts and walks the 7^3 neighbour cells on every step
 * (fluidSystem.cpp:257-319).  skin > 0 (in particle spacings 2r, at most 4):
 * a rebuild step hashes and sorts as the reference does and records, for every
 * particle, all other particles within 2h + skin; the following steps gather the
 * current positions in that order and sum density and forces over the lists,
 * testing q < 2 per pair, until some particle has moved more than skin/2 since
 * the rebuild (checked on the device by integration), which makes the next step
 * a rebuild.  Every pair within 2h is therefore visited, as the reference's
 * walk does, in another summation order (results within FP32 rounding of it).
 *  - Between rebuilds the sorted-order arrays (HASH, INDEX, CELLSTART/END,
 *    CELLOFFSET, SORTEDPOSITION, SORTEDVELOCITY, MEASURES) keep the order of
 *    the last rebuild; SORTEDPOSITION/SORTEDVELOCITY hold the step's positions
 *    and leap-frog velocities in that order.  skin 0 restores the reference's
 *    per-step sort.
 *  - Needs a cut-off on every interaction (DamBreak: lj_cutoff = 1).  Setting
 *    arrays or parameters forces a rebuild; a list that outgrows its room makes
 *    every step a rebuild until it fits again.  Not used while a learned closure
 *    is attached (its features walk this step's cells).
 *  - Memory: the interaction lists at radius 2h + skin plus 16 bytes per particle.
 * get_verlet: the skin (0: off) and the number of rebuilds so far. */
int cmag_system_set_verlet(cmag_system *s, float skin);
int cmag_system_get_verlet(cmag_system *s, float *skin, uint32_t *rebuilds);
/* Autotune: on the current state, time the density and force kernels for every
 * lane count and with interaction lists (`reps` launches each) and keep the
 * fastest.  Both kernels are recomputed from scratch every step; the choice
 * changes only the summation order of the lanes' partial sums. */
int cmag_system_autotune(cmag_system *s, int32_t reps);

/* Per-stage timing: when enabled, every step records CUDA events around each
 * stage on the instance's stream; read back the accumulated milliseconds per stage
 * (6 entries, enum cmag_stage order) and the number of timed steps. */
int cmag_system_set_stage_timing(cmag_system *s, int32_t enable);
int cmag_system_stage_times(cmag_system *s, float ms_out[6], uint32_t *steps_out);

const char *cmag_system_last_error(const cmag_system *s);
/* thread-local message of the last failed call that had no handle */
const char *cmag_last_error(void);

/* ---- launcher-level entry points ---------------------------------------- */
/* sortParticles (fluidSystem.cu:94-99, poiseuilleFlowSystem.cu:103-108,
 * PeristalsisSystem.cu:116-121): stable ascending sort of the (hash, index) pairs
 * in place on the device, keys below 2^key_bits.  Replaces thrust::sort_by_key
 * with a onesweep LSD radix sort (8-bit digits).  Scratch memory is allocated on
 * the first call and cached per device (grown when a larger n arrives). */
int cmag_sort_particles(uint32_t *d_hash, uint32_t *d_index, uint32_t n, uint32_t key_bits,
                        void *cuda_stream);

/* The same stable sort without allocating anything, for callers that cannot call
 * cudaMalloc where they sort: latency-critical loops where an allocation would
 * stall the device, and hosts whose device memory all comes from their own pool
 * (a framework's caching allocator, a runtime with a fixed memory budget).  No
 * counterpart in the reference (its thrust::sort_by_key allocates temporaries).
 *  - Works on at most 1,048,576 pairs; larger n returns CMAG_ERR_INVALID.
 *  - Its workspace (about 9.3 MB: look-back status and alternate key/value
 *    buffers) is a fixed device array inside this library, held by every GPU that
 *    loads the library until the process exits; no cudaMalloc/cudaFree is called.
 *  - The first call in each CUDA context (normally once per device, in its
 *    primary context) looks up that array's device address
 *    (cudaGetSymbolAddress) with the context current and caches it under the
 *    context; make that first call before any stream capture.
 *  - Every call shares the one array: calls whose work overlaps on the GPU (other
 *    streams, other threads) race and must be serialised by the caller.
 *  - It waits for the stream before returning, to report a failed device-side
 *    check (look-back timeout, out-of-range scatter); messages:
 *    cmag_sort_particles_noalloc_error(). */
int cmag_sort_particles_noalloc(uint32_t *d_hash, uint32_t *d_index, uint32_t n,
                                uint32_t key_bits, void *cuda_stream);
const char *cmag_sort_particles_noalloc_error(void);

/* Testing only (no reference counterpart; the reference's sort has no bounded
 * waits).  Number of polls after which a look-back wait of the radix sort
 * (cmag_sort_particles, cmag_sort_particles_noalloc) gives up on the current
 * device and records CMAG_DEVERR_LOOKBACK_TIMEOUT; negative restores the default
 * (4,194,304).  0 makes every wait that finds its predecessor tile unpublished
 * give up at once, so tests can reach the failure path without a real stall: the
 * sort then returns CMAG_ERR_DEVICE and its output is wrong but stays in bounds. */
int cmag_testing_set_sort_spin_limit(int32_t polls);

/* ---- headless colours and point view ----------------------------------- */
/* The Demo programs' colour buffers without OpenGL: per particle (original
 * order) the RGBA values the reference writes into its colour VBO -- DamBreak
 * colorRamp by index (fluidSystem.cpp:97-114, 165-181), Poiseuille likewise
 * (poiseuilleFlowSystem.cpp:152-166), Peristalsis Coloring by type and x
 * (PeristalsisSystem.cpp:409-442, values 0/255).  rgba: host, num_particles x 4. */
int cmag_system_colors(cmag_system *s, float *rgba);
/* The point view as a binary PPM image: particles projected on x-y over the
 * grid's extent, each pixel coloured by the last particle (highest index) in it.
 * height 0: from the grid's aspect ratio. */
int cmag_system_render_ppm(cmag_system *s, const char *path, uint32_t width, uint32_t height);

/* ---- batches of independent scenes -------------------------------------- */
/* No counterpart in the reference, which runs one scene per process (its kernels
 * read one global __constant__ parameter block per library: fluidSystem.cu:17-19,
 * poiseuilleFlowSystem.cu:19-21, PeristalsisSystem.cu:21-23).  A batch advances
 * S scenes of any families and sizes with one set of launches per step (one hash,
 * scan, sort, gather and integration; one density and one force launch per launch
 * group), captured as one CUDA graph.  Each scene follows exactly the arithmetic
 * of a cmag_system with the same parameters and lanes, so its trajectory equals
 * that system's bit for bit.
 *  - Scenes are addressed by their index in the create call.  Particle arrays
 *    are scene-local in set/get_array; the device arrays hold scene s at
 *    [first, first + count) (cmag_batch_scene_range).
 *  - A 2-D scene with zero z gravity and more than cell_count z layers is
 *    planar: its particles must share one z and have no z velocity (set_array
 *    refuses other data); its cell table covers that z layer only.
 *  - Launch groups: scenes of one family, search shape and factor-4 size class;
 *    each has its own lanes per particle (cmag_batch_autotune). */
typedef struct cmag_batch cmag_batch;

typedef struct cmag_batch_group {
    int32_t system;          /* enum cmag_system_kind                     */
    int32_t planar;          /* 1: single z layer search                  */
    int32_t trim;            /* 1: rows trimmed to the support sphere     */
    uint32_t size_bucket;    /* scenes with 2^(2k-1) < n <= 2^(2k+1)       */
    uint32_t scenes;
    uint32_t particles;
    int32_t density_lanes;
    int32_t force_lanes;
    int32_t lists;           /* 1: interaction lists (one lane per particle) */
} cmag_batch_group;

int cmag_batch_create(const cmag_sph_params *params, const uint32_t *counts, uint32_t scenes,
                      cmag_batch **out);
int cmag_batch_destroy(cmag_batch *b);
int cmag_batch_num_scenes(const cmag_batch *b, uint32_t *out);
int cmag_batch_num_particles(const cmag_batch *b, uint32_t *out);
int cmag_batch_scene_range(cmag_batch *b, uint32_t scene, uint32_t *first, uint32_t *count);
/* every scene's / one scene's reference initial state (cmag_system_reset) */
int cmag_batch_reset(cmag_batch *b);
int cmag_batch_reset_scene(cmag_batch *b, uint32_t scene);
int cmag_batch_set_array(cmag_batch *b, uint32_t scene, int32_t array, const float *host,
                         uint32_t start, uint32_t count);
int cmag_batch_get_array(cmag_batch *b, uint32_t scene, int32_t array, float *host,
                         uint32_t start, uint32_t count);
/* Every scene's float4 array in one call: host holds the scenes one after another
 * in scene order (cmag_batch_num_particles(b) x 4 floats); one copy per scene and
 * one synchronisation.  A planar 2-D scene must keep one z (positions) and no z
 * velocity: checked on the device after the transfer, so on that error the array
 * holds the new data and should be set again.  No reference counterpart (the
 * reference has one scene per process). */
int cmag_batch_set_array_all(cmag_batch *b, int32_t array, const float *host);
int cmag_batch_get_array_all(cmag_batch *b, int32_t array, float *host);
/* scene-local: HASH = the scene's reference hash, INDEX = scene-local original
 * index, CELLOFFSET = offsets over the scene's table (scan_cells + 1 entries),
 * CELLSTART / CELLEND = the reference arrays over the scene's grid */
int cmag_batch_get_uint_array(cmag_batch *b, uint32_t scene, int32_t array, uint32_t *host,
                              uint32_t start, uint32_t count);
/* whole-batch device array (NULL for arrays the batch does not hold) */
void *cmag_batch_device_array(cmag_batch *b, int32_t array);
int cmag_batch_get_params(cmag_batch *b, uint32_t scene, cmag_sph_params *out);
/* family, grid size and search shape are fixed at creation */
int cmag_batch_set_params(cmag_batch *b, uint32_t scene, const cmag_sph_params *p);
int cmag_batch_update(cmag_batch *b);
int cmag_batch_update_n(cmag_batch *b, uint32_t steps);
int cmag_batch_timed_update(cmag_batch *b, uint32_t steps, float *ms_out);
int cmag_batch_run_stages(cmag_batch *b, int32_t last_stage);
int cmag_batch_elapsed_time(cmag_batch *b, uint32_t scene, float *out);
int cmag_batch_dambreak_change_right_boundary(cmag_batch *b, uint32_t scene);
int cmag_batch_dambreak_remove_right_boundary(cmag_batch *b, uint32_t scene);
int cmag_batch_poiseuille_change_gravity(cmag_batch *b, uint32_t scene);
/* fluid extents of every scene from one reduction: lo/hi hold scenes*3 floats */
int cmag_batch_fluid_extents(cmag_batch *b, float *lo, float *hi);
int cmag_batch_set_stream(cmag_batch *b, void *cuda_stream);
void *cmag_batch_stream(const cmag_batch *b);
/* graphs on/off; steps_per_graph (1..1024) steps are captured in one graph */
int cmag_batch_set_graphs(cmag_batch *b, int32_t enable, uint32_t steps_per_graph);
int cmag_batch_synchronize(cmag_batch *b);
int cmag_batch_device_error_bits(cmag_batch *b, uint32_t *bits);
int cmag_batch_num_groups(const cmag_batch *b, uint32_t *out);
int cmag_batch_group_info(cmag_batch *b, uint32_t group, cmag_batch_group *out);
int cmag_batch_scene_group(cmag_batch *b, uint32_t scene, uint32_t *group);
int cmag_batch_set_group_lanes(cmag_batch *b, uint32_t group, int32_t density_lanes,
                               int32_t force_lanes);
/* Interaction lists for one launch group (enable 1) or the cell walk (0): the
 * density pass records each particle's neighbours and the force pass reads
 * them; one lane per particle, the same results as the one-lane walk.  No
 * reference counterpart (the reference walks the cells in both passes). */
int cmag_batch_set_group_lists(cmag_batch *b, uint32_t group, int32_t enable);
/* per launch group, the fastest lanes per particle for density and force */
int cmag_batch_autotune(cmag_batch *b, int32_t reps);
/* Kept densities of dam-break walls in every DamBreak scene of the batch, as
 * cmag_system_set_wall_cache (same bits either way; on by default when the batch
 * holds a dam-break scene, which enable = 1 requires). */
int cmag_batch_set_wall_cache(cmag_batch *b, int32_t enable);
int cmag_batch_get_wall_cache(const cmag_batch *b, int32_t *enabled);
int cmag_batch_set_stage_timing(cmag_batch *b, int32_t enable);
int cmag_batch_stage_times(cmag_batch *b, float ms_out[6], uint32_t *steps_out);
const char *cmag_batch_last_error(const cmag_batch *b);

/* ---- learned closure ----------------------------------------------------- */
/* No counterpart in the reference.  A 16-64-64-64-3 SiLU network that adds a
 * learned correction to the pressure + viscous + wall acceleration of every fluid
 * particle of a (coarse) DamBreak scene, right after the force stage.  BF16
 * parameters and activations, FP32 accumulation; trained on the GPU by the
 * library's own forward/backward kernels and Adam (FP32 master copy).
 *  - Parameters: cmag_closure_param_count() floats, order W1[64][16] b1[64]
 *    W2[64][64] b2[64] W3[64][64] b3[64] W4[3][64] b4[3] (W[out][in]).
 *  - Features (16 per fluid particle, raw): cmag_system_closure_features writes
 *    them for the state of the last run_stages(CMAG_STAGE_FORCE) into a device
 *    array of num_particles x 16 floats (original order; wall rows untouched).
 *    The network sees bf16((f - mean) * inv_std); the correction is out_scale * y.
 *  - Device arrays (features n x 16, targets / outputs n x 3, row-major floats)
 *    are the caller's; stream NULL means the closure's own stream. */
typedef struct cmag_closure cmag_closure;

size_t cmag_closure_param_count(void);
/* params: FP32 initial parameters, or NULL for zeros */
int cmag_closure_create(const float *params, cmag_closure **out);
int cmag_closure_destroy(cmag_closure *c);
int cmag_closure_set_params(cmag_closure *c, const float *params);
int cmag_closure_get_params(cmag_closure *c, float *params);
/* the BF16 values the kernels use, widened to float */
int cmag_closure_get_bf16_params(cmag_closure *c, float *params);
int cmag_closure_set_normalization(cmag_closure *c, const float mean[16], const float inv_std[16],
                                   float out_scale);
int cmag_closure_get_normalization(cmag_closure *c, float mean[16], float inv_std[16],
                                   float *out_scale);
/* inside a step the correction is out_scale * clamp(y, -limit, limit) per
 * component (default: no limit); cmag_closure_forward is not clamped */
int cmag_closure_set_output_limit(cmag_closure *c, float limit);
/* network outputs y (unscaled) for n feature rows */
int cmag_closure_forward(cmag_closure *c, const float *d_features, uint32_t n, float *d_out,
                         void *stream);
/* loss 0.5/n sum |y - t|^2 and its gradient with respect to the (BF16) parameters,
 * copied to the host (grad_out: param_count floats); parameters unchanged */
int cmag_closure_gradient(cmag_closure *c, const float *d_features, const float *d_targets,
                          uint32_t n, float *grad_out, float *loss_out, void *stream);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) on the loss over the n rows; the loss
 * before the step is returned when loss_out is given (that call waits) */
int cmag_closure_train_step(cmag_closure *c, const float *d_features, const float *d_targets,
                            uint32_t n, float lr, float *loss_out, void *stream);
int cmag_closure_reset_optimizer(cmag_closure *c);
int cmag_closure_synchronize(cmag_closure *c);
const char *cmag_closure_last_error(const cmag_closure *c);
/* attach (or with NULL detach) a closure to a DamBreak system: every later step
 * adds its correction after the force stage; the closure must outlive the
 * attachment */
int cmag_system_set_closure(cmag_system *s, cmag_closure *c);
int cmag_system_closure_features(cmag_system *s, float *d_features);
/* Shepard-normalised SPH interpolation of a float4 array (POSITION, VELOCITY,
 * ACCELERATION or VELOCITYLEAPFROG) over the fluid particles of a DamBreak system,
 * at n points (device, n x 4 floats; .w ignored): d_out (device, n x 4) gets
 * sum V_j W a_j / sum V_j W in xyz and sum V_j W in w (0: no fluid in reach).
 * Uses the sorted state and densities of the last run_stages (>= DENSITY). */
int cmag_system_interpolate(cmag_system *s, int32_t array, const float *d_points, uint32_t n,
                            float *d_out);

/* Library version string. */
const char *cmag_version(void);
/* sizeof(cmag_sph_params) as compiled into the library (for FFI layout checks). */
size_t cmag_sph_params_size(void);

#ifdef __cplusplus
}
#endif

#endif /* CMAG_SPH_H */
