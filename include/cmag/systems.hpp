// cmag/systems.hpp -- the reference's solver classes over the C ABI.
//
// Drop-in replacements, same names, constructors and methods, for
//   DamBreakSystem        DamBreak.Core/fluidSystem.h:6-113
//   PoiseuilleFlowSystem  Poiseuille.Core/poiseuilleFlowSystem.h:6-112
//   PeristalsisSystem     Peristalsis.Core/PeristalsisSystem.h:6-132
// Header-only; link libcmag_sph.so.  Differences from the reference: failures
// throw cmag::Error instead of printing and calling exit(); any number of
// instances may live in one process; bUseOpenGL is ignored (no VBOs: the position
// array is a plain device buffer and the VBO ids read 0).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <vector_functions.h>
#include <vector_types.h>

#include "../cmag_sph.h"

namespace cmag {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const cmag_system *s = nullptr)
{
    if (rc != CMAG_OK) throw Error(rc, s ? cmag_system_last_error(s) : cmag_last_error());
}

inline const uint32_t *u3p(const uint3 &v, uint32_t (&a)[3])
{
    a[0] = v.x; a[1] = v.y; a[2] = v.z;
    return a;
}

// Shared owner of one solver instance.
class SystemBase {
public:
    SystemBase(const SystemBase &) = delete;
    SystemBase &operator=(const SystemBase &) = delete;
    ~SystemBase() { cmag_system_destroy(h_); }

    int getNumParticles() const { return (int)n_; }
    cmag_system *handle() const { return h_; }
    cmag_sph_params params() const
    {
        cmag_sph_params p;
        check(cmag_system_get_params(h_, &p), h_);
        return p;
    }
    void setParams(const cmag_sph_params &p) { check(cmag_system_set_params(h_, &p), h_); }
    void getArray(int array, float *data, int start, int count) const
    {
        check(cmag_system_get_array(h_, array, data, (uint32_t)start, (uint32_t)count), h_);
    }
    // several whole float4 arrays with one synchronisation (arrays[k] <-> data[k])
    void setArrays(uint32_t count, const int32_t *arrays, const float *const *data)
    {
        check(cmag_system_set_arrays(h_, count, arrays, data), h_);
    }
    void getArrays(uint32_t count, const int32_t *arrays, float *const *data) const
    {
        check(cmag_system_get_arrays(h_, count, arrays, data), h_);
    }
    void updateSteps(uint32_t steps) { check(cmag_system_update_n(h_, steps), h_); }
    void synchronize() { check(cmag_system_synchronize(h_), h_); }
    // neighbour-loop choices (none changes a result bit beyond the lanes' summation order)
    void autotune(int reps = 3) { check(cmag_system_autotune(h_, reps), h_); }
    void setNeighborLists(bool enable) { check(cmag_system_set_neighbor_lists(h_, enable ? 1 : 0), h_); }
    void setGroups(int densityLanes, int forceLanes) { check(cmag_system_set_groups(h_, densityLanes, forceLanes), h_); }
    // dam breaks: kept wall densities (on by default; same bits either way)
    void setWallCache(bool enable) { check(cmag_system_set_wall_cache(h_, enable ? 1 : 0), h_); }
    bool wallCache() const
    {
        int32_t e = 0;
        check(cmag_system_get_wall_cache(h_, &e), h_);
        return e != 0;
    }
    // max x, y, z of a fluid particle (device reduction)
    float3 fluidMax() const
    {
        float lo[3], hi[3];
        check(cmag_system_fluid_extent(h_, lo, hi), h_);
        return make_float3(hi[0], hi[1], hi[2]);
    }
    // average of a float4 array over the fluid particles (device reduction)
    float4 fluidAverage(int array, uint32_t divisor = 0) const
    {
        double s[4];
        uint32_t c = 0;
        check(cmag_system_fluid_sum(h_, array, s, &c), h_);
        const double d = divisor ? divisor : (c ? c : 1);
        return make_float4((float)(s[0] / d), (float)(s[1] / d), (float)(s[2] / d), (float)(s[3] / d));
    }

    float getHalfWorldXSize() const { auto p = params(); return p.grid_size[0] * p.particle_radius; }
    float getHalfWorldYSize() const { auto p = params(); return p.grid_size[1] * p.particle_radius; }
    float getHalfWorldZSize() const { auto p = params(); return p.grid_size[2] * p.particle_radius; }
    uint3 getGridSize() const { auto p = params(); return make_uint3(p.grid_size[0], p.grid_size[1], p.grid_size[2]); }
    float3 getWorldOrigin() const { auto p = params(); return make_float3(p.world_origin[0], p.world_origin[1], p.world_origin[2]); }
    float3 getCellSize() const { auto p = params(); return make_float3(p.cell_size[0], p.cell_size[1], p.cell_size[2]); }
    float3 getGravity() const { auto p = params(); return make_float3(p.gravity[0], p.gravity[1], p.gravity[2]); }

    unsigned int getCurrentReadBuffer() const { return 0; }
    unsigned int getColorBuffer() const { return 0; }
    void *getCudaPosVBO() const { return cmag_system_device_array(h_, CMAG_POSITION); }
    void *getCudaVelVBO() const { return cmag_system_device_array(h_, CMAG_VELOCITY); }
    void *getCudaColorVBO() const { return nullptr; }
    void *getCudaHash() const { return cmag_system_device_array(h_, CMAG_HASH); }
    void *getCudaIndex() const { return cmag_system_device_array(h_, CMAG_INDEX); }
    void *getCudaSortedPosition() const { return cmag_system_device_array(h_, CMAG_SORTEDPOSITION); }
    void *getLeapFrogVelocity() const { return cmag_system_device_array(h_, CMAG_VELOCITYLEAPFROG); }

protected:
    explicit SystemBase(const cmag_sph_params &p, uint32_t n = 0)
    {
        if (n == 0) check(cmag_reference_particle_count(&p, &n));
        check(cmag_system_create(&p, n, &h_));
        n_ = n;
    }
    void setRaw(int array, const float *data, int start, int count)
    {
        check(cmag_system_set_array(h_, array, data, (uint32_t)start, (uint32_t)count), h_);
    }
    float elapsed() const
    {
        float t;
        check(cmag_system_elapsed_time(h_, &t), h_);
        return t;
    }

    cmag_system *h_ = nullptr;
    uint32_t n_ = 0;
};

inline cmag_sph_params dambreak_params(uint3 fs, int off, uint3 gs, float r)
{
    cmag_sph_params p;
    uint32_t a[3], b[3];
    check(cmag_dambreak_default_params(u3p(fs, a), off, u3p(gs, b), r, &p));
    return p;
}

inline cmag_sph_params poiseuille_params(uint3 fs, int off, uint3 gs, float r)
{
    cmag_sph_params p;
    uint32_t a[3], b[3];
    check(cmag_poiseuille_default_params(u3p(fs, a), off, u3p(gs, b), r, &p));
    return p;
}

inline cmag_sph_params peristalsis_params(float dt, uint3 fs, float amplitude, float wave_speed,
                                          float soundspeed, float3 g, int off, uint3 gs, float r)
{
    cmag_sph_params p;
    uint32_t a[3], b[3];
    const float gv[3] = {g.x, g.y, g.z};
    check(cmag_peristalsis_default_params(dt, u3p(fs, a), amplitude, wave_speed, soundspeed, gv,
                                          off, u3p(gs, b), r, &p));
    return p;
}

}  // namespace cmag

class DamBreakSystem : public cmag::SystemBase {
public:
    DamBreakSystem(uint3 fluidParticlesSize, int boundaryOffset, uint3 gridSize, float particleRadius,
                   bool bUseOpenGL)
        : SystemBase(cmag::dambreak_params(fluidParticlesSize, boundaryOffset, gridSize, particleRadius))
    {
        (void)bUseOpenGL;
    }
    explicit DamBreakSystem(const cmag_sph_params &p, uint32_t numParticles = 0) : SystemBase(p, numParticles) {}

    // fluidSystem.h:17-24
    enum ParticleArray { POSITION, VELOCITY, MEASURES, ACCELERATION, VELOCITYLEAPFROG };

    void update() { cmag::check(cmag_system_update(h_), h_); }
    // one step of length dt (kept in the parameter block for later update() calls)
    void update(float dt) { cmag::check(cmag_system_update_dt(h_, dt), h_); }
    void reset() { cmag::check(cmag_system_reset(h_), h_); }
    void setArray(ParticleArray array, const float *data, int start, int count) { setRaw((int)array, data, start, count); }
    float getElapsedTime() const { return elapsed(); }
    void *getCudaMeasures() const { return cmag_system_device_array(h_, CMAG_MEASURES); }
    void *getCudaAcceleration() const { return cmag_system_device_array(h_, CMAG_ACCELERATION); }
    void changeRightBoundary() { cmag::check(cmag_dambreak_change_right_boundary(h_), h_); }
    void removeRightBoundary() { cmag::check(cmag_dambreak_remove_right_boundary(h_), h_); }
    float getParticleRadius() const { return params().particle_radius; }
};

class PoiseuilleFlowSystem : public cmag::SystemBase {
public:
    PoiseuilleFlowSystem(uint3 fluidParticlesSize, int boundaryOffset, uint3 gridSize,
                         float particleRadius, bool bUseOpenGL)
        : SystemBase(cmag::poiseuille_params(fluidParticlesSize, boundaryOffset, gridSize, particleRadius))
    {
        (void)bUseOpenGL;
    }
    explicit PoiseuilleFlowSystem(const cmag_sph_params &p, uint32_t numParticles = 0) : SystemBase(p, numParticles) {}

    // poiseuilleFlowSystem.h:17-24
    enum ParticleArray { POSITION, VELOCITY, MEASURES, ACCELERATION, VELOCITYLEAPFROG };

    void update() { cmag::check(cmag_system_update(h_), h_); }
    // one step of length dt (kept in the parameter block for later update() calls)
    void update(float dt) { cmag::check(cmag_system_update_dt(h_, dt), h_); }
    void reset() { cmag::check(cmag_system_reset(h_), h_); }
    void setArray(ParticleArray array, const float *data, int start, int count) { setRaw((int)array, data, start, count); }
    float getElapsedTime() const { return elapsed(); }
    void *getCudaMeasures() const { return cmag_system_device_array(h_, CMAG_MEASURES); }
    void *getCudaAcceleration() const { return cmag_system_device_array(h_, CMAG_ACCELERATION); }
    void changeGravity() { cmag::check(cmag_poiseuille_change_gravity(h_), h_); }
    float getParticleRadius() const { return params().particle_radius; }
};

class PeristalsisSystem : public cmag::SystemBase {
public:
    PeristalsisSystem(float deltaTime, uint3 fluid_size, float amplitude, float wave_speed,
                      float soundspeed, float3 gravity, int boundaryOffset, uint3 gridSize,
                      float radius, bool bUseOpenGL)
        : SystemBase(cmag::peristalsis_params(deltaTime, fluid_size, amplitude, wave_speed, soundspeed,
                                              gravity, boundaryOffset, gridSize, radius))
    {
        (void)bUseOpenGL;
    }
    explicit PeristalsisSystem(const cmag_sph_params &p, uint32_t numParticles = 0) : SystemBase(p, numParticles) {}

    // PeristalsisSystem.h:22-31 (its own order)
    enum ParticleArray { POSITION, PREDICTEDPOSITION, VELOCITY, MEASURES, VISCOUSFORCE, PRESSUREFORCE, VELOCITYLEAPFROG };

    void Update() { cmag::check(cmag_system_update(h_), h_); }
    // one step of length dt (kept in the parameter block for later Update() calls)
    void Update(float dt) { cmag::check(cmag_system_update_dt(h_, dt), h_); }
    void Reset() { cmag::check(cmag_system_reset(h_), h_); }
    void setArray(ParticleArray array, const float *data, int start, int count)
    {
        static const int map[] = {CMAG_POSITION, CMAG_PREDICTEDPOSITION, CMAG_VELOCITY, CMAG_MEASURES,
                                  CMAG_VISCOUSFORCE, CMAG_PRESSUREFORCE, CMAG_VELOCITYLEAPFROG};
        setRaw(map[(int)array], data, start, count);
    }
    float GetElapsedTime() const { return elapsed(); }
    float getradius() const { return params().particle_radius; }
    void *getSortedVelocity() const { return cmag_system_device_array(h_, CMAG_SORTEDVELOCITY); }
    void *getMeasures() const { return cmag_system_device_array(h_, CMAG_MEASURES); }
    void *viscous_force() const { return cmag_system_device_array(h_, CMAG_VISCOUSFORCE); }
    void *pressure_force() const { return cmag_system_device_array(h_, CMAG_PRESSUREFORCE); }
    void *getPredictedPos() const { return cmag_system_device_array(h_, CMAG_PREDICTEDPOSITION); }
};

namespace cmag {

// Many independent scenes advanced together (cmag_batch_*); no reference
// counterpart.  Scene indices are the positions in the constructor's vectors.
class Batch {
public:
    Batch(const std::vector<cmag_sph_params> &params, const std::vector<uint32_t> &counts)
    {
        if (params.size() != counts.size()) throw Error(CMAG_ERR_INVALID, "one particle count per scene");
        check(cmag_batch_create(params.data(), counts.data(), (uint32_t)params.size(), &h_));
    }
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;
    ~Batch() { cmag_batch_destroy(h_); }

    cmag_batch *handle() const { return h_; }
    uint32_t numScenes() const { uint32_t v = 0; chk(cmag_batch_num_scenes(h_, &v)); return v; }
    uint32_t numParticles() const { uint32_t v = 0; chk(cmag_batch_num_particles(h_, &v)); return v; }
    std::pair<uint32_t, uint32_t> sceneRange(uint32_t scene) const
    {
        uint32_t a = 0, n = 0;
        chk(cmag_batch_scene_range(h_, scene, &a, &n));
        return {a, n};
    }
    void reset() { chk(cmag_batch_reset(h_)); }
    void reset(uint32_t scene) { chk(cmag_batch_reset_scene(h_, scene)); }
    void update() { chk(cmag_batch_update(h_)); }
    void update(uint32_t steps) { chk(cmag_batch_update_n(h_, steps)); }
    void setArray(uint32_t scene, int array, const float *data, int start, int count)
    {
        chk(cmag_batch_set_array(h_, scene, array, data, (uint32_t)start, (uint32_t)count));
    }
    void getArray(uint32_t scene, int array, float *data, int start, int count) const
    {
        chk(cmag_batch_get_array(h_, scene, array, data, (uint32_t)start, (uint32_t)count));
    }
    // every scene's rows at once, scenes one after another in scene order
    void setArrayAll(int array, const float *data) { chk(cmag_batch_set_array_all(h_, array, data)); }
    void getArrayAll(int array, float *data) const { chk(cmag_batch_get_array_all(h_, array, data)); }
    void *deviceArray(int array) const { return cmag_batch_device_array(h_, array); }
    float elapsedTime(uint32_t scene) const { float t = 0; chk(cmag_batch_elapsed_time(h_, scene, &t)); return t; }
    void removeRightBoundary(uint32_t scene) { chk(cmag_batch_dambreak_remove_right_boundary(h_, scene)); }
    void changeRightBoundary(uint32_t scene) { chk(cmag_batch_dambreak_change_right_boundary(h_, scene)); }
    void changeGravity(uint32_t scene) { chk(cmag_batch_poiseuille_change_gravity(h_, scene)); }
    // fluid bounding boxes of every scene (scenes * 3 floats each)
    void fluidExtents(float *lo, float *hi) const { chk(cmag_batch_fluid_extents(h_, lo, hi)); }
    void setGraphs(bool enable, uint32_t stepsPerGraph = 1) { chk(cmag_batch_set_graphs(h_, enable ? 1 : 0, stepsPerGraph)); }
    void autotune(int reps = 3) { chk(cmag_batch_autotune(h_, reps)); }
    void set_group_lists(uint32_t group, bool enable) { chk(cmag_batch_set_group_lists(h_, group, enable ? 1 : 0)); }
    void setWallCache(bool enable) { chk(cmag_batch_set_wall_cache(h_, enable ? 1 : 0)); }
    void synchronize() { chk(cmag_batch_synchronize(h_)); }

private:
    void chk(int rc) const
    {
        if (rc != CMAG_OK) throw Error(rc, cmag_batch_last_error(h_));
    }
    cmag_batch *h_ = nullptr;
};

}  // namespace cmag
