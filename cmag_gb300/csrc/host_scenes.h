// host_scenes.h -- reference parameter blocks and scene generators (host code).
#pragma once

#include <cstdint>

#include "../../include/cmag_sph.h"

namespace cmag {

void dambreak_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                     cmag_sph_params &p);
void poiseuille_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                       cmag_sph_params &p);
void peristalsis_params(float dt, const uint32_t fs[3], float amplitude, float wave_speed,
                        float soundspeed, const float g[3], int32_t off, const uint32_t gs[3],
                        float r, cmag_sph_params &p);
uint32_t reference_particle_count(const cmag_sph_params &p);
void reference_scene(const cmag_sph_params &p, float *pos, uint32_t n);
float peristalsis_mass_sum(const cmag_sph_params &p, const float *pos, uint32_t n);
uint32_t dambreak3d_count(const uint32_t fs[3], const uint32_t tank[3], uint32_t layers);
void dambreak3d_scene(const cmag_sph_params &p, const uint32_t tank[3], uint32_t layers,
                      float jitter_frac, uint64_t seed, float *pos, uint32_t n);

}  // namespace cmag
