// host_common.h -- host helpers shared by the single-scene solver (system.cu)
// and the batch solver (batch.cu): parameter checks, the device parameter
// block, the planar layout decision and error reporting.
#pragma once

#include <string>

#include "kernels.h"

namespace cmag {

bool is_pow2(uint32_t v);
uint32_t log2u(uint64_t v);

// 0 when p can drive a scene of n particles, else 1 with the reason in why
int validate_params(const cmag_sph_params &p, uint32_t n, std::string &why);

// The cell table a scene's search covers: the whole grid, or one z layer of a
// planar 2-D scene.
struct SceneLayout {
    bool planar = false;
    uint32_t planar_layer = 0;
    uint32_t scan_base = 0, scan_cells = 0;
};

// Kernel parameter block of one scene (table_base and part_base zero).
DevParams make_dev_params(const cmag_sph_params &p, uint32_t n, const SceneLayout &lay);

// z cell of a position, as the hash computes it
int z_cell(const cmag_sph_params &p, float z);

// Whether a scene may search only its own z layer: a 2-D scene whose particles
// share one z, that has no z motion, and whose grid has more than cell_count
// layers (the layer is then reached only with dz = 0 and every other layer is
// empty, so the result equals the full search).
bool planar_allowed(const cmag_sph_params &p, bool z_uniform, bool vz_nonzero);
SceneLayout layout_for(const cmag_sph_params &p, bool planar, float z_value);

// Interaction-list entries per particle: 1.5 times the lattice neighbour count
// inside the support, or inside 2h + skin (skin in particle spacings) for lists
// kept over several steps (every particle of the searched cell box when rows are
// not trimmed), plus 32.  Particles with more walk the cells.
uint32_t list_cap(const cmag_sph_params &p, bool trim, double skin = 0.0);

// thread-local message returned by cmag_last_error
void set_last_error(const std::string &msg);
const std::string &last_error();

}  // namespace cmag
