// Host-side helpers shared by the C-ABI translation units (no device code).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "pbf.h"
#include "pbf_internal.cuh"

namespace pbf {

// Records the text of a CUDA error for pbf_last_error_message and maps it to
// a status code.
int cuda_status(cudaError_t e, const char *where);
void set_error_message(const std::string &msg);

// The reference's constant baking (src/main.cpp:149-168): a value printed
// with std::showpoint at precision 6 and read back as a float literal.
float baked6(double v);

// Derived constants.  `h` is (x_max - x_min) / x_n in float arithmetic, as
// src/main.cpp:164 computes it.
float params_h(const pbf_params &p);
RefConsts make_ref_consts(const pbf_params &p);
PaperConsts make_paper_consts(const pbf_params &p, uint32_t n);
// Scene descriptor of the whole box of `p` (grid origin, cell lengths,
// clamp bounds).  cell_base / particle range are left for the caller.
SceneDesc make_scene(const pbf_params &p);
// Validates a parameter set for a simulation of n particles.
int validate_params(const pbf_params &p, uint32_t n);
uint64_t grid_cells(const pbf_params &p);

// Checks a scene for a batch (grid, cell lengths against the batch's h) and
// returns the batch's solver settings with the scene's box, grid and walls,
// and the scene's cell count.  No capacity check.
int batch_check_scene(const pbf_batch *b, const pbf_params &scene, uint32_t n,
                      pbf_params *merged, uint64_t *cells);
void batch_capacity(const pbf_batch *b, uint32_t *scenes, uint32_t *particles,
                    uint32_t *cells);

// pbf_tuning <-> GatherTuning.  to_gather_tuning returns PBF_ERR_INVALID for
// a shape outside 64/128/256 threads and 4/8 loads in flight.
void to_pbf_tuning(const GatherTuning &g, const double trial_ms[kGatherKinds], pbf_tuning *out);
int to_gather_tuning(const pbf_tuning &t, GatherTuning *out);

// Renders n particles (X: position, .w = |v|; ID: input index of each slot,
// or null when slot = input index) of the box of `prm` into rgb (host).
int render_particles(const float4 *X, const uint32_t *ID, uint32_t n, const pbf_params &prm,
                     const pbf_camera &cam, uint32_t width, uint32_t height, uint8_t *rgb,
                     cudaStream_t st);

}  // namespace pbf
