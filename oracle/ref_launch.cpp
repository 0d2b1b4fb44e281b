/*
 * TEST INFRASTRUCTURE (oracle) -- never linked into the product library.
 *
 * Runs the reference's own live OpenCL kernels (MrMagne/position-based-fluids
 * src/kernels/{predict_positions,init_cells_old,update_cells,compute_scaling,
 * compute_delta,update_predicted,update_velocities,
 * apply_vorticity_and_viscosity,update_positions}.cl), compiled unchanged as
 * C++ through oracle/clshim.hpp, on the host cores.  This file plays the part
 * of an OpenCL runtime plus the reference host:
 *
 *   - constants: derived and printed exactly as src/main.cpp:149-168 does
 *     (std::showpoint, default precision 6, "f" suffix) and parsed back, so
 *     every constant has the value the OpenCL compiler would have seen;
 *   - NDRange: global size ceil(N/32)*32 for the per-particle kernels
 *     (src/Simulation.cpp:138-141) and max(4N, 4C) work-items for
 *     initCellsOld (src/Simulation.cpp:338-340), one call per work-item;
 *   - step order: src/Simulation.cpp:455-576 (predict, initCellsOld,
 *     updateCells, 4 x {computeScaling, computeDelta, updatePredicted},
 *     updateVelocities, applyVorticityAndViscosity, updatePositions).
 *
 * updateCells runs its work-items in ascending order unless the caller asks
 * for a parallel launch, so each cell's list comes out in descending particle
 * index (every atomic_xchg pushes a new head).  That makes the summation order
 * of the gather kernels, and hence their results, deterministic.  The other
 * kernels are data-parallel with no intra-kernel dependency and run under
 * OpenMP.
 */
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

#include "clshim.hpp"

thread_local size_t clshim_global_id = 0;
clshim_constants clshim_k;

/* The reference's kernels, compiled from its .cl files. */
void predictPositions(const float4 *positions, float4 *predicted,
                      float4 *velocities, const uint N);
void initCellsOld(int *cells, int *particles_list, const uint numCells,
                  const uint numParticles);
void updateCells(const float4 *predicted, int *cells, int *particles_list,
                 const uint N);
void computeScaling(float4 *predicted, float *scaling, const int *cells,
                    const int *particles_list, const int N);
void computeDelta(float4 *delta, const float4 *predicted, const float *scaling,
                  const int *cells, const int *particles_list,
                  const float wave_generator, const int N);
void updatePredicted(float4 *predicted, const float4 *delta, const uint N);
void updateVelocities(const float4 *positions, const float4 *predicted,
                      float4 *velocities, const uint N);
void applyVorticityAndViscosity(const float4 *predicted,
                                const float4 *velocities,
                                float4 *deltaVelocities, const int *cells,
                                const int *particles_list, const int N);
void updatePositions(float4 *positions, const float4 *predicted,
                     float4 *velocities, const float4 *deltaVelocities,
                     const uint N);

extern "C" {

/* Raw .par values (reference src/Parameters.hpp:12-31, the fields the
 * simulation reads). */
typedef struct {
  float x_min, x_max, y_min, y_max, z_min, z_max;
  float x_n, y_n, z_n;
  float timestep_length;
  float rest_density;
} ref_config;

}  // extern "C"

namespace {

/* One constant as main.cpp:149-168 prints it: ostream << showpoint << value,
 * followed by "f", read back by the OpenCL C compiler as a float literal. */
template <typename T>
float baked(T value) {
  std::ostringstream os;
  os << std::showpoint << value;
  return std::strtof(os.str().c_str(), nullptr);
}

void derive_constants(const ref_config &p, clshim_constants *k) {
  k->k_SYSTEM_MIN_X = baked(p.x_min);
  k->k_SYSTEM_MAX_X = baked(p.x_max);
  k->k_SYSTEM_MIN_Y = baked(p.y_min);
  k->k_SYSTEM_MAX_Y = baked(p.y_max);
  k->k_SYSTEM_MIN_Z = baked(p.z_min);
  k->k_SYSTEM_MAX_Z = baked(p.z_max);
  k->k_NUMBER_OF_CELLS_X = baked(p.x_n);
  k->k_NUMBER_OF_CELLS_Y = baked(p.y_n);
  k->k_NUMBER_OF_CELLS_Z = baked(p.z_n);
  k->k_CELL_LENGTH_X = baked((p.x_max - p.x_min) / p.x_n);
  k->k_CELL_LENGTH_Y = baked((p.y_max - p.y_min) / p.y_n);
  k->k_CELL_LENGTH_Z = baked((p.z_max - p.z_min) / p.z_n);
  k->k_TIMESTEP = baked(p.timestep_length);
  k->k_REST_DENSITY = baked(p.rest_density);
  const float h = (p.x_max - p.x_min) / p.x_n;
  k->k_PBF_H = baked(h);
  k->k_PBF_H_2 = baked(std::pow(h, 2));
  k->k_POLY6_FACTOR = baked(315.0f / (64.0f * M_PI * std::pow(h, 9)));
  k->k_GRAD_SPIKY_FACTOR = baked(45.0f / (M_PI * std::pow(h, 6)));
}

inline uint global_size(uint n) {
  return (uint)(std::ceil(n / 32.0f) * 32);
}

template <typename F>
void launch(uint gsize, int threads, F &&body) {
#pragma omp parallel for schedule(static) num_threads(threads)
  for (long i = 0; i < (long)gsize; ++i) {
    clshim_global_id = (size_t)i;
    body();
  }
}

template <typename F>
void launch_sequential(uint gsize, F &&body) {
  for (uint i = 0; i < gsize; ++i) {
    clshim_global_id = i;
    body();
  }
}

struct RefState {
  uint n = 0, ncells = 0;
  std::vector<float4> positions, velocities, predicted, delta, dvel;
  std::vector<float> scaling;
  std::vector<int> cells, list;
};

void build_cells(RefState &s, int threads, bool parallel_cells) {
  /* Simulation::updateCells (src/Simulation.cpp:330-349). */
  const uint init_range = std::max<uint>(s.n * 4u, s.ncells * 4u);
  launch(init_range, threads, [&] {
    initCellsOld(s.cells.data(), s.list.data(), s.ncells, s.n);
  });
  const uint g = global_size(s.n);
  if (parallel_cells) {
    launch(g, threads, [&] {
      updateCells(s.predicted.data(), s.cells.data(), s.list.data(), s.n);
    });
  } else {
    launch_sequential(g, [&] {
      updateCells(s.predicted.data(), s.cells.data(), s.list.data(), s.n);
    });
  }
}

void step(RefState &s, float wave, int threads, bool parallel_cells) {
  const uint g = global_size(s.n);
  const int N = (int)s.n;
  launch(g, threads, [&] {
    predictPositions(s.positions.data(), s.predicted.data(),
                     s.velocities.data(), s.n);
  });
  build_cells(s, threads, parallel_cells);
  const unsigned int solver_iterations = 4; /* Simulation.cpp:503 */
  for (unsigned int it = 0; it < solver_iterations; ++it) {
    launch(g, threads, [&] {
      computeScaling(s.predicted.data(), s.scaling.data(), s.cells.data(),
                     s.list.data(), N);
    });
    launch(g, threads, [&] {
      computeDelta(s.delta.data(), s.predicted.data(), s.scaling.data(),
                   s.cells.data(), s.list.data(), wave, N);
    });
    launch(g, threads, [&] {
      updatePredicted(s.predicted.data(), s.delta.data(), s.n);
    });
  }
  launch(g, threads, [&] {
    updateVelocities(s.positions.data(), s.predicted.data(),
                     s.velocities.data(), s.n);
  });
  launch(g, threads, [&] {
    applyVorticityAndViscosity(s.predicted.data(), s.velocities.data(),
                               s.dvel.data(), s.cells.data(), s.list.data(),
                               N);
  });
  launch(g, threads, [&] {
    updatePositions(s.positions.data(), s.predicted.data(),
                    s.velocities.data(), s.dvel.data(), s.n);
  });
}

bool setup(RefState &s, const ref_config *cfg, uint32_t n) {
  if (!cfg || n == 0) return false;
  derive_constants(*cfg, &clshim_k);
  const double c = (double)cfg->x_n * (double)cfg->y_n * (double)cfg->z_n;
  if (!(c >= 1.0) || c > 1.0e9) return false;
  s.n = n;
  s.ncells = (uint)c;
  /* The kernels read/write past N up to the NDRange only through their own
   * i >= N guards; buffers are sized exactly as the reference sizes them. */
  s.positions.assign(n, float4());
  s.velocities.assign(n, float4());
  s.predicted.assign(n, float4());
  s.delta.assign(n, float4());
  s.dvel.assign(n, float4());
  s.scaling.assign(n, 0.0f);
  s.cells.assign(s.ncells, -1);
  s.list.assign(n, -1);
  return true;
}

void load4(std::vector<float4> &dst, const float *src, uint n) {
  for (uint i = 0; i < n; ++i)
    dst[i] = float4(src[4 * i], src[4 * i + 1], src[4 * i + 2], src[4 * i + 3]);
}
void store4(float *dst, const std::vector<float4> &src, uint n) {
  for (uint i = 0; i < n; ++i) {
    dst[4 * i] = src[i].x;
    dst[4 * i + 1] = src[i].y;
    dst[4 * i + 2] = src[i].z;
    dst[4 * i + 3] = src[i].w;
  }
}

}  // namespace

extern "C" {

/* The 18 baked constants in clshim_constants field order. */
int ref_constants(const ref_config *cfg, float *out18) {
  if (!cfg || !out18) return 1;
  clshim_constants k;
  derive_constants(*cfg, &k);
  const float *src = &k.k_SYSTEM_MIN_X;
  for (int i = 0; i < 18; ++i) out18[i] = src[i];
  return 0;
}

/* Advances `steps` reference steps in place.  pos4/vel4 hold N float4 in the
 * layout of Simulation::dumpData (positions.w = |v|, velocities.w = mass).
 * Optional outputs (NULL to skip), all from the last step: predicted4 (N
 * float4; .w = density of the last computeScaling), scaling (N), cells (C
 * list heads) and list (N next links). */
int ref_run_steps(const ref_config *cfg, uint32_t n, float *pos4, float *vel4,
                  uint32_t steps, float wave, int threads, int parallel_cells,
                  float *predicted4_out, float *scaling_out, int *cells_out,
                  int *list_out) {
  RefState s;
  if (!setup(s, cfg, n) || !pos4 || !vel4) return 1;
  if (threads <= 0) threads = omp_get_max_threads();
  load4(s.positions, pos4, n);
  load4(s.velocities, vel4, n);
  for (uint32_t k = 0; k < steps; ++k) step(s, wave, threads, parallel_cells);
  store4(pos4, s.positions, n);
  store4(vel4, s.velocities, n);
  if (predicted4_out) store4(predicted4_out, s.predicted, n);
  if (scaling_out)
    for (uint i = 0; i < n; ++i) scaling_out[i] = s.scaling[i];
  if (cells_out)
    for (uint c = 0; c < s.ncells; ++c) cells_out[c] = s.cells[c];
  if (list_out)
    for (uint i = 0; i < n; ++i) list_out[i] = s.list[i];
  return 0;
}

/* initCellsOld + updateCells on caller-supplied predicted positions. */
int ref_build_cells(const ref_config *cfg, uint32_t n, const float *pred4,
                    int *cells_out, int *list_out) {
  RefState s;
  if (!setup(s, cfg, n) || !pred4 || !cells_out || !list_out) return 1;
  load4(s.predicted, pred4, n);
  build_cells(s, 1, false);
  for (uint c = 0; c < s.ncells; ++c) cells_out[c] = s.cells[c];
  for (uint i = 0; i < n; ++i) list_out[i] = s.list[i];
  return 0;
}

/* One computeScaling pass on caller-supplied predicted positions and lists;
 * writes predicted4 in place (.w = density) and scaling. */
int ref_compute_scaling(const ref_config *cfg, uint32_t n, float *pred4,
                        const int *cells, const int *list, float *scaling_out) {
  RefState s;
  if (!setup(s, cfg, n) || !pred4 || !cells || !list || !scaling_out) return 1;
  load4(s.predicted, pred4, n);
  for (uint c = 0; c < s.ncells; ++c) s.cells[c] = cells[c];
  for (uint i = 0; i < n; ++i) s.list[i] = list[i];
  launch(global_size(n), 1, [&] {
    computeScaling(s.predicted.data(), s.scaling.data(), s.cells.data(),
                   s.list.data(), (int)n);
  });
  store4(pred4, s.predicted, n);
  for (uint i = 0; i < n; ++i) scaling_out[i] = s.scaling[i];
  return 0;
}

}  // extern "C"
