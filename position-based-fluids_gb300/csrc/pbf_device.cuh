// Device helpers shared by the CUDA translation units (nvcc only).
#pragma once

#include "pbf_internal.cuh"

namespace pbf {

// Device helpers used by several translation units.
__device__ __forceinline__ int axis_cell(float p, float mn, float cl, int n) {
  // trunc((p - min) / cell_length) as the reference's (int) cast, clamped.
  const int c = __float2int_rz(__fdiv_rn(__fsub_rn(p, mn), cl));
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

__device__ __forceinline__ uint32_t scene_cell(float x, float y, float z,
                                               const SceneDesc &s) {
  const int cx = axis_cell(x, s.gmin[0], s.clen[0], s.ncell[0]);
  const int cy = axis_cell(y, s.gmin[1], s.clen[1], s.ncell[1]);
  const int cz = axis_cell(z, s.gmin[2], s.clen[2], s.ncell[2]);
  return (uint32_t)cx +
         (uint32_t)s.ncell[0] * ((uint32_t)cy + (uint32_t)s.ncell[1] * (uint32_t)cz);
}

// Accumulates the per-pass digit histograms (digit_bits wide, pass p's
// histogram at p << digit_bits) of one key per lane into shared memory,
// aggregating equal digits within the warp first.
__device__ __forceinline__ void warp_digit_histogram(uint32_t key, bool valid,
                                                     uint32_t passes, uint32_t digit_bits,
                                                     uint32_t *s_hist) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t mask = (1u << digit_bits) - 1u;
  for (uint32_t p = 0; p < passes; ++p) {
    const uint32_t d = (key >> (p * digit_bits)) & mask;
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0xffffffffu);
    if (valid && lane == (unsigned)(__ffs(peers) - 1))
      atomicAdd(&s_hist[(p << digit_bits) + d], (uint32_t)__popc(peers));
  }
}

// Counts key into counts[] for the counting sort: equal keys of a warp
// aggregated into one atomic; pos[i] = the particle's place among the
// increments of its cell (warp lanes in order, warps in atomic order).
__device__ __forceinline__ void count_cell_key(uint32_t key, bool valid, uint32_t i,
                                               uint32_t *__restrict__ counts,
                                               uint32_t *__restrict__ pos) {
  const uint32_t lane = threadIdx.x & 31u;
  const unsigned peers = __match_any_sync(0xffffffffu, valid ? key : 0xffffffffu);
  const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
  uint32_t base = 0;
  if (valid && lane == leader) base = atomicAdd(&counts[key], (uint32_t)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, (int)leader);
  if (valid) pos[i] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

}  // namespace pbf
