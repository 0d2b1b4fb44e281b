// Solver kernels of the GB300 position-based-fluids step, reference
// equations (PBF_MODE_REF_COMPAT).  This translation unit is compiled with
// -fmad=false: every expression is evaluated operator by operator in IEEE
// binary32 with correctly rounded division and square root, in the operator
// order of the reference's kernels (MrMagne/position-based-fluids):
//   predict_positions.cl:8-9, update_cells.cl:10-15, compute_scaling.cl:11-140,
//   compute_delta.cl:13-152 + update_predicted.cl:7, update_velocities.cl:8,
//   apply_vorticity_and_viscosity.cl:12-104, update_positions.cl:9-12.
//
// State stays in input order (X, V, P = predicted with .w = density).  The
// neighbour structure is the stable sort of (cell, index) plus CSR offsets;
// each gather kernel visits the 27 cells around the particle's *current*
// cell in the reference's loop order (x outer, z inner) and each cell's
// particles in descending index -- the order a sequential launch of
// update_cells.cl leaves in the reference's linked lists.  With that order
// the results equal the reference's kernels bit for bit.  During the step
// the passes keep P, V and lambda by sorted slot as well (PS, VS, SS), so a
// cell's particles are read from consecutive slots -- the same values in
// the same order as through the permutation.
#include "pbf_device.cuh"

namespace pbf {

namespace {

constexpr int kThreads = 128;

// Calls f(m, load(m)) for the sorted slot m != q of every particle of the 27
// cells around the current cell of position p, in the reference's order.
// A cell's slots are loaded kGroup at a time (indices clamped into the cell),
// so the group's loads are in flight together; f still sees them one by one
// in descending slot order.
template <int kGroup = 4, typename Load, typename F>
__device__ __forceinline__ void ref_neighbours(uint32_t q, float4 p,
                                               const RefConsts &k,
                                               const uint32_t *__restrict__ off,
                                               Load &&load, F &&f) {
  int cc[3];
  cc[0] = (int)((p.x - k.min[0]) / k.clen[0]);
  cc[1] = (int)((p.y - k.min[1]) / k.clen[1]);
  cc[2] = (int)((p.z - k.min[2]) / k.clen[2]);
  const int nx = (int)k.ncell[0], ny = (int)k.ncell[1];
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        const int n0 = cc[0] + dx, n1 = cc[1] + dy, n2 = cc[2] + dz;
        if (n0 < 0 || (float)n0 >= k.ncell[0] || n1 < 0 ||
            (float)n1 >= k.ncell[1] || n2 < 0 || (float)n2 >= k.ncell[2])
          continue;
        const uint32_t ci = (uint32_t)n0 + (uint32_t)nx * ((uint32_t)n1 + (uint32_t)ny * (uint32_t)n2);
        const uint32_t a = __ldg(&off[ci]);
        for (uint32_t top = __ldg(&off[ci + 1]); top > a; top = top - a > kGroup ? top - kGroup : a) {
          decltype(load(0u)) d[kGroup];
#pragma unroll
          for (int e = 0; e < kGroup; ++e) d[e] = load(top - a > (uint32_t)e ? top - 1u - e : a);
#pragma unroll
          for (int e = 0; e < kGroup; ++e) {
            const uint32_t m = top - 1u - e;
            if (top - a > (uint32_t)e && m != q) f(m, d[e]);
          }
        }
      }
}

__global__ void __launch_bounds__(256)
    k_rc_predict_hash(const float4 *__restrict__ X, float4 *__restrict__ V,
                      float4 *__restrict__ P, uint32_t n, RefConsts k,
                      const SceneDesc *__restrict__ scenes,
                      uint32_t *__restrict__ keys, uint32_t passes,
                      uint32_t digit_bits, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_hist[kMaxHistWords];
  const uint32_t hist_words = passes << digit_bits;
  for (uint32_t t = threadIdx.x; t < hist_words; t += blockDim.x) s_hist[t] = 0;
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  uint32_t key = 0;
  if (valid) {
    const float4 x = X[i];
    float4 v = V[i];
    v.x = v.x + k.dt * 0.0f;
    v.y = v.y + k.dt * -9.81f;
    v.z = v.z + k.dt * 0.0f;
    V[i] = v;
    float4 p = P[i];
    p.x = x.x + k.dt * v.x;
    p.y = x.y + k.dt * v.y;
    p.z = x.z + k.dt * v.z;
    P[i] = p;
    key = scene_cell(p.x, p.y, p.z, scenes[0]);
    keys[i] = key;
  }
  warp_digit_histogram(key, valid, passes, digit_bits, s_hist);
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < hist_words; t += blockDim.x)
    if (s_hist[t]) atomicAdd(&hist[t], s_hist[t]);
}

__global__ void __launch_bounds__(256)
    k_rc_gather(const float4 *__restrict__ P, const uint32_t *__restrict__ perm, uint32_t n,
                float4 *__restrict__ PS) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  // perm is a permutation of [0, n) unless the sort reported an error.
  PS[q] = P[min(perm[q], n - 1u)];
}

__global__ void __launch_bounds__(kThreads)
    k_rc_lambda(float4 *__restrict__ PS, float *__restrict__ SS,
                const uint32_t *__restrict__ off, uint32_t n, RefConsts k) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float4 pi = PS[q];
  float dens = 0.0f, gsum = 0.0f, gvx = 0.0f, gvy = 0.0f, gvz = 0.0f;
  ref_neighbours(q, pi, k, off, [&](uint32_t m) { return PS[m]; }, [&](uint32_t, float4 pj) {
    const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (r2 > 0.0f && r2 < k.h2) {
      const float rl = sqrtf(r2);
      const float gx = rx / rl * k.spiky * (k.h - rl) * (k.h - rl);
      const float gy = ry / rl * k.spiky * (k.h - rl) * (k.h - rl);
      const float gz = rz / rl * k.spiky * (k.h - rl) * (k.h - rl);
      const float poly = k.poly6 * (k.h2 - r2) * (k.h2 - r2) * (k.h2 - r2);
      dens += poly;
      gsum += sqrtf(gx * gx + gy * gy + gz * gz);
      gvx += gx;
      gvy += gy;
      gvz += gz;
    }
  });
  gsum += sqrtf(gvx * gvx + gvy * gvy + gvz * gvz);
  // Only .w changes; concurrent readers use .xyz.
  reinterpret_cast<float *>(&PS[q])[3] = dens;
  const float c = dens / k.rest_density - 1.0f;
  SS[q] = -1.0f * c / (gsum * gsum / (k.rest_density * k.rest_density) + 10000.0f);
}

__global__ void __launch_bounds__(kThreads)
    k_rc_delta(const float4 *__restrict__ PS, float4 *__restrict__ PS2,
               const float *__restrict__ SS, const uint32_t *__restrict__ perm,
               const uint32_t *__restrict__ off, const float4 *__restrict__ X,
               float4 *__restrict__ V, float4 *__restrict__ P, float4 *__restrict__ VS,
               uint32_t n, RefConsts k, const SceneDesc *__restrict__ scenes, int last) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float4 pi = PS[q];
  const float si = SS[q];
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  struct PSl {
    float4 p;
    float s;
  };
  ref_neighbours(
      q, pi, k, off, [&](uint32_t m) { return PSl{__ldg(&PS[m]), __ldg(&SS[m])}; },
      [&](uint32_t, const PSl &d) {
    const float4 pj = d.p;
    const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (r2 > 0.0f && r2 < k.h2) {
      const float rl = sqrtf(r2);
      const float gx = -1.0f * rx / rl * k.spiky * (k.h - rl) * (k.h - rl);
      const float gy = -1.0f * ry / rl * k.spiky * (k.h - rl) * (k.h - rl);
      const float gz = -1.0f * rz / rl * k.spiky * (k.h - rl) * (k.h - rl);
      const float sc = si + d.s;
      sx += sc * gx;
      sy += sc * gy;
      sz += sc * gz;
    }
  });
  const float wave = scenes[0].wave;
  float fx = pi.x + sx / k.rest_density;
  float fy = pi.y + sy / k.rest_density;
  float fz = pi.z + sz / k.rest_density;
  if ((fx - k.h) < (k.min[0] + wave)) fx = k.min[0] + wave + k.h;
  else if ((fx + k.h) > k.max[0]) fx = k.max[0] - k.h;
  if ((fy - k.h) < k.min[1]) fy = k.min[1] + k.h;
  else if ((fy + k.h) > k.max[1]) fy = k.max[1] - k.h;
  if ((fz - k.h) < k.min[2]) fz = k.min[2] + k.h;
  else if ((fz + k.h) > k.max[2]) fz = k.max[2] - k.h;
  // computeDelta writes delta = future - predicted; updatePredicted adds it.
  const float dx = fx - pi.x, dy = fy - pi.y, dz = fz - pi.z;
  const float4 np = make_float4(pi.x + dx, pi.y + dy, pi.z + dz, pi.w);
  PS2[q] = np;
  if (last) {
    const uint32_t i = min(perm[q], n - 1u);
    P[i] = np;
    // updateVelocities
    const float4 x = X[i];
    float4 v = V[i];
    v.x = (np.x - x.x) / k.dt;
    v.y = (np.y - x.y) / k.dt;
    v.z = (np.z - x.z) / k.dt;
    V[i] = v;
    VS[q] = v;
  }
}

__global__ void __launch_bounds__(kThreads)
    k_rc_xsph(const float4 *__restrict__ PS, const float4 *__restrict__ VS,
              float4 *__restrict__ DV, const uint32_t *__restrict__ perm,
              const uint32_t *__restrict__ off, uint32_t n, RefConsts k) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float4 pi = PS[q];
  const float4 vi = VS[q];
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  ref_neighbours(q, pi, k, off, [&](uint32_t m) { return __ldg(&PS[m]); }, [&](uint32_t m, float4 pj) {
    const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (r2 > 0.0f && r2 < k.h2) {
      const float4 vj = __ldg(&VS[m]);
      const float vx = vj.x - vi.x, vy = vj.y - vi.y, vz = vj.z - vi.z;
      const float poly = k.poly6 * (k.h2 - r2) * (k.h2 - r2) * (k.h2 - r2);
      const float inv = 1.0f / pj.w;
      sx += inv * vx * poly;
      sy += inv * vy * poly;
      sz += inv * vz * poly;
    }
  });
  DV[min(perm[q], n - 1u)] = make_float4(0.01f * sx, 0.01f * sy, 0.01f * sz, 0.0f);
}

__global__ void __launch_bounds__(256)
    k_rc_commit(float4 *__restrict__ X, float4 *__restrict__ V,
                const float4 *__restrict__ P, const float4 *__restrict__ DV,
                uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = P[i];
  const float4 dv = DV[i];
  float4 v = V[i];
  v.x += dv.x;
  v.y += dv.y;
  v.z += dv.z;
  V[i] = v;
  X[i] = make_float4(p.x, p.y, p.z, sqrtf(v.x * v.x + v.y * v.y + v.z * v.z));
}

inline uint32_t blocks_for(uint64_t n, uint32_t t) {
  return (uint32_t)((n + t - 1) / t);
}

}  // namespace

cudaError_t rc_predict_hash(float4 *X, float4 *V, float4 *P, uint32_t n,
                            const RefConsts &k, const SceneDesc *scenes,
                            uint32_t *keys, const SortPlan &plan,
                            uint32_t *sort_scratch, cudaStream_t st) {
  k_rc_predict_hash<<<blocks_for(n, 256), 256, 0, st>>>(
      X, V, P, n, k, scenes, keys, plan.passes, plan.digit_bits,
      sort_scratch + plan.off_hist);
  return cudaGetLastError();
}

cudaError_t rc_gather(const float4 *P, const uint32_t *perm, uint32_t n, float4 *PS,
                      cudaStream_t st) {
  k_rc_gather<<<blocks_for(n, 256), 256, 0, st>>>(P, perm, n, PS);
  return cudaGetLastError();
}

cudaError_t rc_lambda(float4 *PS, float *SS, const uint32_t *offsets, uint32_t n,
                      const RefConsts &k, cudaStream_t st) {
  k_rc_lambda<<<blocks_for(n, kThreads), kThreads, 0, st>>>(PS, SS, offsets, n, k);
  return cudaGetLastError();
}

cudaError_t rc_delta(const float4 *PS, float4 *PS2, const float *SS, const uint32_t *perm,
                     const uint32_t *offsets, const float4 *X, float4 *V, float4 *P,
                     float4 *VS, uint32_t n, const RefConsts &k, const SceneDesc *scenes,
                     bool last, cudaStream_t st) {
  k_rc_delta<<<blocks_for(n, kThreads), kThreads, 0, st>>>(
      PS, PS2, SS, perm, offsets, X, V, P, VS, n, k, scenes, last ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t rc_xsph(const float4 *PS, const float4 *VS, float4 *DV, const uint32_t *perm,
                    const uint32_t *offsets, uint32_t n, const RefConsts &k,
                    cudaStream_t st) {
  k_rc_xsph<<<blocks_for(n, kThreads), kThreads, 0, st>>>(PS, VS, DV, perm, offsets, n, k);
  return cudaGetLastError();
}

cudaError_t rc_commit(float4 *X, float4 *V, const float4 *P, const float4 *DV,
                      uint32_t n, cudaStream_t st) {
  k_rc_commit<<<blocks_for(n, 256), 256, 0, st>>>(X, V, P, DV, n);
  return cudaGetLastError();
}

}  // namespace pbf
