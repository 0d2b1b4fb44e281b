// Solver kernels of the GB300 position-based-fluids step, paper equations
// (PBF_MODE_PAPER): Macklin & Mueller, "Position Based Fluids", ACM TOG
// 32(4) 2013, Algorithm 1.  The reference's kernels this path replaces:
//   predict_positions.cl, update_cells.cl / calc_hash.cl (predict + hash),
//   compute_scaling.cl (lambda), compute_delta.cl + update_predicted.cl
//   (delta p with s_corr, wall clamp, Jacobi apply), update_velocities.cl,
//   apply_vorticity_and_viscosity.cl + update_positions.cl (vorticity
//   confinement, XSPH, commit).
//
// Layout: the particle state stays sorted by cell from one step to the next
// (X, V, and ID = input index), so the reorder gather after each sort reads
// nearly sequential memory.  After the sort every array below is indexed by
// sorted slot k:
//   X2, V2  state at the start of the step, V2 with gravity applied
//   P       predicted position x + d
//   D       displacement d since the start of the step (kept apart from x so
//           that positions round once per step, not once per iteration);
//           the vorticity pass then reuses it for (p, |vorticity|)
//   Q       (predicted position, lambda) as read by the delta-p pass
//   U       (velocity, 1/rho) as read by the velocity passes
//   W       (vorticity, |vorticity|)
// Neighbour sets are built once per step from the predicted positions
// (Algorithm 1 line 6): N_k = { j != k : r0 <= |p_k - p_j| < h } over the
// 27 cells around k's cell, r0 = sqrt(FLT_MIN) ~ 1.1e-19 (closer particles
// count as coincident).  Every later pass evaluates the kernels at the
// current positions with W = 0 beyond h and below r0.
//
// Gather passes run one thread per sorted particle.  Neighbour lists hold
// each neighbour as its 32-bit sorted slot, four per 16-byte word: group g of
// particle k is nbr4[g*N + k], so a warp reads its particles' next four
// neighbours with one coalesced load per thread, and the neighbour loads of
// a batch (4 or 8 entries, a launch-shape choice) are independent.  A
// particle whose set exceeds the list capacity re-derives it from the cells
// and the step-start positions in every pass instead (same order, same
// arithmetic).
//
// Cache policy: the list words (~100 MB per pass at 1M particles, each read
// once) are loaded without allocating in L1 and first in line for eviction
// from L2, and the values a thread reads only for itself skip L1 as well, so
// both caches keep the neighbour data that dozens of threads re-read (7%
// off the whole step on GB300).  The next batch's list words are loaded into
// registers one batch ahead, so a batch's neighbour loads do not wait on a
// list word from DRAM.
//
// Measured on GB300 (1M-particle dam break after 500 steps, per step):
// absolute 32-bit entries run 9% faster than 16-bit entries relative to a
// per-tile table of row ranges -- the decode and the per-tile set-up cost
// more issue slots than the larger lists cost DRAM time (the passes run at
// a third of DRAM bandwidth or less); a variant that first staged each tile's
// neighbourhood into shared memory with cp.async.bulk ran 1.1-2x slower than
// these L1 gathers; a persistent grid that kept neighbouring tiles on one SM
// raised the L1 hit rate from 69% to 77% but ran 4% slower; four threads per
// particle (neighbour entries split between them, shuffle reduction) ran
// 1.4x slower.
#include <type_traits>

#include "pbf_device.cuh"

namespace pbf {

namespace {


struct NbrCtx {
  const uint4 *__restrict__ nbr4;
  const uint32_t *__restrict__ cnt;
  const uint32_t *__restrict__ skeys;
  const uint32_t *__restrict__ off;
  const float4 *__restrict__ X2;
  const float4 *__restrict__ V2;
  const SceneDesc *__restrict__ scenes;
  const uint16_t *__restrict__ sid;
  uint32_t *err;
  uint32_t n, maxn;
  float dt, h2;
};

__device__ __forceinline__ const SceneDesc &scene_of(const SceneDesc *scenes,
                                                     const uint16_t *sid,
                                                     uint32_t k) {
  return scenes[sid ? sid[k] : 0];
}

// List words are read once per pass: load them without keeping them in L1
// and first in line for eviction from L2 (policy from l2_evict_first), so
// the caches keep the neighbour data that is re-read.
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t policy;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
  return policy;
}
__device__ __forceinline__ uint4 load_list_word(const uint4 *p, uint64_t policy) {
  uint4 v;
  asm volatile(
      "ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(p), "l"(policy));
  return v;
}

// A value only its own thread reads (once per pass): loaded without
// allocating in L1, so L1 keeps the neighbour data the CTA re-reads.
__device__ __forceinline__ float4 load_own(const float4 *p) {
  float4 v;
  asm volatile("ld.global.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}
__device__ __forceinline__ uint32_t load_own(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.global.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float load_own(const float *p) {
  float v;
  asm volatile("ld.global.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// For the `cnt` listed neighbours of particle k, kBatch (4 or 8) at a time:
// the batch's list words, then load(slot) for every entry of the batch, then
// f(data) for each in list order -- the loads of a batch are in flight
// together, and the next batch's list words are loaded into registers while
// the current batch's neighbour data loads and computes.  The list build
// pads the last word with k's own slot and words past the count read as k:
// those entries are the particle itself, which every pass drops through the
// pair test (r^2 = 0), so no entry needs a bound or a count test.
template <int kBatch, typename Load, typename F>
__device__ __forceinline__ void for_each_listed(const NbrCtx &c, uint32_t k, uint32_t cnt,
                                                Load &&load, F &&f) {
  static_assert(kBatch % 4 == 0, "whole list words per batch");
  constexpr int kWords = kBatch / 4;
  const uint64_t pol = l2_evict_first();
  uint4 cur[kWords];
#pragma unroll
  for (int w = 0; w < kWords; ++w)
    cur[w] = (w == 0 || 4u * (uint32_t)w < cnt) ? load_list_word(&c.nbr4[(size_t)w * c.n + k], pol)
                                                : make_uint4(k, k, k, k);
  for (uint32_t e0 = 0; e0 < cnt; e0 += kBatch) {
    uint4 nxt[kWords];
#pragma unroll
    for (int w = 0; w < kWords; ++w) {
      const uint32_t g = (e0 >> 2) + (uint32_t)(kWords + w);
      nxt[w] = 4u * g < cnt ? load_list_word(&c.nbr4[(size_t)g * c.n + k], pol)
                            : make_uint4(k, k, k, k);
    }
    uint32_t slot[kBatch];
#pragma unroll
    for (int w = 0; w < kWords; ++w) {
      slot[4 * w + 0] = cur[w].x;
      slot[4 * w + 1] = cur[w].y;
      slot[4 * w + 2] = cur[w].z;
      slot[4 * w + 3] = cur[w].w;
    }
    decltype(load(0u)) data[kBatch];
#pragma unroll
    for (int e = 0; e < kBatch; ++e) data[e] = load(slot[e]);
#pragma unroll
    for (int e = 0; e < kBatch; ++e) f(data[e]);
#pragma unroll
    for (int w = 0; w < kWords; ++w) cur[w] = nxt[w];
  }
}

// v' = v + dt g;  d = dt v';  p = x + d  -- rounded op by op (no
// contraction) so that every kernel that recomputes them gets the same bits.
__device__ __forceinline__ float4 gravity_velocity(float4 v, float dt, float gy) {
  v.y = __fadd_rn(v.y, __fmul_rn(dt, gy));
  return v;
}
__device__ __forceinline__ float3 displacement(float4 v1, float dt) {
  return make_float3(__fmul_rn(dt, v1.x), __fmul_rn(dt, v1.y), __fmul_rn(dt, v1.z));
}
__device__ __forceinline__ float3 add3(float4 x, float3 d) {
  return make_float3(__fadd_rn(x.x, d.x), __fadd_rn(x.y, d.y), __fadd_rn(x.z, d.z));
}

// Step-start predicted position of slot j (as written by the reorder).
__device__ __forceinline__ float3 start_position(const NbrCtx &c, uint32_t j) {
  return add3(__ldg(&c.X2[j]), displacement(__ldg(&c.V2[j]), c.dt));
}

// Particles j != k closer than h form a pair.  Distances below
// sqrt(FLT_MIN) ~ 1.1e-19 count as coincident (like r = 0, whose direction
// is undefined), so r^2 is a normal number wherever a kernel is evaluated.
__device__ __forceinline__ bool is_pair(float r2, float h2) {
  return r2 >= 1.17549435e-38f && r2 < h2;
}

// Visits the 9 rows around the cell with key `key` (order: dz, dy, slot);
// f(q, j) gets the row index q = (dz+1)*3 + (dy+1) and the slot j != k.
template <typename F>
__device__ __forceinline__ void scan_rows(uint32_t k, uint32_t key, const SceneDesc &s,
                                          const uint32_t *__restrict__ off, F &&f) {
  const int nx = s.ncell[0], ny = s.ncell[1], nz = s.ncell[2];
  const uint32_t local = key - s.cell_base;
  const int cx = (int)(local % (uint32_t)nx);
  const uint32_t t = local / (uint32_t)nx;
  const int cy = (int)(t % (uint32_t)ny);
  const int cz = (int)(t / (uint32_t)ny);
  const int x0 = cx > 0 ? cx - 1 : 0;
  const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
  for (int dz = -1; dz <= 1; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= ny) continue;
      const int q = (dz + 1) * 3 + (dy + 1);
      const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
      const uint32_t a = __ldg(&off[row + x0]);
      const uint32_t b = __ldg(&off[row + x1 + 1]);
      for (uint32_t j = a; j < b; ++j)
        if (j != k) f(q, j);
    }
  }
}

// Re-derives N_k from the cells and the step-start positions (global loads).
template <typename F>
__device__ __forceinline__ void visit_fallback(const NbrCtx &c, uint32_t k, F &&f) {
  const SceneDesc &sc = scene_of(c.scenes, c.sid, k);
  const float3 pk = start_position(c, k);
  scan_rows(k, __ldg(&c.skeys[k]), sc, c.off, [&](int, uint32_t j) {
    const float3 pj = start_position(c, j);
    const float rx = pk.x - pj.x, ry = pk.y - pj.y, rz = pk.z - pj.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (is_pair(r2, c.h2)) f(j);
  });
}

// Calls f(load(slot)) for every neighbour of particle k (and, in the listed
// path, for k itself as the padding of the last group): from the list when
// k's set fits, otherwise re-derived.
template <int kBatch, typename Load, typename F>
__device__ __forceinline__ void visit_neighbours(const NbrCtx &c, uint32_t k, Load &&load,
                                                 F &&f) {
  const uint32_t cnt = load_own(&c.cnt[k]);
  if (cnt <= c.maxn) {
    for_each_listed<kBatch>(c, k, cnt, load, f);
  } else {
    visit_fallback(c, k, [&](uint32_t j) { f(load(j)); });
  }
}

__device__ __forceinline__ float ipow(float b, int e) {
  float r = 1.0f;
  while (e > 0) {
    if (e & 1) r *= b;
    b *= b;
    e >>= 1;
  }
  return r;
}

// -k h^2 (W(r)/W(dq h))^n with W(r)/W(dq h) = ((h^2-r^2)/(h^2-dq^2 h^2))^3;
// kTwelve: the exponent 3n is 12 (n = 4, the paper's choice).
template <bool kTwelve>
__device__ __forceinline__ float scorr_term(float r2, const PaperConsts &c) {
  const float ratio = (c.h2 - r2) * c.inv_scorr_den;
  if constexpr (kTwelve) {
    const float r3 = ratio * ratio * ratio;
    const float r6 = r3 * r3;
    return -c.scorr_k * (r6 * r6);
  } else {
    return -c.scorr_k * ipow(ratio, c.scorr_n3);
  }
}

// Spiky gradient factor: grad_i W(r_vec) = f * r_vec, f = -S (h-r)^2 / r,
// for a pair (r^2 normal, so the MUFU reciprocal square root without the
// subnormal-input path equals rsqrtf).
__device__ __forceinline__ float spiky_factor(float r2, const PaperConsts &c) {
  float rinv;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rinv) : "f"(r2));
  const float hr = c.h - r2 * rinv;
  return -c.spiky * hr * hr * rinv;
}

struct LambdaAcc {
  float rho, gx, gy, gz, s;
  __device__ __forceinline__ void add(float rx, float ry, float rz, float r2,
                                      const PaperConsts &c) {
    const float t = c.h2 - r2;
    rho += c.poly6 * t * t * t;
    const float f = spiky_factor(r2, c);
    gx += f * rx;
    gy += f * ry;
    gz += f * rz;
    s += f * f * r2;
  }
  __device__ __forceinline__ float lambda(const PaperConsts &c) const {
    const float C = rho * c.inv_rho0 - 1.0f;
    const float den = (gx * gx + gy * gy + gz * gz + s) * (c.inv_rho0 * c.inv_rho0);
    return -C / (den + c.relax_eps);
  }
};

// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_predict_hash(const float4 *__restrict__ X, const float4 *__restrict__ V,
                   uint32_t n, PaperConsts c,
                   const SceneDesc *__restrict__ scenes,
                   const uint16_t *__restrict__ sid, uint32_t *__restrict__ keys,
                   uint32_t passes, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_hist[kMaxSortPasses * kRadix];
  for (uint32_t i = threadIdx.x; i < passes * kRadix; i += blockDim.x) s_hist[i] = 0;
  __syncthreads();
  // Grid-stride over the particles (whole warps iterate together so that
  // __match_any_sync sees every lane): one histogram flush per CTA.
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t k = base + threadIdx.x;
    const bool valid = k < n;
    uint32_t key = 0;
    if (valid) {
      const float4 x = X[k];
      const float4 v1 = gravity_velocity(V[k], c.dt, c.gy);
      const float3 p = add3(x, displacement(v1, c.dt));
      const SceneDesc &s = scene_of(scenes, sid, k);
      key = s.cell_base + scene_cell(p.x, p.y, p.z, s);
      keys[k] = key;
    }
    warp_digit_histogram(key, valid, passes, s_hist);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
    if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

__global__ void __launch_bounds__(256)
    k_reorder(const uint32_t *__restrict__ perm, const float4 *__restrict__ X,
              const float4 *__restrict__ V, const uint32_t *__restrict__ ID,
              uint32_t n, PaperConsts c, float4 *__restrict__ X2,
              float4 *__restrict__ V2, uint32_t *__restrict__ ID2,
              float4 *__restrict__ P, float4 *__restrict__ D) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  // perm is a permutation of [0, n) unless the sort reported an error.
  const uint32_t src = min(perm[k], n - 1);
  const float4 x = X[src];
  const float4 v1 = gravity_velocity(V[src], c.dt, c.gy);
  const float3 d = displacement(v1, c.dt);
  const float3 p = add3(x, d);
  X2[k] = x;
  V2[k] = v1;
  ID2[k] = ID[src];
  P[k] = make_float4(p.x, p.y, p.z, 0.0f);
  D[k] = make_float4(d.x, d.y, d.z, 0.0f);
}

// Calls member(j, rx, ry, rz, r2) for every slot j that forms a pair with k
// (is_pair(r2 = |p_k - p_j|^2)) in the 27 cells around k's cell (key `key`),
// in the order the lists store and the re-derived path visits: rows by
// (dz, dy), each row's slots ascending.  The self pair and coincident
// particles drop out.
template <typename F>
__device__ __forceinline__ void scan_members(const float4 &pk, uint32_t key, const SceneDesc &s,
                                             const uint32_t *__restrict__ off,
                                             const float4 *__restrict__ P, const PaperConsts &c,
                                             F &&member) {
  const int nx = s.ncell[0], ny = s.ncell[1], nz = s.ncell[2];
  const uint32_t local = key - s.cell_base;
  const int cx = (int)(local % (uint32_t)nx);
  const uint32_t t = local / (uint32_t)nx;
  const int cy = (int)(t % (uint32_t)ny);
  const int cz = (int)(t / (uint32_t)ny);
  const int x0 = cx > 0 ? cx - 1 : 0;
  const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
  for (int dz = -1; dz <= 1; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= ny) continue;
      const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
      const uint32_t a = __ldg(&off[row + x0]);
      const uint32_t b = __ldg(&off[row + x1 + 1]);
      // whole groups of four candidates (loads at fixed offsets from one
      // pointer, no per-load bound), then the last one to three
      uint32_t j = a;
      for (; j + 4u <= b; j += 4) {
        const float4 *__restrict__ q = P + j;
        float4 d[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) d[e] = __ldg(q + e);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float rx = pk.x - d[e].x, ry = pk.y - d[e].y, rz = pk.z - d[e].z;
          const float r2 = rx * rx + ry * ry + rz * rz;
          if (is_pair(r2, c.h2)) member(j + e, rx, ry, rz, r2);
        }
      }
      if (j < b) {
        float4 d[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) d[e] = __ldg(&P[min(j + e, b - 1u)]);
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          const float rx = pk.x - d[e].x, ry = pk.y - d[e].y, rz = pk.z - d[e].z;
          const float r2 = rx * rx + ry * ry + rz * rz;
          if (j + e < b && is_pair(r2, c.h2)) member(j + e, rx, ry, rz, r2);
        }
      }
    }
  }
}

// Fills the rest of a listed set's last word with the particle's own slot
// (maxn is a multiple of 8, so the word is inside the list capacity).
__device__ __forceinline__ void pad_list(uint32_t *__restrict__ out, size_t stride,
                                         uint32_t cnt, uint32_t maxn, uint32_t k) {
  if (cnt <= maxn)
    for (uint32_t e = cnt; e & 3u; ++e) out[(size_t)(e >> 2) * stride + (e & 3u)] = k;
}

// Neighbour-list build from the predicted positions P (which equal the
// step-start positions the fallback recomputes).  Each member's slot is
// stored straight into its list word; the rest of the last word holds the
// particle's own slot.
template <int kBlock>
__global__ void __launch_bounds__(kBlock)
    k_nbr_build(const float4 *__restrict__ P, NbrCtx nc, PaperConsts c,
                uint4 *__restrict__ nbr4, uint32_t *__restrict__ nbr_cnt) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = P[k];
  uint32_t *__restrict__ out = reinterpret_cast<uint32_t *>(nbr4) + 4ull * k;
  const size_t stride = 4ull * c.n;  // words from one list group to the next
  uint32_t cnt = 0;
  scan_members(pk, nc.skeys[k], scene_of(nc.scenes, nc.sid, k), nc.off, P, c,
               [&](uint32_t j, float, float, float, float) {
                 if (cnt < c.maxn) out[(size_t)(cnt >> 2) * stride + (cnt & 3u)] = j;
                 ++cnt;
               });
  pad_list(out, stride, cnt, c.maxn, k);
  nbr_cnt[k] = cnt;
}

// k_nbr_build fused with the first lambda pass: the same lists, and lambda
// summed over the members in the order the lists store them -- the bits
// k_lambda computes from the lists.  (In one kernel a warp executes the
// lambda arithmetic whenever any of its lanes has a member, so which form is
// faster depends on the scene; the tuner picks.)
template <int kBlock>
__global__ void __launch_bounds__(kBlock)
    k_nbr_lambda(const float4 *__restrict__ P, NbrCtx nc, PaperConsts c,
                 uint4 *__restrict__ nbr4, uint32_t *__restrict__ nbr_cnt,
                 float4 *__restrict__ Q, float *__restrict__ R) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = P[k];
  uint32_t *__restrict__ out = reinterpret_cast<uint32_t *>(nbr4) + 4ull * k;
  const size_t stride = 4ull * c.n;  // words from one list group to the next
  uint32_t cnt = 0;
  LambdaAcc acc{c.w_self, 0.f, 0.f, 0.f, 0.f};
  scan_members(pk, nc.skeys[k], scene_of(nc.scenes, nc.sid, k), nc.off, P, c,
               [&](uint32_t j, float rx, float ry, float rz, float r2) {
                 if (cnt < c.maxn) out[(size_t)(cnt >> 2) * stride + (cnt & 3u)] = j;
                 ++cnt;
                 acc.add(rx, ry, rz, r2, c);
               });
  pad_list(out, stride, cnt, c.maxn, k);
  nbr_cnt[k] = cnt;
  Q[k] = make_float4(pk.x, pk.y, pk.z, acc.lambda(c));
  R[k] = acc.rho;
}

template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock)
    k_lambda(const float4 *__restrict__ P, NbrCtx nc, PaperConsts c,
             float4 *__restrict__ Q, float *__restrict__ R) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = P[k];
  LambdaAcc acc{c.w_self, 0.f, 0.f, 0.f, 0.f};
  visit_neighbours<kBatch>(
      nc, k, [&](uint32_t j) { return __ldg(&P[j]); },
      [&](float4 pj) {
        const float rx = pk.x - pj.x, ry = pk.y - pj.y, rz = pk.z - pj.z;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (is_pair(r2, c.h2)) acc.add(rx, ry, rz, r2, c);
      });
  Q[k] = make_float4(pk.x, pk.y, pk.z, acc.lambda(c));
  R[k] = acc.rho;
}

template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock)
    k_delta(const float4 *__restrict__ Q, NbrCtx nc, PaperConsts c,
            float4 *__restrict__ D, float4 *__restrict__ P,
            const float *__restrict__ R, float4 *__restrict__ U, int last) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 qk = Q[k];
  float sx = 0.f, sy = 0.f, sz = 0.f;
  // one neighbour walk per s_corr exponent form, chosen once per thread
  const auto walk = [&](auto twelve) {
    visit_neighbours<kBatch>(
        nc, k, [&](uint32_t j) { return __ldg(&Q[j]); },
        [&](float4 qj) {
          const float rx = qk.x - qj.x, ry = qk.y - qj.y, rz = qk.z - qj.z;
          const float r2 = rx * rx + ry * ry + rz * rz;
          if (is_pair(r2, c.h2)) {
            const float wgt = (qk.w + qj.w + scorr_term<decltype(twelve)::value>(r2, c)) *
                              spiky_factor(r2, c);
            sx += wgt * rx;
            sy += wgt * ry;
            sz += wgt * rz;
          }
        });
  };
  if (c.scorr_n3 == 12) walk(std::true_type{});
  else walk(std::false_type{});
  const float4 x = load_own(&nc.X2[k]);
  const float4 d0 = load_own(&D[k]);
  float3 d = make_float3(d0.x + sx * c.inv_rho0, d0.y + sy * c.inv_rho0,
                         d0.z + sz * c.inv_rho0);
  float3 p = add3(x, d);
  const SceneDesc &sc = scene_of(nc.scenes, nc.sid, k);
  const float lo_x = sc.lo[0] + sc.wave;
  // Collision response: clamp to the admissible box (moving x-min wall).
  if (p.x < lo_x) { d.x = lo_x - x.x; p.x = x.x + d.x; }
  else if (p.x > sc.hi[0]) { d.x = sc.hi[0] - x.x; p.x = x.x + d.x; }
  if (p.y < sc.lo[1]) { d.y = sc.lo[1] - x.y; p.y = x.y + d.y; }
  else if (p.y > sc.hi[1]) { d.y = sc.hi[1] - x.y; p.y = x.y + d.y; }
  if (p.z < sc.lo[2]) { d.z = sc.lo[2] - x.z; p.z = x.z + d.z; }
  else if (p.z > sc.hi[2]) { d.z = sc.hi[2] - x.z; p.z = x.z + d.z; }
  D[k] = make_float4(d.x, d.y, d.z, 0.0f);
  P[k] = make_float4(p.x, p.y, p.z, 0.0f);
  if (last)
    U[k] = make_float4(__fdiv_rn(d.x, c.dt), __fdiv_rn(d.y, c.dt),
                       __fdiv_rn(d.z, c.dt), 1.0f / load_own(&R[k]));
}

// Vorticity omega_k; also writes (p_k, |omega_k|) into PW for the next pass.
template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock)
    k_vorticity(const float4 *__restrict__ P, const float4 *__restrict__ U,
                NbrCtx nc, PaperConsts c, float4 *__restrict__ Wo,
                float4 *__restrict__ PW) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = P[k];
  const float4 uk = U[k];
  float wx = 0.f, wy = 0.f, wz = 0.f;
  struct PU {
    float4 p, u;
  };
  visit_neighbours<kBatch>(
      nc, k, [&](uint32_t j) { return PU{__ldg(&P[j]), __ldg(&U[j])}; },
      [&](const PU &d) {
    const float4 pj = d.p;
    const float rx = pk.x - pj.x, ry = pk.y - pj.y, rz = pk.z - pj.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (is_pair(r2, c.h2)) {
      const float4 uj = d.u;
      const float f = spiky_factor(r2, c) * uj.w;
      const float gx = f * rx, gy = f * ry, gz = f * rz;
      const float ux = uj.x - uk.x, uy = uj.y - uk.y, uz = uj.z - uk.z;
      wx += gy * uz - gz * uy;
      wy += gz * ux - gx * uz;
      wz += gx * uy - gy * ux;
    }
  });
  const float wn = sqrtf(wx * wx + wy * wy + wz * wz);
  Wo[k] = make_float4(wx, wy, wz, wn);
  PW[k] = make_float4(pk.x, pk.y, pk.z, wn);
}

// At least 1024 resident threads per SM (64 registers): no spills in any
// shape.  Left to itself the compiler takes more (96 with eight loads in
// flight) and halves the resident warps.
template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock, 1024 / kBlock)
    k_xsph_commit(const float4 *__restrict__ PW, const float4 *__restrict__ U,
                  const float4 *__restrict__ Wv, NbrCtx nc, PaperConsts c,
                  const uint32_t *__restrict__ ID2, float4 *__restrict__ X,
                  float4 *__restrict__ V, uint32_t *__restrict__ ID) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = PW[k];
  const float4 uk = U[k];
  const float4 wk = load_own(&Wv[k]);
  float ex = 0.f, ey = 0.f, ez = 0.f, xx = 0.f, xy = 0.f, xz = 0.f;
  struct PU {
    float4 p, u;
  };
  visit_neighbours<kBatch>(
      nc, k, [&](uint32_t j) { return PU{__ldg(&PW[j]), __ldg(&U[j])}; },
      [&](const PU &d) {
    const float4 pj = d.p;
    const float rx = pk.x - pj.x, ry = pk.y - pj.y, rz = pk.z - pj.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (is_pair(r2, c.h2)) {
      const float4 uj = d.u;
      const float e = spiky_factor(r2, c) * uj.w * (pj.w - wk.w);
      ex += e * rx;
      ey += e * ry;
      ez += e * rz;
      const float t = c.h2 - r2;
      const float wp = c.poly6 * t * t * t * uj.w;
      xx += wp * (uj.x - uk.x);
      xy += wp * (uj.y - uk.y);
      xz += wp * (uj.z - uk.z);
    }
  });
  const float el2 = ex * ex + ey * ey + ez * ez;
  float nx = 0.f, ny = 0.f, nz = 0.f;
  if (el2 > 0.0f) {
    const float inv = rsqrtf(el2);
    nx = ex * inv;
    ny = ey * inv;
    nz = ez * inv;
  }
  const float fx = c.vort_eps * (ny * wk.z - nz * wk.y);
  const float fy = c.vort_eps * (nz * wk.x - nx * wk.z);
  const float fz = c.vort_eps * (nx * wk.y - ny * wk.x);
  const float vx = uk.x + c.dt * fx + c.xsph_c * xx;
  const float vy = uk.y + c.dt * fy + c.xsph_c * xy;
  const float vz = uk.z + c.dt * fz + c.xsph_c * xz;
  X[k] = make_float4(pk.x, pk.y, pk.z, sqrtf(vx * vx + vy * vy + vz * vz));
  V[k] = make_float4(vx, vy, vz, load_own(&nc.V2[k]).w);
  ID[k] = load_own(&ID2[k]);
}

__global__ void k_gather_out(const float4 *__restrict__ X,
                             const float4 *__restrict__ V,
                             const uint32_t *__restrict__ ID, uint32_t n,
                             float4 *__restrict__ out_pos,
                             float4 *__restrict__ out_vel) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = ID[k];
  out_pos[i] = X[k];
  out_vel[i] = V[k];
}

__global__ void k_scatter_in(const float4 *__restrict__ in_pos,
                             const float4 *__restrict__ in_vel,
                             const uint32_t *__restrict__ ID, uint32_t n,
                             float4 *__restrict__ X, float4 *__restrict__ V) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = ID[k];
  X[k] = in_pos[i];
  V[k] = in_vel[i];
}

__global__ void k_gather_scalar(const float *__restrict__ src,
                                const uint32_t *__restrict__ ID, uint32_t n,
                                float *__restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  out[ID[k]] = src[k];
}

__global__ void k_iota(uint32_t *__restrict__ dst, uint32_t n) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = k;
}

// sid[k] = the scene whose [p_begin, p_end) holds slot k (scenes in slot
// order, found by binary search on p_begin).
__global__ void k_scene_ids(const SceneDesc *__restrict__ scenes, uint32_t nscenes, uint32_t n,
                            uint16_t *__restrict__ sid) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t lo = 0, hi = nscenes - 1u;  // largest s with p_begin <= k
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1u) >> 1;
    if (scenes[mid].p_begin <= k) lo = mid;
    else hi = mid - 1u;
  }
  sid[k] = (uint16_t)lo;
}

inline uint32_t blocks_for(uint64_t n, uint32_t t) {
  return (uint32_t)((n + t - 1) / t);
}

NbrCtx make_ctx(const DeviceState &d, const PaperConsts &c, const uint16_t *sid) {
  NbrCtx nc;
  nc.nbr4 = d.nbr;
  nc.cnt = d.nbr_cnt;
  nc.skeys = d.skeys;
  nc.off = d.offsets;
  nc.X2 = d.X2;
  nc.V2 = d.V2;
  nc.scenes = d.scenes;
  nc.sid = sid;
  nc.err = d.err;
  nc.n = c.n;
  nc.maxn = c.maxn;
  nc.dt = c.dt;
  nc.h2 = c.h2;
  return nc;
}

}  // namespace

cudaError_t paper_predict_hash(const float4 *X, const float4 *V, uint32_t n,
                               const PaperConsts &c, const SceneDesc *scenes,
                               const uint16_t *sid, uint32_t *keys,
                               const SortPlan &plan, uint32_t *sort_scratch,
                               cudaStream_t st) {
  k_predict_hash<<<min(blocks_for(n, 256), kStrideCtas), 256, 0, st>>>(
      X, V, n, c, scenes, sid, keys, plan.passes, sort_scratch + plan.off_hist);
  return cudaGetLastError();
}

cudaError_t paper_reorder(const uint32_t *perm, const float4 *X,
                          const float4 *V, const uint32_t *ID, uint32_t n,
                          const PaperConsts &c, float4 *X2, float4 *V2,
                          uint32_t *ID2, float4 *P, float4 *D,
                          cudaStream_t st) {
  k_reorder<<<blocks_for(n, 256), 256, 0, st>>>(perm, X, V, ID, n, c, X2, V2, ID2, P, D);
  return cudaGetLastError();
}

// Launches KERNEL<threads, loads in flight> (or KERNEL<threads> for the list
// builds) in the shape d.tune gives for KIND, between the tuner's events
// when its timer is attached.
#define PBF_GATHER_LAUNCH(KERNEL, KIND, ...)                                          \
  do {                                                                                 \
    const int slot_ = d.timer ? d.timer->begin(KIND, st) : -1;                         \
    switch (d.tune.block[KIND] * kBatchCodes + d.tune.batch[KIND]) {                   \
      case 0: KERNEL<64, 4><<<blocks_for(c.n, 64), 64, 0, st>>>(__VA_ARGS__); break;    \
      case 1: KERNEL<64, 8><<<blocks_for(c.n, 64), 64, 0, st>>>(__VA_ARGS__); break;    \
      case 2: KERNEL<128, 4><<<blocks_for(c.n, 128), 128, 0, st>>>(__VA_ARGS__); break; \
      case 3: KERNEL<128, 8><<<blocks_for(c.n, 128), 128, 0, st>>>(__VA_ARGS__); break; \
      case 4: KERNEL<256, 4><<<blocks_for(c.n, 256), 256, 0, st>>>(__VA_ARGS__); break; \
      case 5: KERNEL<256, 8><<<blocks_for(c.n, 256), 256, 0, st>>>(__VA_ARGS__); break; \
      default: return cudaErrorInvalidValue;                                           \
    }                                                                                  \
    if (d.timer) d.timer->end(slot_, st);                                              \
  } while (0)

#define PBF_BUILD_LAUNCH(KERNEL, KIND, ...)                                           \
  do {                                                                                 \
    const int slot_ = d.timer ? d.timer->begin(KIND, st) : -1;                         \
    switch (d.tune.block[KIND]) {                                                      \
      case 0: KERNEL<64><<<blocks_for(c.n, 64), 64, 0, st>>>(__VA_ARGS__); break;       \
      case 1: KERNEL<128><<<blocks_for(c.n, 128), 128, 0, st>>>(__VA_ARGS__); break;    \
      case 2: KERNEL<256><<<blocks_for(c.n, 256), 256, 0, st>>>(__VA_ARGS__); break;    \
      default: return cudaErrorInvalidValue;                                           \
    }                                                                                  \
    if (d.timer) d.timer->end(slot_, st);                                              \
  } while (0)

cudaError_t paper_nbr_build(const DeviceState &d, const PaperConsts &c,
                            const uint16_t *sid, cudaStream_t st) {
  PBF_BUILD_LAUNCH(k_nbr_build, kKindNbr, d.P, make_ctx(d, c, sid), c, d.nbr, d.nbr_cnt);
  return cudaGetLastError();
}

cudaError_t paper_nbr_lambda(const DeviceState &d, const PaperConsts &c,
                             const uint16_t *sid, cudaStream_t st) {
  PBF_BUILD_LAUNCH(k_nbr_lambda, kKindNbrLambda, d.P, make_ctx(d, c, sid), c, d.nbr, d.nbr_cnt,
                   d.Q, d.R);
  return cudaGetLastError();
}

cudaError_t paper_lambda(const DeviceState &d, const PaperConsts &c,
                         const uint16_t *sid, cudaStream_t st) {
  PBF_GATHER_LAUNCH(k_lambda, kKindLambda, d.P, make_ctx(d, c, sid), c, d.Q, d.R);
  return cudaGetLastError();
}

cudaError_t paper_delta(const DeviceState &d, const PaperConsts &c,
                        const uint16_t *sid, bool last, cudaStream_t st) {
  PBF_GATHER_LAUNCH(k_delta, kKindDelta, d.Q, make_ctx(d, c, sid), c, d.D, d.P, d.R, d.U,
                    last ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t paper_vorticity(const DeviceState &d, const PaperConsts &c,
                            const uint16_t *sid, cudaStream_t st) {
  PBF_GATHER_LAUNCH(k_vorticity, kKindVorticity, d.P, d.U, make_ctx(d, c, sid), c, d.W, d.D);
  return cudaGetLastError();
}

cudaError_t paper_xsph_commit(const DeviceState &d, const PaperConsts &c,
                              const uint16_t *sid, cudaStream_t st) {
  PBF_GATHER_LAUNCH(k_xsph_commit, kKindXsph, d.D, d.U, d.W, make_ctx(d, c, sid), c, d.ID2,
                    d.X, d.V, d.ID);
  return cudaGetLastError();
}

#undef PBF_GATHER_LAUNCH
#undef PBF_BUILD_LAUNCH

cudaError_t gather_to_input_order(const float4 *X, const float4 *V,
                                  const uint32_t *ID, uint32_t n,
                                  float4 *out_pos, float4 *out_vel,
                                  cudaStream_t st) {
  k_gather_out<<<blocks_for(n, 256), 256, 0, st>>>(X, V, ID, n, out_pos, out_vel);
  return cudaGetLastError();
}

cudaError_t scatter_from_input_order(const float4 *in_pos,
                                     const float4 *in_vel, const uint32_t *ID,
                                     uint32_t n, float4 *X, float4 *V,
                                     cudaStream_t st) {
  k_scatter_in<<<blocks_for(n, 256), 256, 0, st>>>(in_pos, in_vel, ID, n, X, V);
  return cudaGetLastError();
}

cudaError_t gather_scalar_to_input_order(const float *src, const uint32_t *ID,
                                         uint32_t n, float *out,
                                         cudaStream_t st) {
  k_gather_scalar<<<blocks_for(n, 256), 256, 0, st>>>(src, ID, n, out);
  return cudaGetLastError();
}

cudaError_t iota_u32(uint32_t *dst, uint32_t n, cudaStream_t st) {
  k_iota<<<blocks_for(n, 256), 256, 0, st>>>(dst, n);
  return cudaGetLastError();
}

cudaError_t iota_range(uint32_t *dst, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  return iota_u32(dst, n, st);
}

cudaError_t scene_ids(const SceneDesc *scenes, uint32_t nscenes, uint32_t n, uint16_t *sid,
                      cudaStream_t st) {
  if (n == 0 || nscenes == 0) return cudaSuccess;
  k_scene_ids<<<blocks_for(n, 256), 256, 0, st>>>(scenes, nscenes, n, sid);
  return cudaGetLastError();
}


}  // namespace pbf
