// Device code shared by the gather passes of the paper equations
// (PBF_MODE_PAPER): the neighbour walks, the pair arithmetic of every pass
// and each pass's per-particle epilogue.  Both launch paths include it -- the
// passes that gather neighbours through L1 (pbf_paper.cu) and the passes that
// stage each tile's neighbourhood in shared memory (pbf_tile.cu) -- so a
// particle's arithmetic is the same operations in the same order whichever
// path runs it, and the two give the same bits.  nvcc only.
#pragma once

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
  uint32_t *cnt_max;  // largest neighbour count of the step (may be null)
  uint32_t n, maxn;
  float dt, h2;
};

// Folds the neighbour counts of the calling warp's active threads into the
// step's largest count: one atomic per warp.
__device__ __forceinline__ void record_count(uint32_t *cnt_max, uint32_t cnt) {
  const unsigned m = __activemask();
  const uint32_t mx = __reduce_max_sync(m, cnt);
  if (cnt_max && (threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicMax(cnt_max, mx);
}

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

// All arithmetic on pair and particle values below is written with
// explicitly rounded operations (__fadd_rn, __fmul_rn, __fmaf_rn, ...): the
// compiler may not contract or reassociate them, so every kernel that
// evaluates a pair -- fused or not, any launch shape, staged or through L1 --
// rounds it the same way and gets the same bits.  (Left to itself, nvcc
// contracts a*b + c*d into an FMA on either product, and its choice can
// differ from one kernel to another.)
struct Sep {
  float x, y, z, r2;  // p_k - p_j and its squared length
};
__device__ __forceinline__ Sep separation(const float4 &a, const float4 &b) {
  Sep r;
  r.x = __fsub_rn(a.x, b.x);
  r.y = __fsub_rn(a.y, b.y);
  r.z = __fsub_rn(a.z, b.z);
  r.r2 = __fmaf_rn(r.z, r.z, __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x)));
  return r;
}
__device__ __forceinline__ Sep separation(const float3 &a, const float3 &b) {
  return separation(make_float4(a.x, a.y, a.z, 0.f), make_float4(b.x, b.y, b.z, 0.f));
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
    if (is_pair(separation(pk, start_position(c, j)).r2, c.h2)) f(j);
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
    if (e & 1) r = __fmul_rn(r, b);
    b = __fmul_rn(b, b);
    e >>= 1;
  }
  return r;
}

// -k h^2 (W(r)/W(dq h))^n with W(r)/W(dq h) = ((h^2-r^2)/(h^2-dq^2 h^2))^3;
// kTwelve: the exponent 3n is 12 (n = 4, the paper's choice).
template <bool kTwelve>
__device__ __forceinline__ float scorr_term(float r2, const PaperConsts &c) {
  const float ratio = __fmul_rn(__fsub_rn(c.h2, r2), c.inv_scorr_den);
  if constexpr (kTwelve) {
    const float r3 = __fmul_rn(__fmul_rn(ratio, ratio), ratio);
    const float r6 = __fmul_rn(r3, r3);
    return __fmul_rn(-c.scorr_k, __fmul_rn(r6, r6));
  } else {
    return __fmul_rn(-c.scorr_k, ipow(ratio, c.scorr_n3));
  }
}

// Spiky gradient factor: grad_i W(r_vec) = f * r_vec, f = -S (h-r)^2 / r,
// for a pair (r^2 normal, so the MUFU reciprocal square root without the
// subnormal-input path equals rsqrtf).
__device__ __forceinline__ float spiky_factor(float r2, const PaperConsts &c) {
  float rinv;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rinv) : "f"(r2));
  const float hr = __fmaf_rn(-r2, rinv, c.h);  // h - r, one rounding (r close to h cancels)
  return __fmul_rn(__fmul_rn(__fmul_rn(-c.spiky, hr), hr), rinv);
}

// Poly6 kernel value W(r) = poly6 (h^2 - r^2)^3.
__device__ __forceinline__ float poly6_value(float r2, const PaperConsts &c) {
  const float t = __fsub_rn(c.h2, r2);
  return __fmul_rn(__fmul_rn(__fmul_rn(c.poly6, t), t), t);
}

struct LambdaAcc {
  float rho, gx, gy, gz, s;
  __device__ __forceinline__ void add(const Sep &r, const PaperConsts &c) {
    const float t = __fsub_rn(c.h2, r.r2);
    rho = __fmaf_rn(__fmul_rn(__fmul_rn(c.poly6, t), t), t, rho);
    const float f = spiky_factor(r.r2, c);
    gx = __fmaf_rn(f, r.x, gx);
    gy = __fmaf_rn(f, r.y, gy);
    gz = __fmaf_rn(f, r.z, gz);
    s = __fmaf_rn(__fmul_rn(f, f), r.r2, s);
  }
  __device__ __forceinline__ float lambda(const PaperConsts &c) const {
    const float C = __fmaf_rn(rho, c.inv_rho0, -1.0f);
    const float g2 = __fmaf_rn(gz, gz, __fmaf_rn(gy, gy, __fmaf_rn(gx, gx, s)));
    const float den = __fmul_rn(g2, __fmul_rn(c.inv_rho0, c.inv_rho0));
    return __fdiv_rn(-C, __fadd_rn(den, c.relax_eps));
  }
};

// Calls member(j, sep) for every slot j that forms a pair with k
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
          const Sep r = separation(pk, d[e]);
          if (is_pair(r.r2, c.h2)) member(j + e, r);
        }
      }
      if (j < b) {
        float4 d[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) d[e] = __ldg(&P[min(j + e, b - 1u)]);
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          const Sep r = separation(pk, d[e]);
          if (j + e < b && is_pair(r.r2, c.h2)) member(j + e, r);
        }
      }
    }
  }
}

// scan_members with the member work taken out of the candidate loop: each
// row is tested 32 candidates at a time into a membership mask (bit e for
// candidate c0 + e), then member(j) runs for the mask's set bits in
// ascending order -- the same members in the same order as scan_members.
// Lanes of a warp test candidates of different cells, so in scan_members
// the member branch runs for nearly every candidate (some lane of the warp
// has a member); here the candidate loop is the load, the distance and one
// bit in every lane, and the member work runs as many times per chunk as
// the warp's largest member count in it.
template <typename F>
__device__ __forceinline__ void scan_members_masked(const float4 &pk, uint32_t key,
                                                    const SceneDesc &s,
                                                    const uint32_t *__restrict__ off,
                                                    const float4 *__restrict__ P,
                                                    const PaperConsts &c, F &&member) {
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
      for (uint32_t c0 = a; c0 < b; c0 += 32u) {
        const uint32_t c1 = min(c0 + 32u, b);
        uint32_t m = 0, bit = 1u;
        uint32_t j = c0;
        for (; j + 4u <= c1; j += 4, bit <<= 4) {
          const float4 *__restrict__ q = P + j;
          float4 d[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) d[e] = __ldg(q + e);
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (is_pair(separation(pk, d[e]).r2, c.h2)) m |= bit << e;
        }
        if (j < c1) {
          float4 d[3];
#pragma unroll
          for (int e = 0; e < 3; ++e) d[e] = __ldg(&P[min(j + e, c1 - 1u)]);
#pragma unroll
          for (int e = 0; e < 3; ++e)
            if (j + e < c1 && is_pair(separation(pk, d[e]).r2, c.h2)) m |= bit << e;
        }
        while (m) {
          const uint32_t e = (uint32_t)__ffs(m) - 1u;
          m &= m - 1u;
          member(c0 + e);
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

// ------------------------------------------------------------ pair terms --
// Lambda pass: density, constraint gradient sums over the pairs of k.
__device__ __forceinline__ void lambda_pair(LambdaAcc &acc, const float4 &pk, const float4 &pj,
                                            const PaperConsts &c) {
  const Sep r = separation(pk, pj);
  if (is_pair(r.r2, c.h2)) acc.add(r, c);
}
__device__ __forceinline__ void lambda_commit(uint32_t k, const float4 &pk, const LambdaAcc &acc,
                                              const PaperConsts &c, float4 *__restrict__ Q,
                                              float *__restrict__ R) {
  Q[k] = make_float4(pk.x, pk.y, pk.z, acc.lambda(c));
  R[k] = acc.rho;
}

// Delta-p pass: sum of (lambda_k + lambda_j + s_corr) grad W over the pairs.
struct DeltaAcc {
  float sx, sy, sz;
  template <bool kTwelve>
  __device__ __forceinline__ void pair(const float4 &qk, const float4 &qj, const PaperConsts &c) {
    const Sep r = separation(qk, qj);
    if (is_pair(r.r2, c.h2)) {
      const float wgt = __fmul_rn(__fadd_rn(__fadd_rn(qk.w, qj.w), scorr_term<kTwelve>(r.r2, c)),
                                  spiky_factor(r.r2, c));
      sx = __fmaf_rn(wgt, r.x, sx);
      sy = __fmaf_rn(wgt, r.y, sy);
      sz = __fmaf_rn(wgt, r.z, sz);
    }
  }
};
// delta-p, collision response (clamp to the admissible box with the moving
// x-min wall), Jacobi update of d and p; the last iteration also writes the
// velocity d/dt and 1/rho for the velocity passes.
__device__ __forceinline__ void delta_commit(uint32_t k, const DeltaAcc &a, const NbrCtx &nc,
                                             const PaperConsts &c, float4 *__restrict__ D,
                                             float4 *__restrict__ P, const float *__restrict__ R,
                                             float4 *__restrict__ U, int last) {
  const float4 x = load_own(&nc.X2[k]);
  const float4 d0 = load_own(&D[k]);
  float3 d = make_float3(__fmaf_rn(a.sx, c.inv_rho0, d0.x), __fmaf_rn(a.sy, c.inv_rho0, d0.y),
                         __fmaf_rn(a.sz, c.inv_rho0, d0.z));
  float3 p = add3(x, d);
  const SceneDesc &sc = scene_of(nc.scenes, nc.sid, k);
  const float lo_x = __fadd_rn(sc.lo[0], sc.wave);
  if (p.x < lo_x) { d.x = __fsub_rn(lo_x, x.x); p.x = __fadd_rn(x.x, d.x); }
  else if (p.x > sc.hi[0]) { d.x = __fsub_rn(sc.hi[0], x.x); p.x = __fadd_rn(x.x, d.x); }
  if (p.y < sc.lo[1]) { d.y = __fsub_rn(sc.lo[1], x.y); p.y = __fadd_rn(x.y, d.y); }
  else if (p.y > sc.hi[1]) { d.y = __fsub_rn(sc.hi[1], x.y); p.y = __fadd_rn(x.y, d.y); }
  if (p.z < sc.lo[2]) { d.z = __fsub_rn(sc.lo[2], x.z); p.z = __fadd_rn(x.z, d.z); }
  else if (p.z > sc.hi[2]) { d.z = __fsub_rn(sc.hi[2], x.z); p.z = __fadd_rn(x.z, d.z); }
  D[k] = make_float4(d.x, d.y, d.z, 0.0f);
  P[k] = make_float4(p.x, p.y, p.z, 0.0f);
  if (last)
    U[k] = make_float4(__fdiv_rn(d.x, c.dt), __fdiv_rn(d.y, c.dt), __fdiv_rn(d.z, c.dt),
                       __fdiv_rn(1.0f, load_own(&R[k])));
}

// A neighbour's (position, velocity) as the velocity passes read it.
struct PU {
  float4 p, u;
};

// a x b, component by component with one rounding per product and sum.
__device__ __forceinline__ float cross_component(float a1, float b2, float a2, float b1) {
  return __fmaf_rn(a1, b2, __fmul_rn(-a2, b1));  // a1 b2 - a2 b1
}

// Vorticity pass, which also carries the neighbour sums the XSPH pass would
// otherwise gather velocities for:
//   omega_k = sum (1/rho_j) grad W x (v_j - v_k),
//   S_k     = sum (1/rho_j) grad W,
//   X_k     = sum (1/rho_j) W (v_j - v_k)   (XSPH viscosity).
// With |omega_j| / rho_j gathered in the next pass, the vorticity location
// vector eta_k = sum (1/rho_j)(|omega_j| - |omega_k|) grad W is
// sum (|omega_j|/rho_j) grad W - |omega_k| S_k, so that pass gathers one
// float4 per neighbour instead of two.
struct VortAcc {
  float wx, wy, wz, sx, sy, sz, xx, xy, xz;
  __device__ __forceinline__ void pair(const float4 &pk, const float4 &uk, const PU &d,
                                       const PaperConsts &c) {
    const Sep r = separation(pk, d.p);
    if (is_pair(r.r2, c.h2)) {
      const float4 uj = d.u;
      const float f = __fmul_rn(spiky_factor(r.r2, c), uj.w);
      const float gx = __fmul_rn(f, r.x), gy = __fmul_rn(f, r.y), gz = __fmul_rn(f, r.z);
      const float ux = __fsub_rn(uj.x, uk.x), uy = __fsub_rn(uj.y, uk.y),
                  uz = __fsub_rn(uj.z, uk.z);
      wx = __fadd_rn(wx, cross_component(gy, uz, gz, uy));
      wy = __fadd_rn(wy, cross_component(gz, ux, gx, uz));
      wz = __fadd_rn(wz, cross_component(gx, uy, gy, ux));
      sx = __fadd_rn(sx, gx);
      sy = __fadd_rn(sy, gy);
      sz = __fadd_rn(sz, gz);
      const float wp = __fmul_rn(poly6_value(r.r2, c), uj.w);
      xx = __fmaf_rn(wp, ux, xx);
      xy = __fmaf_rn(wp, uy, xy);
      xz = __fmaf_rn(wp, uz, xz);
    }
  }
};
__device__ __forceinline__ float norm3(float x, float y, float z) {
  return __fsqrt_rn(__fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x))));
}
// Writes (omega_k, |omega_k|), (p_k, |omega_k| / rho_k) for the XSPH pass to
// gather, and k's own sums X_k and S_k.
__device__ __forceinline__ void vort_commit(uint32_t k, const float4 &pk, const float4 &uk,
                                            const VortAcc &a, float4 *__restrict__ Wo,
                                            float4 *__restrict__ PW, float4 *__restrict__ XS,
                                            float4 *__restrict__ SS) {
  const float wn = norm3(a.wx, a.wy, a.wz);
  Wo[k] = make_float4(a.wx, a.wy, a.wz, wn);
  PW[k] = make_float4(pk.x, pk.y, pk.z, __fmul_rn(wn, uk.w));
  XS[k] = make_float4(a.xx, a.xy, a.xz, 0.0f);
  SS[k] = make_float4(a.sx, a.sy, a.sz, 0.0f);
}

// XSPH + vorticity-confinement pass: E_k = sum (|omega_j|/rho_j) grad W over
// the pairs (pj.w = |omega_j|/rho_j).
struct XsphAcc {
  float ex, ey, ez;
  __device__ __forceinline__ void pair(const float4 &pk, const float4 &pj, const PaperConsts &c) {
    const Sep r = separation(pk, pj);
    if (is_pair(r.r2, c.h2)) {
      const float e = __fmul_rn(spiky_factor(r.r2, c), pj.w);
      ex = __fmaf_rn(e, r.x, ex);
      ey = __fmaf_rn(e, r.y, ey);
      ez = __fmaf_rn(e, r.z, ez);
    }
  }
};
// eta = E - |omega_k| S_k; v = v + dt f_vorticity + c_xsph X_k with
// f_vorticity = eps (eta/|eta|) x omega; commits x (.w = |v|), v (.w = mass)
// and the input index of slot k.
__device__ __forceinline__ void xsph_commit(uint32_t k, const float4 &pk, const float4 &uk,
                                            const float4 &wk, const float4 &xs, const float4 &ss,
                                            const XsphAcc &a, const NbrCtx &nc,
                                            const PaperConsts &c, const uint32_t *__restrict__ ID2,
                                            float4 *__restrict__ X, float4 *__restrict__ V,
                                            uint32_t *__restrict__ ID) {
  const float ex = __fmaf_rn(-wk.w, ss.x, a.ex), ey = __fmaf_rn(-wk.w, ss.y, a.ey),
              ez = __fmaf_rn(-wk.w, ss.z, a.ez);
  const float el2 = __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
  float nx = 0.f, ny = 0.f, nz = 0.f;
  if (el2 > 0.0f) {
    const float inv = rsqrtf(el2);
    nx = __fmul_rn(ex, inv);
    ny = __fmul_rn(ey, inv);
    nz = __fmul_rn(ez, inv);
  }
  const float fx = __fmul_rn(c.vort_eps, cross_component(ny, wk.z, nz, wk.y));
  const float fy = __fmul_rn(c.vort_eps, cross_component(nz, wk.x, nx, wk.z));
  const float fz = __fmul_rn(c.vort_eps, cross_component(nx, wk.y, ny, wk.x));
  const float vx = __fmaf_rn(c.xsph_c, xs.x, __fmaf_rn(c.dt, fx, uk.x));
  const float vy = __fmaf_rn(c.xsph_c, xs.y, __fmaf_rn(c.dt, fy, uk.y));
  const float vz = __fmaf_rn(c.xsph_c, xs.z, __fmaf_rn(c.dt, fz, uk.z));
  X[k] = make_float4(pk.x, pk.y, pk.z, norm3(vx, vy, vz));
  V[k] = make_float4(vx, vy, vz, load_own(&nc.V2[k]).w);
  ID[k] = load_own(&ID2[k]);
}

}  // namespace
}  // namespace pbf
