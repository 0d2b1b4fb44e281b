// Gather passes of the paper equations on staged cell blocks: persistent
// CTAs walk the step's list of occupied blocks of 4 x 4 x 4 cells; for each
// block one warp copies the neighbourhood the block's particles read (the
// positions, or whatever the pass gathers) into shared memory with bulk
// asynchronous copies (cp.async.bulk, completion on an mbarrier), and every
// thread then walks its particles' neighbour lists out of shared memory.
// The reference's kernels these passes replace are the same as
// pbf_paper.cu's: compute_scaling.cl:32-128 (lambda), compute_delta.cl:30-123
// (delta-p), apply_vorticity_and_viscosity.cl:28-101 (velocity passes), each
// of which walks the 27 cells around a particle.
//
// Why stage: the L1 gather passes of pbf_paper.cu are bound by the L1 data
// stage.  On GB300 a warp-wide 16-byte gather of 32 neighbours through L1
// costs about 12 data-stage wavefronts (the lanes touch ~19 sectors in ~8
// lines), and 28% of the sectors miss L1; the same index pattern out of
// shared memory costs about 9 wavefronts and never misses.
//
// The neighbourhood of a block.  Particles are sorted by cell key
// cx + nx (cy + ny cz) (scene-major in a batch), so each grid row (y, z) of
// cells is a contiguous slot range.  A block [x0, x1) x [y0, y1) x [z0, z1)
// owns 16 row segments (its rows, cells [x0, x1)); its particles' 27 candidate
// cells lie in the 36 rows (y, z) in [y0-1, y1] x [z0-1, z1], cells
// [x0-1, x1] of each -- 36 contiguous halo segments, staged back to back (an
// index into this staging is a "staged index").  About 3.4 candidates are
// staged per own particle (6^3 cells for 4^3), against ~10 for a run of 128
// sorted slots.  A block whose halo holds more than kStageCap candidates is
// not staged: its passes gather through L1 as pbf_paper.cu does.
//
// Lists.  In a staged block the list build writes each neighbour as its
// 16-bit staged index, eight per 16-byte word (word g of particle k at
// nbr4[g*N + k], as the 32-bit lists of pbf_paper.cu), in the same order as
// those lists (rows by (dz, dy), slots ascending); in an unstaged block it
// writes the 32-bit lists.  The last word of a set is padded with the
// particle's own entry, which the pair test drops (r^2 = 0).  A particle with
// more neighbours than the list capacity re-derives its set from the cells in
// every pass, as in pbf_paper.cu.  Every pass evaluates each particle in one
// thread with the pair functions and epilogues of pbf_paper.cuh, in the list
// order, so the staged path gives the same bits as the L1 path; the order of
// blocks in the work list (atomic appends) changes nothing.
//
// Work list.  k_block_plan (one thread per block of the layout) appends
// every block that owns a particle; the passes run a persistent grid (as many
// CTAs as fit on the SMs) whose CTA c takes list entries c, c + grid, ...
//
// Waits.  A CTA waits for its copies on an mbarrier with a bounded number of
// polls; if the bound runs out it sets kDevErrStage in the simulation's error
// word, waits once more (bounded) for the copies still in flight and returns
// without computing, and the host reports PBF_ERR_DEVICE.
#include <algorithm>
#include <mutex>

#include "pbf_paper.cuh"

namespace pbf {
namespace {

constexpr int kB = kBlockCells;
constexpr int kOwnRows = kB * kB;                  // 16
constexpr int kHaloRows = (kB + 2) * (kB + 2);     // 36
constexpr uint32_t kThreads = 512;                 // threads per CTA
// CTAs per SM the kernels are compiled for (register budget): three for the
// passes staging one array (~49 KB of shared memory each), two for those
// staging two (~97 KB each).
constexpr int kCtasOne = 3;
constexpr int kCtasTwo = 2;
constexpr uint32_t kStageCap = 3072;               // staged candidates per array
constexpr uint32_t kSmemHeader = 1024;             // mbarrier, flags, block tables
constexpr uint32_t kStageSpin = 1u << 20;          // polls of a bounded wait
constexpr uint32_t kSuspendNs = 1000;              // hint per poll

constexpr size_t stage_smem_bytes(int arrays) {
  return kSmemHeader + (size_t)arrays * kStageCap * sizeof(float4);
}

// ---------------------------------------------------------------- PTX ----
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// Makes the initialised barrier visible to the asynchronous (bulk copy) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
// Global -> this CTA's shared memory, `bytes` a multiple of 16, both
// addresses 16-byte aligned; completes `bytes` transactions on the barrier.
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                              uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < kStageSpin; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ------------------------------------------------------------- blocks ----
struct BlockCtx {
  const uint32_t *__restrict__ list;  // occupied blocks
  uint32_t *count;                    // [0] list length, [1] staged, [2] unstaged
  uint32_t cap;                       // list capacity
  uint32_t nscenes;
};

// The scene owning global block index b (scenes in block order).
__device__ __forceinline__ uint32_t scene_of_block(const SceneDesc *__restrict__ scenes,
                                                   uint32_t nscenes, uint32_t b) {
  uint32_t lo = 0, hi = nscenes - 1u;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1u) >> 1;
    if (scenes[mid].block_base <= b) lo = mid;
    else hi = mid - 1u;
  }
  return lo;
}

// Cell range [lo, hi) of a block along one axis.
struct Span {
  int lo, hi;
};
__device__ __forceinline__ Span block_span(uint32_t bi, int cells) {
  const int lo = (int)bi * kB;
  return Span{lo, min(lo + kB, cells)};
}

// Shared-memory layout of a block kernel (dynamic shared memory):
//   [0, 8)       mbarrier
//   [8, 12)      flags of the current block: 1 staged
//   [12, 16)     particles the block owns
//   [32, 320)    halo table: (first slot, staged base) per halo row (36)
//   [320, 384)   own rows: first slot (16)
//   [448, 516)   own rows: exclusive prefix of particle counts (17)
//   [1024, ...)  staged arrays, kStageCap float4 each
struct BlockSmem {
  unsigned char *raw;
  __device__ uint64_t *bar() const { return reinterpret_cast<uint64_t *>(raw); }
  __device__ uint32_t *flags() const { return reinterpret_cast<uint32_t *>(raw + 8); }
  __device__ uint32_t *owned() const { return reinterpret_cast<uint32_t *>(raw + 12); }
  __device__ uint2 *halo() const { return reinterpret_cast<uint2 *>(raw + 32); }
  __device__ uint32_t *own_start() const { return reinterpret_cast<uint32_t *>(raw + 320); }
  __device__ uint32_t *own_prefix() const { return reinterpret_cast<uint32_t *>(raw + 448); }
  __device__ float4 *stage(int a) const {
    return reinterpret_cast<float4 *>(raw + kSmemHeader) + (size_t)a * kStageCap;
  }
};
static_assert(32 + kHaloRows * 8 <= 320, "halo table overlaps the own rows");
static_assert(448 + (kOwnRows + 1) * 4 <= (int)kSmemHeader, "block tables beyond the header");

// One warp describes block `blk` into shared memory -- own rows with their
// particle counts, halo rows with their staged bases -- and, when the halo
// fits the staging, issues its bulk copies (NA source arrays).
template <int NA>
__device__ __forceinline__ void describe_block(const NbrCtx &nc, const BlockCtx &bc, uint32_t blk,
                                               const float4 *const (&src)[NA], const BlockSmem &sm,
                                               uint32_t bar, uint32_t lane) {
  const uint32_t si = nc.sid ? scene_of_block(nc.scenes, bc.nscenes, blk) : 0u;
  const SceneDesc &s = nc.scenes[si];
  const int nx = s.ncell[0], ny = s.ncell[1], nz = s.ncell[2];
  const uint32_t b = blk - s.block_base;
  const uint32_t nbx = blocks_along(nx), nby = blocks_along(ny);
  const Span sx = block_span(b % nbx, nx), sy = block_span((b / nbx) % nby, ny),
             sz = block_span(b / (nbx * nby), nz);
  // own rows: lane r < 16 -> (y0 + r % 4, z0 + r / 4)
  uint32_t own_first = 0u, own_len = 0u;
  if (lane < (uint32_t)kOwnRows) {
    const int y = sy.lo + (int)(lane % kB), z = sz.lo + (int)(lane / kB);
    if (y < sy.hi && z < sz.hi) {
      const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
      own_first = __ldg(&nc.off[row + sx.lo]);
      own_len = __ldg(&nc.off[row + sx.hi]) - own_first;
    }
  }
  // halo rows h = lane and h = lane + 32 (< 36): (y0-1 + h % 6, z0-1 + h / 6)
  uint2 hs[2] = {make_uint2(0u, 0u), make_uint2(0u, 0u)};
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const uint32_t h = lane + 32u * q;
    if (h < (uint32_t)kHaloRows) {
      const int y = sy.lo - 1 + (int)(h % (kB + 2)), z = sz.lo - 1 + (int)(h / (kB + 2));
      if (y >= 0 && y < ny && z >= 0 && z < nz && y <= sy.hi && z <= sz.hi) {
        const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
        const int xa = max(sx.lo - 1, 0), xb = min(sx.hi + 1, nx);
        hs[q].x = __ldg(&nc.off[row + xa]);
        hs[q].y = __ldg(&nc.off[row + xb]) - hs[q].x;
      }
    }
  }
  // exclusive prefixes: own counts; halo lengths of rows 0..31, then 32..35
  uint32_t own_incl = own_len, halo_incl = hs[0].y, tail_incl = hs[1].y;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t a = __shfl_up_sync(0xffffffffu, own_incl, o);
    const uint32_t h = __shfl_up_sync(0xffffffffu, halo_incl, o);
    const uint32_t t = __shfl_up_sync(0xffffffffu, tail_incl, o);
    if (lane >= (uint32_t)o) {
      own_incl += a;
      halo_incl += h;
      tail_incl += t;
    }
  }
  const uint32_t head = __shfl_sync(0xffffffffu, halo_incl, 31);
  const uint32_t total = head + __shfl_sync(0xffffffffu, tail_incl, 31);
  const uint32_t base0 = halo_incl - hs[0].y, base1 = head + tail_incl - hs[1].y;
  const bool fits = (uint64_t)hs[0].x + hs[0].y <= nc.n && (uint64_t)hs[1].x + hs[1].y <= nc.n;
  const bool ok = __all_sync(0xffffffffu, fits) && total <= kStageCap;
  sm.halo()[lane] = make_uint2(hs[0].x, base0);
  if (lane < (uint32_t)(kHaloRows - 32)) sm.halo()[32 + lane] = make_uint2(hs[1].x, base1);
  if (lane < (uint32_t)kOwnRows) {
    sm.own_start()[lane] = own_first;
    sm.own_prefix()[lane] = own_incl - own_len;
  }
  if (lane == (uint32_t)kOwnRows - 1u) {
    sm.own_prefix()[kOwnRows] = own_incl;
    *sm.owned() = own_incl;
  }
  if (lane == 0) {
    *sm.flags() = ok ? 1u : 0u;
    if (ok) mbar_arrive_expect_tx(bar, total * (uint32_t)sizeof(float4) * NA);
  }
  __syncwarp();
  if (ok) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const uint2 h = hs[q];
      const uint32_t base = q == 0 ? base0 : base1;
      if (h.y) {
#pragma unroll
        for (int a = 0; a < NA; ++a)
          bulk_copy_g2s(smem_addr(sm.stage(a) + base), src[a] + h.x,
                        h.y * (uint32_t)sizeof(float4), bar);
      }
    }
  }
}

// Walks the step's occupied blocks (persistent CTA): stages each block's
// halo (NA arrays), then calls body(slot, own row, staged) once per owned
// particle, particle q of the block in thread q % kThreads.  kCount: count
// the staged and unstaged blocks into bc.count[1], [2].  Returns false when a
// bounded wait ran out (error bit set).
template <int NA, bool kCount = false, typename Body>
__device__ __forceinline__ bool for_each_block(const NbrCtx &nc, const BlockCtx &bc,
                                               const float4 *const (&src)[NA],
                                               const BlockSmem &sm, Body &&body) {
  const uint32_t bar = smem_addr(sm.bar());
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const uint32_t count = min(*reinterpret_cast<volatile uint32_t *>(bc.count), bc.cap);
  uint32_t phase = 0;
  for (uint32_t w = blockIdx.x; w < count; w += gridDim.x) {
    if (tid < 32) describe_block<NA>(nc, bc, __ldg(&bc.list[w]), src, sm, bar, lane);
    __syncthreads();
    const bool staged = *sm.flags() != 0;
    if (kCount && tid == 0) atomicAdd(&bc.count[staged ? 1 : 2], 1u);
    if (staged) {
      const bool done = mbar_wait_bounded(bar, phase);
      if (__syncthreads_or(!done)) {
        if (tid == 0) atomicOr(nc.err, kDevErrStage);
        mbar_wait_bounded(bar, phase);  // let copies still in flight land
        return false;
      }
      phase ^= 1u;
    }
    const uint32_t owned = *sm.owned();
    const uint32_t *pre = sm.own_prefix();
    for (uint32_t q = tid; q < owned; q += kThreads) {
      uint32_t r = 0;  // own row: the last r with pre[r] <= q
#pragma unroll
      for (int step = 8; step > 0; step >>= 1)
        if (pre[r + step] <= q) r += step;
      body(sm.own_start()[r] + (q - pre[r]), r, staged);
    }
    __syncthreads();  // the next block overwrites the tables and the staging
  }
  return true;
}

// For the `cnt` listed neighbours of particle k in a staged block: eight
// 16-bit staged indices per list word, the next word loaded one word ahead;
// the neighbour data of four entries at a time is loaded (load(index))
// before f(data) runs for each, in list order.  Entries past the count in the
// last word are k's own index (dropped by the pair test).
template <typename Load, typename F>
__device__ __forceinline__ void for_each_staged(const NbrCtx &c, uint32_t k, uint32_t cnt,
                                                Load &&load, F &&f) {
  const uint64_t pol = l2_evict_first();
  uint4 cur = load_list_word(&c.nbr4[k], pol);
  for (uint32_t e0 = 0; e0 < cnt; e0 += 8) {
    const uint32_t g = (e0 >> 3) + 1u;
    const uint4 nxt = 8u * g < cnt ? load_list_word(&c.nbr4[(size_t)g * c.n + k], pol) : cur;
    const uint32_t wd[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      if (half == 1 && e0 + 4u >= cnt) break;
      decltype(load(0u)) d[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const uint32_t w = wd[2 * half + (e >> 1)];
        d[e] = load(min((e & 1) ? (w >> 16) : (w & 0xffffu), kStageCap - 1u));
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) f(d[e]);
    }
    cur = nxt;
  }
}

// Appends 16-bit entries to a particle's list, eight per 16-byte word.
struct WordPacker {
  uint4 w;
  uint32_t cnt;
  __device__ __forceinline__ void put(uint32_t e, uint32_t v) {
    const uint32_t bits = (v & 0xffffu) << ((e & 1u) << 4);
    const uint32_t sel = (e >> 1) & 3u;
    w.x |= sel == 0u ? bits : 0u;
    w.y |= sel == 1u ? bits : 0u;
    w.z |= sel == 2u ? bits : 0u;
    w.w |= sel == 3u ? bits : 0u;
  }
  __device__ __forceinline__ void push(uint32_t v, uint4 *__restrict__ out, size_t stride,
                                       uint32_t maxn) {
    put(cnt, v);
    ++cnt;
    if ((cnt & 7u) == 0u) {
      if (cnt <= maxn) out[(size_t)((cnt - 1u) >> 3) * stride] = w;
      w = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  // Pads the last word with `self` and stores it (a set within capacity).
  __device__ __forceinline__ void finish(uint32_t self, uint4 *__restrict__ out, size_t stride,
                                         uint32_t maxn) {
    if ((cnt & 7u) == 0u || cnt > maxn) return;
    for (uint32_t e = cnt; e & 7u; ++e) put(e, self);
    out[(size_t)(cnt >> 3) * stride] = w;
  }
};

// ------------------------------------------------------------- kernels --
// One thread per block of the layout: appends every block that owns a
// particle to the work list.
__global__ void __launch_bounds__(256)
    k_block_plan(NbrCtx nc, uint32_t nscenes, uint32_t nblocks, uint32_t *__restrict__ list,
                 uint32_t *__restrict__ count, uint32_t cap) {
  const uint32_t blk = blockIdx.x * blockDim.x + threadIdx.x;
  if (blk >= nblocks) return;
  const uint32_t si = nc.sid ? scene_of_block(nc.scenes, nscenes, blk) : 0u;
  const SceneDesc &s = nc.scenes[si];
  const int nx = s.ncell[0], ny = s.ncell[1], nz = s.ncell[2];
  const uint32_t b = blk - s.block_base;
  const uint32_t nbx = blocks_along(nx), nby = blocks_along(ny);
  const Span sx = block_span(b % nbx, nx), sy = block_span((b / nbx) % nby, ny),
             sz = block_span(b / (nbx * nby), nz);
  if (sz.lo >= nz) return;  // past the scene's blocks
  uint32_t owned = 0;
  for (int z = sz.lo; z < sz.hi; ++z)
    for (int y = sy.lo; y < sy.hi; ++y) {
      const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
      owned += __ldg(&nc.off[row + sx.hi]) - __ldg(&nc.off[row + sx.lo]);
    }
  if (owned) {
    const uint32_t slot = atomicAdd(count, 1u);
    if (slot < cap) list[slot] = blk;
  }
}

// Neighbour lists of the step.  Staged blocks: 16-bit staged indices from a
// scan of the 27 cells in shared memory; other blocks: the 32-bit lists of
// pbf_paper.cu from a scan through L1.
__global__ void __launch_bounds__(kThreads, kCtasOne)
    k_nbr_build_tile(const float4 *__restrict__ P, NbrCtx nc, BlockCtx bc, PaperConsts c,
                     uint4 *__restrict__ nbr4, uint32_t *__restrict__ nbr_cnt) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const BlockSmem sm{smem_raw};
  const float4 *const src[1] = {P};
  const float4 *__restrict__ stage = sm.stage(0);
  for_each_block<1, true>(nc, bc, src, sm, [&](uint32_t k, uint32_t r, bool staged) {
    const float4 pk = load_own(&P[k]);
    const uint32_t key = load_own(&nc.skeys[k]);
    const SceneDesc &s = scene_of(nc.scenes, nc.sid, k);
    if (!staged) {
      uint32_t *__restrict__ out = reinterpret_cast<uint32_t *>(nbr4) + 4ull * k;
      const size_t stride = 4ull * c.n;
      uint32_t cnt = 0;
      scan_members(pk, key, s, nc.off, P, c, [&](uint32_t j, const Sep &) {
        if (cnt < c.maxn) out[(size_t)(cnt >> 2) * stride + (cnt & 3u)] = j;
        ++cnt;
      });
      pad_list(out, stride, cnt, c.maxn, k);
      nbr_cnt[k] = cnt;
      record_count(nc.cnt_max, cnt);
      return;
    }
    const int nx = s.ncell[0], ny = s.ncell[1], nz = s.ncell[2];
    const uint32_t local = key - s.cell_base;
    const int cx = (int)(local % (uint32_t)nx);
    const uint32_t tr = local / (uint32_t)nx;
    const int cy = (int)(tr % (uint32_t)ny);
    const int cz = (int)(tr / (uint32_t)ny);
    const int x0 = cx > 0 ? cx - 1 : 0;
    const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
    const int ry = (int)(r % kB), rz = (int)(r / kB);  // own row within the block
    const uint2 *__restrict__ halo = sm.halo();
    uint4 *__restrict__ out = nbr4 + k;
    const size_t stride = c.n;
    WordPacker pack{make_uint4(0u, 0u, 0u, 0u), 0u};
    for (int dz = -1; dz <= 1; ++dz) {
      const int z = cz + dz;
      if (z < 0 || z >= nz) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int y = cy + dy;
        if (y < 0 || y >= ny) continue;
        const uint2 hs = halo[(rz + dz + 1) * (kB + 2) + (ry + dy + 1)];  // (first slot, base)
        const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
        const uint32_t a = __ldg(&nc.off[row + x0]) - hs.x + hs.y;
        const uint32_t b = __ldg(&nc.off[row + x1 + 1]) - hs.x + hs.y;
        uint32_t j = a;
        for (; j + 4u <= b; j += 4) {
          float4 d[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) d[e] = stage[min(j + e, kStageCap - 1u)];
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (is_pair(separation(pk, d[e]).r2, c.h2)) pack.push(j + e, out, stride, c.maxn);
        }
        for (; j < b; ++j)
          if (is_pair(separation(pk, stage[min(j, kStageCap - 1u)]).r2, c.h2))
            pack.push(j, out, stride, c.maxn);
      }
    }
    const uint2 own = halo[(rz + 1) * (kB + 2) + (ry + 1)];  // the particle's own row
    pack.finish(k - own.x + own.y, out, stride, c.maxn);
    nbr_cnt[k] = pack.cnt;
    record_count(nc.cnt_max, pack.cnt);
  });
}

__global__ void __launch_bounds__(kThreads, kCtasOne)
    k_lambda_tile(const float4 *__restrict__ P, NbrCtx nc, BlockCtx bc, PaperConsts c,
                  float4 *__restrict__ Q, float *__restrict__ R) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const BlockSmem sm{smem_raw};
  const float4 *const src[1] = {P};
  const float4 *__restrict__ stage = sm.stage(0);
  for_each_block<1>(nc, bc, src, sm, [&](uint32_t k, uint32_t, bool staged) {
    const float4 pk = load_own(&P[k]);
    LambdaAcc acc{c.w_self, 0.f, 0.f, 0.f, 0.f};
    const auto pair = [&](const float4 &pj) { lambda_pair(acc, pk, pj, c); };
    if (staged) {
      const uint32_t cnt = load_own(&nc.cnt[k]);
      if (cnt <= c.maxn)
        for_each_staged(nc, k, cnt, [&](uint32_t i) { return stage[i]; }, pair);
      else
        visit_fallback(nc, k, [&](uint32_t j) { pair(__ldg(&P[j])); });
    } else {
      visit_neighbours<4>(nc, k, [&](uint32_t j) { return __ldg(&P[j]); }, pair);
    }
    lambda_commit(k, pk, acc, c, Q, R);
  });
}

__global__ void __launch_bounds__(kThreads, kCtasOne)
    k_delta_tile(const float4 *__restrict__ Q, NbrCtx nc, BlockCtx bc, PaperConsts c,
                 float4 *__restrict__ D, float4 *__restrict__ P, const float *__restrict__ R,
                 float4 *__restrict__ U, int last) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const BlockSmem sm{smem_raw};
  const float4 *const src[1] = {Q};
  const float4 *__restrict__ stage = sm.stage(0);
  const auto run = [&](auto twelve) {
    for_each_block<1>(nc, bc, src, sm, [&](uint32_t k, uint32_t, bool staged) {
      const float4 qk = load_own(&Q[k]);
      DeltaAcc acc{0.f, 0.f, 0.f};
      const auto pair = [&](const float4 &qj) {
        acc.template pair<decltype(twelve)::value>(qk, qj, c);
      };
      if (staged) {
        const uint32_t cnt = load_own(&nc.cnt[k]);
        if (cnt <= c.maxn)
          for_each_staged(nc, k, cnt, [&](uint32_t i) { return stage[i]; }, pair);
        else
          visit_fallback(nc, k, [&](uint32_t j) { pair(__ldg(&Q[j])); });
      } else {
        visit_neighbours<4>(nc, k, [&](uint32_t j) { return __ldg(&Q[j]); }, pair);
      }
      delta_commit(k, acc, nc, c, D, P, R, U, last);
    });
  };
  if (c.scorr_n3 == 12) run(std::true_type{});
  else run(std::false_type{});
}

__global__ void __launch_bounds__(kThreads, kCtasTwo)
    k_vorticity_tile(const float4 *__restrict__ P, const float4 *__restrict__ U, NbrCtx nc,
                     BlockCtx bc, PaperConsts c, float4 *__restrict__ Wo, float4 *__restrict__ PW,
                     float4 *__restrict__ XS, float4 *__restrict__ SS) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const BlockSmem sm{smem_raw};
  const float4 *const src[2] = {P, U};
  const float4 *__restrict__ sp = sm.stage(0);
  const float4 *__restrict__ su = sm.stage(1);
  for_each_block<2>(nc, bc, src, sm, [&](uint32_t k, uint32_t, bool staged) {
    const float4 pk = load_own(&P[k]);
    const float4 uk = load_own(&U[k]);
    VortAcc acc{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const auto pair = [&](const PU &d) { acc.pair(pk, uk, d, c); };
    if (staged) {
      const uint32_t cnt = load_own(&nc.cnt[k]);
      if (cnt <= c.maxn)
        for_each_staged(nc, k, cnt, [&](uint32_t i) { return PU{sp[i], su[i]}; }, pair);
      else
        visit_fallback(nc, k, [&](uint32_t j) { pair(PU{__ldg(&P[j]), __ldg(&U[j])}); });
    } else {
      visit_neighbours<4>(nc, k, [&](uint32_t j) { return PU{__ldg(&P[j]), __ldg(&U[j])}; },
                          pair);
    }
    vort_commit(k, pk, uk, acc, Wo, PW, XS, SS);
  });
}

__global__ void __launch_bounds__(kThreads, kCtasOne)
    k_xsph_commit_tile(const float4 *__restrict__ PW, const float4 *__restrict__ U,
                       const float4 *__restrict__ Wv, const float4 *__restrict__ XS,
                       const float4 *__restrict__ SS, NbrCtx nc, BlockCtx bc, PaperConsts c,
                       const uint32_t *__restrict__ ID2, float4 *__restrict__ X,
                       float4 *__restrict__ V, uint32_t *__restrict__ ID) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const BlockSmem sm{smem_raw};
  const float4 *const src[1] = {PW};
  const float4 *__restrict__ sp = sm.stage(0);
  for_each_block<1>(nc, bc, src, sm, [&](uint32_t k, uint32_t, bool staged) {
    const float4 pk = load_own(&PW[k]);
    XsphAcc acc{0.f, 0.f, 0.f};
    const auto pair = [&](const float4 &pj) { acc.pair(pk, pj, c); };
    if (staged) {
      const uint32_t cnt = load_own(&nc.cnt[k]);
      if (cnt <= c.maxn)
        for_each_staged(nc, k, cnt, [&](uint32_t i) { return sp[i]; }, pair);
      else
        visit_fallback(nc, k, [&](uint32_t j) { pair(__ldg(&PW[j])); });
    } else {
      visit_neighbours<4>(nc, k, [&](uint32_t j) { return __ldg(&PW[j]); }, pair);
    }
    xsph_commit(k, pk, load_own(&U[k]), load_own(&Wv[k]), load_own(&XS[k]), load_own(&SS[k]), acc,
                nc, c, ID2, X, V, ID);
  });
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
  nc.cnt_max = d.nbr_max;
  nc.n = c.n;
  nc.maxn = c.maxn;
  nc.dt = c.dt;
  nc.h2 = c.h2;
  return nc;
}

BlockCtx make_blocks(const DeviceState &d, uint32_t nscenes) {
  return BlockCtx{d.blk_list, d.blk_count, d.blk_cap, nscenes};
}

// Persistent grid of the kernels staging one array and of those staging
// two: as many CTAs as fit on the device at once.
uint32_t g_grid_one = 0, g_grid_two = 0;
cudaError_t g_init_status = cudaSuccess;
std::once_flag g_init_once;

template <typename K>
cudaError_t fit(K kernel, int arrays, int *per_sm) {
  const int bytes = (int)stage_smem_bytes(arrays);
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  int b = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, (int)kThreads, bytes);
  if (e == cudaSuccess) *per_sm = std::min(*per_sm, b);
  return e;
}

void init_kernels() {
  int dev = 0, sms = 0, one = 1 << 20, two = 1 << 20;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = fit(k_nbr_build_tile, 1, &one);
  if (e == cudaSuccess) e = fit(k_lambda_tile, 1, &one);
  if (e == cudaSuccess) e = fit(k_delta_tile, 1, &one);
  if (e == cudaSuccess) e = fit(k_vorticity_tile, 2, &two);
  if (e == cudaSuccess) e = fit(k_xsph_commit_tile, 1, &one);
  if (e == cudaSuccess) {
    g_grid_one = (uint32_t)(std::max(1, one) * sms);
    g_grid_two = (uint32_t)(std::max(1, two) * sms);
  }
  g_init_status = e;
}

uint32_t grid_for(uint32_t persistent, uint32_t cap) {
  return std::max(1u, std::min(persistent, cap));
}

}  // namespace

cudaError_t tile_init() {
  std::call_once(g_init_once, init_kernels);
  return g_init_status;
}

#define PBF_BLOCK_LAUNCH(KERNEL, KIND, ARRAYS, ...)                                        \
  do {                                                                                    \
    const cudaError_t ie_ = tile_init();                                                  \
    if (ie_ != cudaSuccess) return ie_;                                                   \
    if (c.n == 0) return cudaSuccess;                                                     \
    const int slot_ = d.timer ? d.timer->begin(KIND, st) : -1;                            \
    const uint32_t grid_ = grid_for((ARRAYS) == 1 ? g_grid_one : g_grid_two, d.blk_cap);  \
    KERNEL<<<grid_, kThreads, stage_smem_bytes(ARRAYS), st>>>(__VA_ARGS__);               \
    if (d.timer) d.timer->end(slot_, st);                                                 \
  } while (0)

cudaError_t tile_plan(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                      uint32_t nscenes, cudaStream_t st) {
  if (c.n == 0 || d.blk_total == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d.blk_count, 0, 3 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_block_plan<<<(d.blk_total + 255u) / 256u, 256, 0, st>>>(make_ctx(d, c, sid), nscenes,
                                                            d.blk_total, d.blk_list, d.blk_count,
                                                            d.blk_cap);
  return cudaGetLastError();
}

cudaError_t tile_nbr_build(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                           uint32_t nscenes, cudaStream_t st) {
  PBF_BLOCK_LAUNCH(k_nbr_build_tile, kKindNbr, 1, d.P, make_ctx(d, c, sid),
                   make_blocks(d, nscenes), c, d.nbr, d.nbr_cnt);
  return cudaGetLastError();
}

cudaError_t tile_lambda(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                        uint32_t nscenes, cudaStream_t st) {
  PBF_BLOCK_LAUNCH(k_lambda_tile, kKindLambda, 1, d.P, make_ctx(d, c, sid),
                   make_blocks(d, nscenes), c, d.Q, d.R);
  return cudaGetLastError();
}

cudaError_t tile_delta(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                       uint32_t nscenes, bool last, cudaStream_t st) {
  PBF_BLOCK_LAUNCH(k_delta_tile, kKindDelta, 1, d.Q, make_ctx(d, c, sid), make_blocks(d, nscenes),
                   c, d.D, d.P, d.R, d.U, last ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t tile_vorticity(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                           uint32_t nscenes, cudaStream_t st) {
  PBF_BLOCK_LAUNCH(k_vorticity_tile, kKindVorticity, 2, d.P, d.U, make_ctx(d, c, sid),
                   make_blocks(d, nscenes), c, d.W, d.D, d.Q, d.S);
  return cudaGetLastError();
}

cudaError_t tile_xsph_commit(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                             uint32_t nscenes, cudaStream_t st) {
  PBF_BLOCK_LAUNCH(k_xsph_commit_tile, kKindXsph, 1, d.D, d.U, d.W, d.Q, d.S, make_ctx(d, c, sid),
                   make_blocks(d, nscenes), c, d.ID2, d.X, d.V, d.ID);
  return cudaGetLastError();
}

#undef PBF_BLOCK_LAUNCH

}  // namespace pbf
