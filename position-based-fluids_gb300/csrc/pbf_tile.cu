// Gather passes of the paper equations on staged tiles: each CTA owns a tile
// of 128 consecutive sorted slots, copies the positions (or whatever the pass
// reads of its neighbours) of the tile's whole neighbourhood into shared
// memory with bulk asynchronous copies (cp.async.bulk, completion on an
// mbarrier), and every thread then walks its particle's neighbour list out
// of shared memory.  The reference's kernels these passes replace are the
// same as pbf_paper.cu's: compute_scaling.cl:32-128 (lambda),
// compute_delta.cl:30-123 (delta-p), apply_vorticity_and_viscosity.cl:28-101
// (velocity passes), each of which walks the 27 cells around a particle.
//
// Why stage: the gather passes are bound by the L1 data stage, not by DRAM
// or arithmetic.  On GB300 a warp-wide 16-byte gather of 32 neighbours
// through L1 costs about 12 data-stage wavefronts (the lanes touch ~19
// sectors in ~8 lines), and 28% of the sectors miss L1; the same index
// pattern out of shared memory costs about 9 wavefronts (bank conflicts within
// each quarter-warp) and never misses.
//
// The neighbourhood of a tile.  Particles are sorted by cell key
// cx + nx (cy + ny cz) (scene-major in a batch), so the tile's slots fall in
// at most a few grid rows (y, z): each maximal run of slots in one row is a
// piece, covering cells [xa, xb] of that row.  A particle's 27 candidate cells
// lie in the 9 rows (y+dy, z+dz) around its own, and within each row in
// [cx-1, cx+1] -- a contiguous slot range.  So the union of the
// neighbourhoods of a piece is 9 contiguous slot ranges (segments), one per
// row, cells [xa-1, xb+1]; a tile of P pieces stages 9P segments back to back
// (an index into this staging is a particle's "staged index").  The plan
// kernel (k_tile_plan, once per step after the cell offsets) records them per
// tile; a tile of more than three pieces, or whose segments hold more than
// kStageCap candidates, is not staged and its passes gather through L1 as
// pbf_paper.cu does.
//
// Lists.  In a staged tile the list build writes each neighbour as its 16-bit
// staged index, eight per 16-byte word (word g of particle k at
// nbr4[g*N + k], as the 32-bit lists of pbf_paper.cu), in the same order as
// those lists (rows by (dz, dy), slots ascending); in a tile that is not
// staged it writes the 32-bit lists.  The last word of a set is padded with
// the particle's own entry, which the pair test drops (r^2 = 0).  A particle
// with more than max_neighbours neighbours re-derives its set from the cells
// in every pass, as in pbf_paper.cu.  Every pass evaluates each particle in one
// thread with the pair functions and epilogues of pbf_paper.cuh, in the list
// order, so the staged path gives the same bits as the L1 path.
//
// Waits.  A CTA waits for its copies on an mbarrier with a bounded number of
// polls; if the bound runs out it sets kDevErrStage in the simulation's error
// word, waits once more (bounded) for the copies still in flight and returns
// without computing, and the host reports PBF_ERR_DEVICE.
#include <mutex>

#include "pbf_paper.cuh"

namespace pbf {
namespace {

constexpr uint32_t kTile = kTileSlots;
constexpr uint32_t kMaxPieces = 3;         // grid rows a staged tile may span
constexpr uint32_t kStageCap = 2048;       // staged candidates per array (power of two)
constexpr uint32_t kSmemHeader = 512;      // mbarrier, mode word, segment table
constexpr uint32_t kStageSpin = 1u << 20;  // polls of a bounded wait
constexpr uint32_t kSuspendNs = 1000;      // hint per poll

static_assert(kTileSegs >= 9 * kMaxPieces, "segment table too small");
static_assert(16 + kTileSegs * 8 <= kSmemHeader, "segment table beyond the header");
static_assert((kStageCap & (kStageCap - 1)) == 0, "staged index mask needs a power of two");

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

// ---------------------------------------------------------------- tiles --
struct TileCtx {
  const uint32_t *__restrict__ info;  // per tile: pieces | first slot of pieces 1, 2
  const uint2 *__restrict__ seg;      // per tile: kTileSegs (start slot, length)
  uint32_t n;
};

__device__ __forceinline__ uint32_t info_pieces(uint32_t info) { return info & 3u; }

// Shared-memory layout of a tile kernel (dynamic shared memory):
//   [0, 8)     mbarrier
//   [8, 12)    mode: 1 staged, 0 not staged
//   [12, 16)   tile info word
//   [16, 272)  segment table: (first slot, staged base) per segment
//   [512, ...) staged arrays, kStageCap float4 each
struct TileSmem {
  unsigned char *raw;
  __device__ uint64_t *bar() const { return reinterpret_cast<uint64_t *>(raw); }
  __device__ uint32_t *mode() const { return reinterpret_cast<uint32_t *>(raw + 8); }
  __device__ uint32_t *info() const { return reinterpret_cast<uint32_t *>(raw + 12); }
  __device__ uint2 *seg() const { return reinterpret_cast<uint2 *>(raw + 16); }
  __device__ float4 *stage(int a) const {
    return reinterpret_cast<float4 *>(raw + kSmemHeader) + (size_t)a * kStageCap;
  }
};

// Stages the neighbourhood of tile t: for each of NA source arrays, its
// entries at every segment's slots, back to back.  Returns 1 when staged, 0
// when the tile is not staged (its passes gather through L1), -1 when the
// copies did not complete within the bounded wait (error bit set).  Every
// thread of the CTA calls it.
template <int NA>
__device__ __forceinline__ int stage_tile(const TileCtx &tc, uint32_t t,
                                          const float4 *const (&src)[NA], const TileSmem &sm,
                                          uint32_t *err) {
  const uint32_t bar = smem_addr(sm.bar());
  if (threadIdx.x < 32) {
    const uint32_t lane = threadIdx.x;
    const uint32_t info = __ldg(&tc.info[t]);
    const uint32_t nseg = 9u * info_pieces(info);
    const uint2 sg = lane < nseg ? __ldg(&tc.seg[(size_t)t * kTileSegs + lane]) : make_uint2(0u, 0u);
    uint32_t incl = sg.y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += v;
    }
    const uint32_t base = incl - sg.y;
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    // a plan that does not fit (it never should) leaves the tile unstaged
    const bool bad = __any_sync(0xffffffffu, (uint64_t)sg.x + sg.y > tc.n);
    const bool staged = nseg != 0 && total <= kStageCap && !bad;
    sm.seg()[lane] = make_uint2(sg.x, base);
    if (lane == 0) {
      *sm.mode() = staged ? 1u : 0u;
      *sm.info() = info;
      if (staged) {
        mbar_init(bar, 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(bar, total * (uint32_t)sizeof(float4) * NA);
      }
    }
    __syncwarp();
    if (staged && sg.y) {
#pragma unroll
      for (int a = 0; a < NA; ++a)
        bulk_copy_g2s(smem_addr(sm.stage(a) + base), src[a] + sg.x, sg.y * (uint32_t)sizeof(float4),
                      bar);
    }
  }
  __syncthreads();
  if (*sm.mode() == 0) return 0;
  if (mbar_wait_bounded(bar, 0)) return 1;
  if (threadIdx.x == 0) atomicOr(err, kDevErrStage);
  mbar_wait_bounded(bar, 0);  // let copies still in flight land before the CTA exits
  return -1;
}

// For the `cnt` listed neighbours of particle k in a staged tile: eight 16-bit
// staged indices per list word, the next word loaded one word ahead; the
// neighbour data of four entries at a time is loaded (load(index)) before
// f(data) runs for each, in list order.  Entries past the count in the last
// word are k's own index (dropped by the pair test).
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
      decltype(load(0u)) d[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const uint32_t w = wd[2 * half + (e >> 1)];
        d[e] = load(((e & 1) ? (w >> 16) : w) & (kStageCap - 1u));
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
  __device__ __forceinline__ void push(uint32_t v, uint4 *__restrict__ out, size_t stride,
                                       uint32_t maxn) {
    const uint32_t bits = (v & 0xffffu) << ((cnt & 1u) << 4);
    const uint32_t sel = (cnt >> 1) & 3u;
    w.x |= sel == 0u ? bits : 0u;
    w.y |= sel == 1u ? bits : 0u;
    w.z |= sel == 2u ? bits : 0u;
    w.w |= sel == 3u ? bits : 0u;
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
    const uint32_t last = cnt >> 3;
    for (uint32_t e = cnt; e & 7u; ++e) {
      const uint32_t bits = (self & 0xffffu) << ((e & 1u) << 4);
      const uint32_t sel = (e >> 1) & 3u;
      w.x |= sel == 0u ? bits : 0u;
      w.y |= sel == 1u ? bits : 0u;
      w.z |= sel == 2u ? bits : 0u;
      w.w |= sel == 3u ? bits : 0u;
    }
    out[(size_t)last * stride] = w;
  }
};

// ------------------------------------------------------------- kernels --
// One warp per tile: the rows its slots fall in (pieces), and for each piece
// the 9 segments of its neighbourhood; a tile of more than kMaxPieces pieces
// or more than kStageCap staged candidates is marked unstaged (info 0).
// stats[0] counts staged tiles, stats[1] unstaged ones.
__global__ void __launch_bounds__(32)
    k_tile_plan(NbrCtx nc, uint32_t n, uint32_t *__restrict__ info_out, uint2 *__restrict__ seg_out,
                uint32_t *__restrict__ stats) {
  const uint32_t t = blockIdx.x;
  const uint32_t lane = threadIdx.x;
  const uint32_t s0 = t * kTile;
  const uint32_t cnt = min(kTile, n - s0);
  uint32_t key[4], tag[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const uint32_t i = lane + 32u * m;
    key[m] = 0u;
    tag[m] = 0xffffffffu;
    if (i < cnt) {
      const uint32_t k = s0 + i;
      key[m] = __ldg(&nc.skeys[k]);
      const SceneDesc &s = scene_of(nc.scenes, nc.sid, k);
      tag[m] = key[m] - (key[m] - s.cell_base) % (uint32_t)s.ncell[0];  // key of the row's first cell
    }
  }
  uint32_t starts[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const uint32_t up = __shfl_up_sync(0xffffffffu, tag[m], 1);
    const uint32_t wrap = __shfl_sync(0xffffffffu, tag[m > 0 ? m - 1 : 0], 31);
    const uint32_t i = lane + 32u * m;
    const uint32_t prev = lane > 0 ? up : wrap;
    const bool is_start = i < cnt && (i == 0 || tag[m] != prev);
    starts[m] = __ballot_sync(0xffffffffu, is_start);
  }
  // first slots of the first kMaxPieces + 1 pieces (warp-uniform)
  uint32_t st[kMaxPieces + 1];
  uint32_t np = 0;
#pragma unroll
  for (uint32_t p = 0; p <= kMaxPieces; ++p) st[p] = cnt;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    uint32_t b = starts[m];
    while (b && np <= kMaxPieces) {
      const uint32_t i = 32u * m + (uint32_t)(__ffs(b) - 1);
      st[0] = np == 0 ? i : st[0];
      st[1] = np == 1 ? i : st[1];
      st[2] = np == 2 ? i : st[2];
      st[3] = np == 3 ? i : st[3];
      ++np;
      b &= b - 1u;
    }
  }
  const bool few = np <= kMaxPieces;
  // lane l < 9 np: segment q = l % 9 of piece p = l / 9
  const uint32_t p = lane / 9u, q = lane % 9u;
  const bool mine = few && lane < 9u * np;
  const uint32_t a = p == 0 ? st[0] : (p == 1 ? st[1] : st[2]);
  const uint32_t bnext = p == 0 ? st[1] : (p == 1 ? st[2] : st[3]);
  const uint32_t b = (mine ? bnext : 1u) - 1u;  // last slot of the piece
  // keys at slots a and b (any lane's register m = slot >> 5)
  uint32_t ka = 0u, kb = 0u;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const uint32_t xa = __shfl_sync(0xffffffffu, key[m], a & 31u);
    const uint32_t xb = __shfl_sync(0xffffffffu, key[m], b & 31u);
    if ((a >> 5) == (uint32_t)m) ka = xa;
    if ((b >> 5) == (uint32_t)m) kb = xb;
  }
  uint32_t start = 0u, len = 0u;
  if (mine) {
    const SceneDesc &s = scene_of(nc.scenes, nc.sid, s0 + a);
    const uint32_t nx = (uint32_t)s.ncell[0], ny = (uint32_t)s.ncell[1], nz = (uint32_t)s.ncell[2];
    const uint32_t la = ka - s.cell_base, lb = kb - s.cell_base;
    const uint32_t xa = la % nx, xb = lb % nx, r = la / nx;
    const int y = (int)(r % ny) + (int)(q % 3u) - 1;
    const int z = (int)(r / ny) + (int)(q / 3u) - 1;
    if (y >= 0 && y < (int)ny && z >= 0 && z < (int)nz) {
      const uint32_t row = s.cell_base + nx * ((uint32_t)y + ny * (uint32_t)z);
      const uint32_t x0 = xa > 0u ? xa - 1u : 0u;
      const uint32_t x1 = xb + 1u < nx ? xb + 1u : nx - 1u;
      start = __ldg(&nc.off[row + x0]);
      len = __ldg(&nc.off[row + x1 + 1u]) - start;
    }
  }
  uint32_t total = len;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
  const bool staged = few && total <= kStageCap;
  if (staged && lane < 9u * np) seg_out[(size_t)t * kTileSegs + lane] = make_uint2(start, len);
  if (lane == 0) {
    const uint32_t s1 = np > 1 ? st[1] : 0xffu, s2 = np > 2 ? st[2] : 0xffu;
    info_out[t] = staged ? (np | (s1 << 8) | (s2 << 16)) : 0u;
    atomicAdd(&stats[staged ? 0 : 1], 1u);
  }
}

// Neighbour lists of the step.  Staged tiles: 16-bit staged indices from a
// scan of the 27 cells in shared memory; other tiles: the 32-bit lists of
// pbf_paper.cu from a scan through L1.
__global__ void __launch_bounds__(kTile)
    k_nbr_build_tile(const float4 *__restrict__ P, NbrCtx nc, TileCtx tc, PaperConsts c,
                     uint4 *__restrict__ nbr4, uint32_t *__restrict__ nbr_cnt) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TileSmem sm{smem_raw};
  const float4 *const src[1] = {P};
  const int mode = stage_tile<1>(tc, blockIdx.x, src, sm, nc.err);
  const uint32_t k = blockIdx.x * kTile + threadIdx.x;
  if (mode < 0 || k >= c.n) return;
  const float4 pk = load_own(&P[k]);
  const uint32_t key = load_own(&nc.skeys[k]);
  const SceneDesc &s = scene_of(nc.scenes, nc.sid, k);
  if (mode == 0) {
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
  const float4 *__restrict__ stage = sm.stage(0);
  const uint32_t info = *sm.info();
  const uint32_t i = threadIdx.x;
  const uint32_t piece = (i >= ((info >> 8) & 0xffu) ? 1u : 0u) + (i >= ((info >> 16) & 0xffu) ? 1u : 0u);
  const uint2 *__restrict__ seg = sm.seg() + 9u * piece;
  const int nx = s.ncell[0], ny = s.ncell[1], nz = s.ncell[2];
  const uint32_t local = key - s.cell_base;
  const int cx = (int)(local % (uint32_t)nx);
  const uint32_t tr = local / (uint32_t)nx;
  const int cy = (int)(tr % (uint32_t)ny);
  const int cz = (int)(tr / (uint32_t)ny);
  const int x0 = cx > 0 ? cx - 1 : 0;
  const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
  uint4 *__restrict__ out = nbr4 + k;
  const size_t stride = c.n;
  WordPacker pack{make_uint4(0u, 0u, 0u, 0u), 0u};
  for (int dz = -1; dz <= 1; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= ny) continue;
      const uint2 sg = seg[(dz + 1) * 3 + (dy + 1)];  // (first slot, staged base) of this row
      const uint32_t row = s.cell_base + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
      const uint32_t a = __ldg(&nc.off[row + x0]) - sg.x + sg.y;
      const uint32_t b = __ldg(&nc.off[row + x1 + 1]) - sg.x + sg.y;
      uint32_t j = a;
      for (; j + 4u <= b; j += 4) {
        float4 d[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) d[e] = stage[(j + e) & (kStageCap - 1u)];
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (is_pair(separation(pk, d[e]).r2, c.h2)) pack.push(j + e, out, stride, c.maxn);
      }
      for (; j < b; ++j) {
        if (is_pair(separation(pk, stage[j & (kStageCap - 1u)]).r2, c.h2))
          pack.push(j, out, stride, c.maxn);
      }
    }
  }
  const uint2 own = seg[4];  // the particle's own row
  pack.finish(k - own.x + own.y, out, stride, c.maxn);
  nbr_cnt[k] = pack.cnt;
  record_count(nc.cnt_max, pack.cnt);
}

__global__ void __launch_bounds__(kTile)
    k_lambda_tile(const float4 *__restrict__ P, NbrCtx nc, TileCtx tc, PaperConsts c,
                  float4 *__restrict__ Q, float *__restrict__ R) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TileSmem sm{smem_raw};
  const float4 *const src[1] = {P};
  const int mode = stage_tile<1>(tc, blockIdx.x, src, sm, nc.err);
  const uint32_t k = blockIdx.x * kTile + threadIdx.x;
  if (mode < 0 || k >= c.n) return;
  const float4 pk = load_own(&P[k]);
  LambdaAcc acc{c.w_self, 0.f, 0.f, 0.f, 0.f};
  const auto pair = [&](const float4 &pj) { lambda_pair(acc, pk, pj, c); };
  if (mode == 1) {
    const float4 *__restrict__ stage = sm.stage(0);
    const uint32_t cnt = load_own(&nc.cnt[k]);
    if (cnt <= c.maxn)
      for_each_staged(nc, k, cnt, [&](uint32_t i) { return stage[i]; }, pair);
    else
      visit_fallback(nc, k, [&](uint32_t j) { pair(__ldg(&P[j])); });
  } else {
    visit_neighbours<4>(nc, k, [&](uint32_t j) { return __ldg(&P[j]); }, pair);
  }
  lambda_commit(k, pk, acc, c, Q, R);
}

__global__ void __launch_bounds__(kTile)
    k_delta_tile(const float4 *__restrict__ Q, NbrCtx nc, TileCtx tc, PaperConsts c,
                 float4 *__restrict__ D, float4 *__restrict__ P, const float *__restrict__ R,
                 float4 *__restrict__ U, int last) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TileSmem sm{smem_raw};
  const float4 *const src[1] = {Q};
  const int mode = stage_tile<1>(tc, blockIdx.x, src, sm, nc.err);
  const uint32_t k = blockIdx.x * kTile + threadIdx.x;
  if (mode < 0 || k >= c.n) return;
  const float4 qk = load_own(&Q[k]);
  DeltaAcc acc{0.f, 0.f, 0.f};
  const auto walk = [&](auto twelve) {
    const auto pair = [&](const float4 &qj) {
      acc.template pair<decltype(twelve)::value>(qk, qj, c);
    };
    if (mode == 1) {
      const float4 *__restrict__ stage = sm.stage(0);
      const uint32_t cnt = load_own(&nc.cnt[k]);
      if (cnt <= c.maxn)
        for_each_staged(nc, k, cnt, [&](uint32_t i) { return stage[i]; }, pair);
      else
        visit_fallback(nc, k, [&](uint32_t j) { pair(__ldg(&Q[j])); });
    } else {
      visit_neighbours<4>(nc, k, [&](uint32_t j) { return __ldg(&Q[j]); }, pair);
    }
  };
  if (c.scorr_n3 == 12) walk(std::true_type{});
  else walk(std::false_type{});
  delta_commit(k, acc, nc, c, D, P, R, U, last);
}

__global__ void __launch_bounds__(kTile)
    k_vorticity_tile(const float4 *__restrict__ P, const float4 *__restrict__ U, NbrCtx nc,
                     TileCtx tc, PaperConsts c, float4 *__restrict__ Wo, float4 *__restrict__ PW) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TileSmem sm{smem_raw};
  const float4 *const src[2] = {P, U};
  const int mode = stage_tile<2>(tc, blockIdx.x, src, sm, nc.err);
  const uint32_t k = blockIdx.x * kTile + threadIdx.x;
  if (mode < 0 || k >= c.n) return;
  const float4 pk = load_own(&P[k]);
  const float4 uk = load_own(&U[k]);
  VortAcc acc{0.f, 0.f, 0.f};
  const auto pair = [&](const PU &d) { acc.pair(pk, uk, d, c); };
  if (mode == 1) {
    const float4 *__restrict__ sp = sm.stage(0);
    const float4 *__restrict__ su = sm.stage(1);
    const uint32_t cnt = load_own(&nc.cnt[k]);
    if (cnt <= c.maxn)
      for_each_staged(nc, k, cnt, [&](uint32_t i) { return PU{sp[i], su[i]}; }, pair);
    else
      visit_fallback(nc, k, [&](uint32_t j) { pair(PU{__ldg(&P[j]), __ldg(&U[j])}); });
  } else {
    visit_neighbours<4>(nc, k, [&](uint32_t j) { return PU{__ldg(&P[j]), __ldg(&U[j])}; }, pair);
  }
  vort_commit(k, pk, acc, Wo, PW);
}

__global__ void __launch_bounds__(kTile)
    k_xsph_commit_tile(const float4 *__restrict__ PW, const float4 *__restrict__ U,
                       const float4 *__restrict__ Wv, NbrCtx nc, TileCtx tc, PaperConsts c,
                       const uint32_t *__restrict__ ID2, float4 *__restrict__ X,
                       float4 *__restrict__ V, uint32_t *__restrict__ ID) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TileSmem sm{smem_raw};
  const float4 *const src[2] = {PW, U};
  const int mode = stage_tile<2>(tc, blockIdx.x, src, sm, nc.err);
  const uint32_t k = blockIdx.x * kTile + threadIdx.x;
  if (mode < 0 || k >= c.n) return;
  const float4 pk = load_own(&PW[k]);
  const float4 uk = load_own(&U[k]);
  const float4 wk = load_own(&Wv[k]);
  XsphAcc acc{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const auto pair = [&](const PU &d) { acc.pair(pk, uk, wk, d, c); };
  if (mode == 1) {
    const float4 *__restrict__ sp = sm.stage(0);
    const float4 *__restrict__ su = sm.stage(1);
    const uint32_t cnt = load_own(&nc.cnt[k]);
    if (cnt <= c.maxn)
      for_each_staged(nc, k, cnt, [&](uint32_t i) { return PU{sp[i], su[i]}; }, pair);
    else
      visit_fallback(nc, k, [&](uint32_t j) { pair(PU{__ldg(&PW[j]), __ldg(&U[j])}); });
  } else {
    visit_neighbours<4>(nc, k, [&](uint32_t j) { return PU{__ldg(&PW[j]), __ldg(&U[j])}; }, pair);
  }
  xsph_commit(k, pk, uk, wk, acc, nc, c, ID2, X, V, ID);
}

inline uint32_t tiles_for(uint32_t n) { return (n + kTile - 1) / kTile; }

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

TileCtx make_tiles(const DeviceState &d, const PaperConsts &c) {
  return TileCtx{d.tile_info, d.tile_seg, c.n};
}

cudaError_t g_attr_status = cudaSuccess;
std::once_flag g_attr_once;
void set_attributes() {
  // The velocity passes stage two arrays: 64 KB of dynamic shared memory.
  cudaError_t e = cudaFuncSetAttribute(k_vorticity_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)stage_smem_bytes(2));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_xsph_commit_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)stage_smem_bytes(2));
  g_attr_status = e;
}

}  // namespace

cudaError_t tile_init() {
  std::call_once(g_attr_once, set_attributes);
  return g_attr_status;
}

uint32_t tile_count(uint32_t n) { return tiles_for(n); }

#define PBF_TILE_LAUNCH(KERNEL, KIND, ARRAYS, ...)                                        \
  do {                                                                                   \
    const cudaError_t ie_ = tile_init();                                                 \
    if (ie_ != cudaSuccess) return ie_;                                                  \
    const int slot_ = d.timer ? d.timer->begin(KIND, st) : -1;                           \
    KERNEL<<<tiles_for(c.n), kTile, stage_smem_bytes(ARRAYS), st>>>(__VA_ARGS__);         \
    if (d.timer) d.timer->end(slot_, st);                                                \
  } while (0)

cudaError_t tile_plan(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                      cudaStream_t st) {
  if (c.n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d.tile_stats, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_tile_plan<<<tiles_for(c.n), 32, 0, st>>>(make_ctx(d, c, sid), c.n, d.tile_info, d.tile_seg,
                                             d.tile_stats);
  return cudaGetLastError();
}

cudaError_t tile_nbr_build(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                           cudaStream_t st) {
  PBF_TILE_LAUNCH(k_nbr_build_tile, kKindNbr, 1, d.P, make_ctx(d, c, sid), make_tiles(d, c), c,
                  d.nbr, d.nbr_cnt);
  return cudaGetLastError();
}

cudaError_t tile_lambda(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                        cudaStream_t st) {
  PBF_TILE_LAUNCH(k_lambda_tile, kKindLambda, 1, d.P, make_ctx(d, c, sid), make_tiles(d, c), c,
                  d.Q, d.R);
  return cudaGetLastError();
}

cudaError_t tile_delta(const DeviceState &d, const PaperConsts &c, const uint16_t *sid, bool last,
                       cudaStream_t st) {
  PBF_TILE_LAUNCH(k_delta_tile, kKindDelta, 1, d.Q, make_ctx(d, c, sid), make_tiles(d, c), c, d.D,
                  d.P, d.R, d.U, last ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t tile_vorticity(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                           cudaStream_t st) {
  PBF_TILE_LAUNCH(k_vorticity_tile, kKindVorticity, 2, d.P, d.U, make_ctx(d, c, sid),
                  make_tiles(d, c), c, d.W, d.D);
  return cudaGetLastError();
}

cudaError_t tile_xsph_commit(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                             cudaStream_t st) {
  PBF_TILE_LAUNCH(k_xsph_commit_tile, kKindXsph, 2, d.D, d.U, d.W, make_ctx(d, c, sid),
                  make_tiles(d, c), c, d.ID2, d.X, d.V, d.ID);
  return cudaGetLastError();
}

#undef PBF_TILE_LAUNCH

}  // namespace pbf
