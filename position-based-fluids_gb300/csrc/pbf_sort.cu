// Neighbour structure for the GB300 position-based-fluids step: cell hash,
// onesweep LSD radix sort of 32-bit cell keys, CSR cell offsets and the
// reference's inclusive cell ranges.
//
// Reference semantics this implements (MrMagne/position-based-fluids):
//   - cell hash: src/kernels/update_cells.cl:10-15 (and calc_hash.cl:15-20);
//   - a stable LSD radix sort of (cell, particle index) pairs, the intent of
//     src/kernels/radix_histogram.cl, radix_scan.cl, radix_paste.cl and
//     radix_reorder.cl driven by src/Simulation.cpp:351-435 (that code does
//     not run as shipped: radix_reorder.cl:28-41 uses an uninitialised
//     counter);
//   - inclusive [first,last] cell ranges with -1 for empty cells, the intent
//     of init_cells.cl and find_cells.cl.
//
// The sort is the onesweep scheme (one upfront histogram pass for every
// digit, then one pass per digit that ranks a tile of keys with warp-level
// multisplit, publishes per-digit tile counts and resolves its global
// offsets by decoupled look-back).  Digits are 8 bits wide, or 9 where that
// saves a pass within two passes: the 18-bit cell keys of a 64^3-cell grid
// take two 9-bit passes instead of three 8-bit ones.  Tiles are numbered by an atomic
// counter in the order CTAs start, so a CTA only ever waits on tiles that
// are already resident; every wait is additionally bounded, and a wait that
// runs out sets a device error bit instead of spinning on.
#include <mutex>

#include "pbf_device.cuh"

namespace pbf {

namespace {

constexpr uint32_t kLbMask = (1u << 30) - 1u;
constexpr uint32_t kLbAggregate = 1u << 30;
constexpr uint32_t kLbInclusive = 2u << 30;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kSortWarps = kSortThreads / 32;
static_assert(kSortThreads == (1 << kMinDigitBits), "at least one digit per scan thread");

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *reinterpret_cast<const volatile uint32_t *>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) {
  *reinterpret_cast<volatile uint32_t *>(p) = v;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v,
                                                         uint32_t *s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kSortWarps ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < kSortWarps; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kSortWarps) s_warp[lane] = wi - w;
  }
  __syncthreads();
  return incl - v + s_warp[warp];
}

__global__ void __launch_bounds__(256)
    k_sort_histogram(const uint32_t *__restrict__ keys, uint32_t n,
                     uint32_t passes, uint32_t digit_bits, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_hist[kMaxHistWords];
  const uint32_t hist_words = passes << digit_bits;
  for (uint32_t i = threadIdx.x; i < hist_words; i += blockDim.x) s_hist[i] = 0;
  __syncthreads();
  const uint32_t stride = gridDim.x * blockDim.x;
  // Whole warps iterate together so that __match_any_sync sees every lane.
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    const bool valid = i < n;
    warp_digit_histogram(valid ? keys[i] : 0u, valid, passes, digit_bits, s_hist);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < hist_words; i += blockDim.x)
    if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

// Exclusive prefix of each pass histogram, in place: each thread owns
// radix / 256 consecutive digits.
__global__ void __launch_bounds__(kSortThreads)
    k_sort_scan(uint32_t passes, uint32_t digit_bits, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_warp[kSortWarps];
  constexpr uint32_t kMaxPer = 1u << (kMaxDigitBits - kMinDigitBits);
  const uint32_t per = 1u << (digit_bits - kMinDigitBits);
  for (uint32_t p = 0; p < passes; ++p) {
    uint32_t *h = hist + (p << digit_bits) + threadIdx.x * per;
    uint32_t v[kMaxPer], sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < kMaxPer; ++j) {
      v[j] = j < per ? h[j] : 0u;
      sum += v[j];
    }
    uint32_t e = block_exclusive_scan(sum, s_warp);
#pragma unroll
    for (uint32_t j = 0; j < kMaxPer; ++j) {
      if (j < per) h[j] = e;
      e += v[j];
    }
    __syncthreads();
  }
}

// Exclusive prefix of digit d over tiles [0, tile) from the look-back
// words, waiting for predecessors that have not published yet.  A wait of
// more than spin_limit polls sets kDevErrLookback in *err and gives up
// (returning what it has), so a kernel never spins without bound.
__device__ __forceinline__ uint32_t lookback_prefix(uint32_t *lookback, uint32_t radix,
                                                    uint32_t tile, uint32_t d,
                                                    uint32_t spin_limit, uint32_t *err) {
  uint32_t excl = 0;
  int t = (int)tile - 1;
  uint32_t spins = 0;
  while (true) {
    const uint32_t v = ld_volatile(&lookback[(size_t)t * radix + d]);
    const uint32_t flag = v & ~kLbMask;
    if (flag == 0u) {
      if (++spins >= spin_limit) {
        atomicOr(err, kDevErrLookback);
        break;
      }
      if (spins > 64) __nanosleep(32);
      continue;
    }
    excl += v & kLbMask;
    if (flag == kLbInclusive || t == 0) break;
    --t;
  }
  return excl;
}

// Runs the look-back wait of one digit against a predecessor tile that
// never publishes (the words are zero): the wait must give up after
// spin_limit polls and report through *err.
__global__ void k_wait_selftest(uint32_t *lookback, uint32_t spin_limit, uint32_t *err) {
  if (threadIdx.x == 0) lookback_prefix(lookback, 1u << kMinDigitBits, 1u, 0u, spin_limit, err);
}

// Dynamic shared memory of one digit pass with 2^kBits digits.
constexpr size_t onesweep_smem_bytes(uint32_t bits) {
  return ((size_t)kSortWarps * (1u << bits) + 2u * (1u << bits) + 2u * kSortTile) *
         sizeof(uint32_t);
}

template <uint32_t kBits, bool kIota>
__global__ void __launch_bounds__(kSortThreads)
    k_onesweep(const uint32_t *__restrict__ keys_in,
               const uint32_t *__restrict__ vals_in,
               uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out,
               uint32_t n, uint32_t shift,
               const uint32_t *__restrict__ global_excl,
               uint32_t *lookback, uint32_t *tile_counter, uint32_t *err) {
  constexpr uint32_t R = 1u << kBits;
  constexpr uint32_t kDig = R / kSortThreads;  // digits per thread, per-digit phases
  extern __shared__ __align__(16) uint32_t s_dyn[];
  uint32_t(*s_wcnt)[R] = reinterpret_cast<uint32_t(*)[R]>(s_dyn);  // [kSortWarps][R]
  uint32_t *s_dexcl = s_dyn + kSortWarps * R;
  uint32_t *s_gbase = s_dexcl + R;
  uint32_t *s_keys = s_gbase + R;
  uint32_t *s_vals = s_keys + kSortTile;
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[kSortWarps];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
  for (uint32_t i = tid; i < kSortWarps * R; i += kSortThreads) (&s_wcnt[0][0])[i] = 0u;
  __syncthreads();

  const uint32_t tile = s_tile;
  const uint32_t tile_base = tile * (uint32_t)kSortTile;
  // Each warp owns a contiguous segment of 32*kSortItems keys and reads it
  // lane-striped; the warp-local order (item, lane) is the input order.
  const uint32_t seg = tile_base + (uint32_t)warp * (32u * kSortItems);

  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const uint32_t idx = seg + (uint32_t)it * 32u + lane;
    const bool ok = idx < n;
    key[it] = ok ? keys_in[idx] : 0u;
    val[it] = ok ? (kIota ? idx : vals_in[idx]) : 0u;
  }

  // Warp-level multisplit: stable rank of each key among the warp's keys of
  // the same digit, item by item.
  const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const uint32_t idx = seg + (uint32_t)it * 32u + lane;
    const bool ok = idx < n;
    const uint32_t d = (key[it] >> shift) & (R - 1);
    const unsigned peers = __match_any_sync(0xffffffffu, ok ? d : 0xffffffffu);
    const uint32_t before = ok ? s_wcnt[warp][d] : 0u;
    __syncwarp();
    rank[it] = before + (uint32_t)__popc(peers & lt_mask);
    if (ok && lane == 31 - __clz(peers))
      s_wcnt[warp][d] = before + (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Per digit (kDig consecutive digits per thread): the tile's count, and
  // each warp's exclusive offset.
  uint32_t tile_count[kDig], excl[kDig];
  uint32_t sum = 0;
#pragma unroll
  for (uint32_t j = 0; j < kDig; ++j) {
    const uint32_t d = (uint32_t)tid * kDig + j;
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t x = s_wcnt[w][d];
      s_wcnt[w][d] = c;
      c += x;
    }
    tile_count[j] = c;
    excl[j] = 0;
    sum += c;
  }

  // Decoupled look-back: publish every aggregate before waiting on any.
  if (tile == 0) {
#pragma unroll
    for (uint32_t j = 0; j < kDig; ++j)
      st_volatile(&lookback[(uint32_t)tid * kDig + j], kLbInclusive | tile_count[j]);
  } else {
    uint32_t *mine = lookback + (size_t)tile * R + (uint32_t)tid * kDig;
#pragma unroll
    for (uint32_t j = 0; j < kDig; ++j) st_volatile(&mine[j], kLbAggregate | tile_count[j]);
#pragma unroll
    for (uint32_t j = 0; j < kDig; ++j) {
      excl[j] = lookback_prefix(lookback, R, tile, (uint32_t)tid * kDig + j, kSpinLimit, err);
      st_volatile(&mine[j], kLbInclusive | ((excl[j] + tile_count[j]) & kLbMask));
    }
  }
  uint32_t e = block_exclusive_scan(sum, s_warp);
#pragma unroll
  for (uint32_t j = 0; j < kDig; ++j) {
    const uint32_t d = (uint32_t)tid * kDig + j;
    s_gbase[d] = global_excl[d] + excl[j];
    s_dexcl[d] = e;
    e += tile_count[j];
  }
  __syncthreads();

  // Stage the tile in digit order in shared memory, then write it out with
  // consecutive threads on consecutive destinations.
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const uint32_t idx = seg + (uint32_t)it * 32u + lane;
    if (idx < n) {
      const uint32_t dg = (key[it] >> shift) & (R - 1);
      const uint32_t lp = s_dexcl[dg] + s_wcnt[warp][dg] + rank[it];
      s_keys[lp] = key[it];
      s_vals[lp] = val[it];
    }
  }
  __syncthreads();
  const uint32_t tile_n = min((uint32_t)kSortTile, n - tile_base);
  for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
    const uint32_t k = s_keys[i];
    const uint32_t dg = (k >> shift) & (R - 1);
    const uint32_t dst = s_gbase[dg] + (i - s_dexcl[dg]);
    // Always true unless a look-back wait gave up (error flag set).
    if (dst < n) {
      keys_out[dst] = k;
      vals_out[dst] = s_vals[i];
    }
  }
}

// Every instantiation takes its tile's shared memory dynamically (above the
// 48 KB static limit with 9-bit digits); the limit is raised once.
std::once_flag g_onesweep_once;
cudaError_t g_onesweep_status = cudaSuccess;

template <uint32_t kBits>
cudaError_t allow_onesweep_smem() {
  const int bytes = (int)onesweep_smem_bytes(kBits);
  cudaError_t e = cudaFuncSetAttribute(k_onesweep<kBits, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_onesweep<kBits, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

cudaError_t onesweep_init() {
  std::call_once(g_onesweep_once, [] {
    cudaError_t e = allow_onesweep_smem<8>();
    if (e == cudaSuccess) e = allow_onesweep_smem<9>();
    g_onesweep_status = e;
  });
  return g_onesweep_status;
}

template <uint32_t kBits>
void launch_onesweep(bool iota, uint32_t tiles, cudaStream_t stream, const uint32_t *ksrc,
                     const uint32_t *vsrc, uint32_t *kdst, uint32_t *vdst, uint32_t n,
                     uint32_t shift, const uint32_t *hist, uint32_t *lb, uint32_t *ctr,
                     uint32_t *err) {
  const size_t smem = onesweep_smem_bytes(kBits);
  if (iota)
    k_onesweep<kBits, true><<<tiles, kSortThreads, smem, stream>>>(ksrc, nullptr, kdst, vdst, n,
                                                                  shift, hist, lb, ctr, err);
  else
    k_onesweep<kBits, false><<<tiles, kSortThreads, smem, stream>>>(ksrc, vsrc, kdst, vdst, n,
                                                                   shift, hist, lb, ctr, err);
}

// off[c] = number of sorted keys < c, for c in [0, ncells]: one thread per
// cell, binary search over the sorted keys.  Neighbouring cells search
// neighbouring key ranges, so the probes of a warp share cache lines.
__global__ void k_cell_offsets(const uint32_t *__restrict__ skeys, uint32_t n,
                               uint32_t ncells, uint32_t *__restrict__ off) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncells) return;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (__ldg(&skeys[mid]) < c) lo = mid + 1;
    else hi = mid;
  }
  off[c] = lo;
}

constexpr uint32_t kShortRun = 64;    // cells a boundary thread writes itself
constexpr uint32_t kRunChunk = 4096;  // cells per queued chunk

// One thread per key boundary i in [0, n]: the cells (key[i-1], key[i]]
// (key[-1] = -1, key[n] = ncells) all take the value i -- the number of keys
// below each of them.  Short runs are written here, long ones queued.
__global__ void k_offset_runs(const uint32_t *__restrict__ skeys, uint32_t n, uint32_t ncells,
                              uint32_t *__restrict__ off, uint4 *__restrict__ runs,
                              uint32_t *__restrict__ runs_count, uint32_t runs_cap) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  const uint32_t lo = i == 0 ? 0u : min(skeys[i - 1], ncells - 1u) + 1u;
  const uint32_t hi = i == n ? ncells : min(skeys[i], ncells - 1u);
  if (hi < lo) return;
  const uint32_t count = hi - lo + 1u;
  if (count <= kShortRun) {
    for (uint32_t c = lo; c <= hi; ++c) off[c] = i;
    return;
  }
  const uint32_t chunks = (count + kRunChunk - 1u) / kRunChunk;
  const uint32_t slot = atomicAdd(runs_count, chunks);
  for (uint32_t q = 0; q < chunks; ++q) {
    const uint32_t a = lo + q * kRunChunk;
    const uint32_t len = min(kRunChunk, hi + 1u - a);
    if (slot + q < runs_cap) {
      runs[slot + q] = make_uint4(a, len, i, 0u);
    } else {  // beyond the capacity bound (keys out of order): write it here
      for (uint32_t c = a; c < a + len; ++c) off[c] = i;
    }
  }
}

// One CTA per queued chunk (grid-stride over the chunks).
__global__ void __launch_bounds__(256)
    k_offset_fill(const uint4 *__restrict__ runs, const uint32_t *__restrict__ runs_count,
                  uint32_t runs_cap, uint32_t *__restrict__ off) {
  const uint32_t total = min(*runs_count, runs_cap);
  for (uint32_t r = blockIdx.x; r < total; r += gridDim.x) {
    const uint4 e = runs[r];
    for (uint32_t t = threadIdx.x; t < e.y; t += blockDim.x) off[e.x + t] = e.z;
  }
}

__global__ void k_find_cells(const uint32_t *__restrict__ off, uint32_t ncells,
                             int2 *__restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const uint32_t a = off[c], b = off[c + 1];
  out[c] = a < b ? make_int2((int)a, (int)(b - 1)) : make_int2(-1, -1);
}

__global__ void k_cell_hash(const float4 *__restrict__ pred, uint32_t n,
                            SceneDesc scene, uint32_t *__restrict__ hash) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pred[i];
  hash[i] = scene.cell_base + scene_cell(p.x, p.y, p.z, scene);
}

inline uint32_t blocks_for(uint64_t n, uint32_t t) {
  return (uint32_t)((n + t - 1) / t);
}

}  // namespace

uint32_t bits_for(uint32_t max_key_exclusive) {
  uint32_t b = 1;
  while (b < 32 && (1ull << b) < (uint64_t)max_key_exclusive) ++b;
  return b;
}

uint32_t sort_pass_launches(const SortPlan &plan) { return 2u + plan.passes; }

cudaError_t wait_selftest(uint32_t *scratch, uint32_t spin_limit, uint32_t *err,
                          cudaStream_t stream) {
  k_wait_selftest<<<1, 32, 0, stream>>>(scratch, spin_limit, err);
  return cudaGetLastError();
}

cudaError_t sort_clear(const SortPlan &plan, uint32_t *scratch,
                       cudaStream_t stream) {
  return cudaMemsetAsync(scratch + plan.off_hist, 0,
                         plan.clear_words * sizeof(uint32_t), stream);
}

cudaError_t sort_histogram(const SortPlan &plan, const uint32_t *keys,
                           uint32_t *scratch, cudaStream_t stream) {
  if (plan.n == 0) return cudaSuccess;
  const uint32_t blocks = min(blocks_for(plan.n, 256), kStrideCtas);
  k_sort_histogram<<<blocks, 256, 0, stream>>>(keys, plan.n, plan.passes, plan.digit_bits,
                                               scratch + plan.off_hist);
  return cudaGetLastError();
}

cudaError_t sort_scan(const SortPlan &plan, uint32_t *scratch,
                      cudaStream_t stream) {
  k_sort_scan<<<1, kSortThreads, 0, stream>>>(plan.passes, plan.digit_bits,
                                              scratch + plan.off_hist);
  return cudaGetLastError();
}

cudaError_t sort_passes(const SortPlan &plan, const uint32_t *keys_in,
                        const uint32_t *vals_in, uint32_t *keys_out,
                        uint32_t *vals_out, uint32_t *scratch, uint32_t *err,
                        cudaStream_t stream) {
  if (plan.n == 0) return cudaSuccess;
  if (plan.digit_bits < kMinDigitBits || plan.digit_bits > kMaxDigitBits ||
      plan.passes > (uint32_t)kMaxSortPasses)
    return cudaErrorInvalidValue;
  const cudaError_t init = onesweep_init();
  if (init != cudaSuccess) return init;
  uint32_t *kalt = scratch + plan.off_keys_alt;
  uint32_t *valt = scratch + plan.off_vals_alt;
  // Arrange the ping-pong so the last pass writes keys_out/vals_out and the
  // inputs are never written.
  const uint32_t *ksrc = keys_in;
  const uint32_t *vsrc = vals_in;
  for (uint32_t p = 0; p < plan.passes; ++p) {
    const bool to_out = ((plan.passes - 1 - p) % 2) == 0;
    uint32_t *kdst = to_out ? keys_out : kalt;
    uint32_t *vdst = to_out ? vals_out : valt;
    uint32_t *hist = scratch + plan.off_hist + (size_t)p * plan.radix;
    uint32_t *lb = scratch + plan.off_lookback + (size_t)p * plan.tiles * plan.radix;
    uint32_t *ctr = scratch + plan.off_counter + p;
    const bool iota = p == 0 && vsrc == nullptr;
    const uint32_t shift = p * plan.digit_bits;
    if (plan.digit_bits == 8)
      launch_onesweep<8>(iota, plan.tiles, stream, ksrc, vsrc, kdst, vdst, plan.n, shift, hist,
                         lb, ctr, err);
    else
      launch_onesweep<9>(iota, plan.tiles, stream, ksrc, vsrc, kdst, vdst, plan.n, shift, hist,
                         lb, ctr, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    ksrc = kdst;
    vsrc = vdst;
  }
  return cudaSuccess;
}

cudaError_t cell_offsets(const uint32_t *sorted_keys, uint32_t n,
                         uint32_t ncells, uint32_t *offsets,
                         cudaStream_t stream) {
  if (n == 0) return cudaMemsetAsync(offsets, 0, (ncells + 1ull) * 4, stream);
  k_cell_offsets<<<blocks_for(ncells + 1ull, 256), 256, 0, stream>>>(
      sorted_keys, n, ncells, offsets);
  return cudaGetLastError();
}

uint32_t offset_runs_capacity(uint32_t ncells) {
  // every queued run is longer than kShortRun cells and adds one chunk per
  // kRunChunk cells or part of it
  const uint64_t cells = (uint64_t)ncells + 1u;
  return (uint32_t)(cells / (kShortRun + 1u) + cells / kRunChunk + 2u);
}

cudaError_t cell_offsets_runs(const uint32_t *sorted_keys, uint32_t n, uint32_t ncells,
                              uint32_t *offsets, uint4 *runs, uint32_t *runs_count,
                              cudaStream_t stream) {
  const uint32_t cap = offset_runs_capacity(ncells);
  cudaError_t e = cudaMemsetAsync(runs_count, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  k_offset_runs<<<blocks_for(n + 1ull, 256), 256, 0, stream>>>(sorted_keys, n, ncells, offsets,
                                                               runs, runs_count, cap);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_offset_fill<<<min(cap, kStrideCtas / 2u), 256, 0, stream>>>(runs, runs_count, cap, offsets);
  return cudaGetLastError();
}

cudaError_t find_cells(const uint32_t *offsets, uint32_t ncells,
                       int32_t *first_last, cudaStream_t stream) {
  if (ncells == 0) return cudaSuccess;
  k_find_cells<<<blocks_for(ncells, 256), 256, 0, stream>>>(
      offsets, ncells, reinterpret_cast<int2 *>(first_last));
  return cudaGetLastError();
}

cudaError_t cell_hash(const float4 *pred, uint32_t n, const SceneDesc &scene,
                      uint32_t *hash, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_cell_hash<<<blocks_for(n, 256), 256, 0, stream>>>(pred, n, scene, hash);
  return cudaGetLastError();
}

}  // namespace pbf
