// Internal declarations shared by the CUDA translation units of the GB300
// position-based-fluids library.  Nothing here crosses the C-ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>

namespace pbf {

// ---------------------------------------------------------------- errors --
// Device-side error bits, OR-ed into a per-simulation flag word that the
// host reads back at synchronisation points.
enum DeviceError : uint32_t {
  kDevErrLookback = 1u,  // a sort's look-back wait hit its bound
  kDevErrStage = 2u,     // a tile's bulk copies did not complete within the bounded wait
  kDevErrKey = 4u,       // the cell-sort operator got a key not below its cell count
};

// ------------------------------------------------------------ grid / scene --
// One simulation box with its uniform cell grid.  In the single-scene path
// the table has one entry; a batch holds one entry per scene, each owning
// the key range [cell_base, cell_base + ncell.x*ncell.y*ncell.z) and the
// particle range [p_begin, p_end) of the sorted state.
struct SceneDesc {
  float gmin[3];      // grid origin (the box minimum)
  float clen[3];      // cell lengths
  int32_t ncell[3];   // cells per axis
  uint32_t cell_base; // first key of this scene
  float lo[3];        // lowest admissible position per axis (x without wave)
  float hi[3];        // highest admissible position per axis
  float wave;         // moving x-min wall offset
  uint32_t p_begin;   // first particle (sorted state)
  uint32_t p_end;     // one past the last particle
  uint32_t block_base; // first cell-block index of this scene (staged passes)
};

// Solver constants of the paper equations (PBF_MODE_PAPER).
struct PaperConsts {
  float dt, gy;
  float h, h2, poly6, spiky, w_self;
  float rho0, inv_rho0, relax_eps;
  float scorr_k, inv_scorr_den;  // 1 / (h^2 - (dq h)^2)
  int32_t scorr_n3;              // 3 * n
  float xsph_c, vort_eps;
  uint32_t n, maxn;
};

// The 18 constants the reference bakes into its OpenCL program
// (src/main.cpp:149-168), already rounded to 6 significant digits.
struct RefConsts {
  float min[3], max[3];
  float ncell[3];
  float clen[3];
  float dt, rest_density, h, h2, poly6, spiky;
  uint32_t n;  // particles
};

// Grid of a grid-stride kernel with 256-thread CTAs: one full wave on the
// 152 SMs of a GB300 (8 CTAs of 256 threads per SM).
constexpr uint32_t kStrideCtas = 152u * 8u;

// ------------------------------------------------------------------ sort --
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kMaxSortPasses = 4;
// Digit widths: 8 bits (one digit per scan thread) or 9 bits (two).
constexpr uint32_t kMinDigitBits = 8;
constexpr uint32_t kMaxDigitBits = 9;
// passes * radix of any plan (four 8-bit passes, two 9-bit ones)
constexpr uint32_t kMaxHistWords = 1024;
// Words of the look-back wait self-test: two tiles of 8-bit digits + flag.
constexpr uint32_t kSelftestWords = 2u * (1u << kMinDigitBits) + 1u;

// 9-bit digits where they save a pass within two passes -- 9-bit keys (one
// pass instead of two) and 17-18-bit keys (two instead of three, e.g. the
// cells of a 64^3 grid) -- and 8-bit digits otherwise.  On GB300 a 9-bit
// pass costs about 1.4 times an 8-bit one: two of them beat three 8-bit
// passes, three do not beat four, and 10-bit passes lost to 8-bit ones.
constexpr uint32_t sort_digit_bits_for(uint32_t key_bits) {
  return (key_bits == 9 || key_bits == 17 || key_bits == 18) ? 9u : 8u;
}
constexpr uint32_t sort_passes_for(uint32_t key_bits) {
  const uint32_t w = sort_digit_bits_for(key_bits);
  return (key_bits + w - 1) / w;
}

// Layout of the radix-sort scratch inside one allocation (32-bit words).
struct SortPlan {
  uint32_t n = 0, key_bits = 0, passes = 0, tiles = 0;
  uint32_t digit_bits = 0, radix = 0;
  size_t off_hist = 0;      // passes * radix: digit histograms, then prefixes
  size_t off_counter = 0;   // 32 words: per-pass tile counters
  size_t off_lookback = 0;  // passes * tiles * radix
  size_t clear_words = 0;   // words from off_hist that must start at zero
  size_t off_keys_alt = 0;  // n
  size_t off_vals_alt = 0;  // n
  size_t words = 0;         // total
};

constexpr SortPlan make_sort_plan(uint32_t n, uint32_t key_bits) {
  SortPlan p;
  p.n = n;
  p.key_bits = key_bits < 1 ? 1 : (key_bits > 32 ? 32 : key_bits);
  p.passes = sort_passes_for(p.key_bits);
  p.digit_bits = sort_digit_bits_for(p.key_bits);
  p.radix = 1u << p.digit_bits;
  p.tiles = (uint32_t)(((uint64_t)n + kSortTile - 1) / kSortTile);
  size_t w = 0;
  p.off_hist = w;
  w += (size_t)p.passes * p.radix;
  p.off_counter = w;
  w += 32;
  p.off_lookback = w;
  w += (size_t)p.passes * p.tiles * p.radix;
  p.clear_words = w - p.off_hist;
  w = (w + 63) & ~size_t(63);
  p.off_keys_alt = w;
  w += (size_t)n;
  w = (w + 63) & ~size_t(63);
  p.off_vals_alt = w;
  w += (size_t)n;
  p.words = w;
  return p;
}
// The largest scratch (words) a plan of n keys of any width lays out.
constexpr size_t sort_words_max(uint32_t n) {
  size_t w = 0;
  for (uint32_t b = 1; b <= 32; ++b) {
    const size_t x = make_sort_plan(n, b).words;
    w = x > w ? x : w;
  }
  return w;
}
uint32_t bits_for(uint32_t max_key_exclusive);

// Zeroes the histogram/counter/look-back words of `scratch`.
cudaError_t sort_clear(const SortPlan &plan, uint32_t *scratch,
                       cudaStream_t stream);
// Digit histograms of keys (all passes); expects sort_clear first.
cudaError_t sort_histogram(const SortPlan &plan, const uint32_t *keys,
                           uint32_t *scratch, cudaStream_t stream);
// Exclusive prefix of each pass histogram, in place.
cudaError_t sort_scan(const SortPlan &plan, uint32_t *scratch,
                      cudaStream_t stream);
// The digit passes (histograms must be scanned).  vals_in may be null
// (values = index).  Results land in keys_out / vals_out; inputs are left
// untouched.
cudaError_t sort_passes(const SortPlan &plan, const uint32_t *keys_in,
                        const uint32_t *vals_in, uint32_t *keys_out,
                        uint32_t *vals_out, uint32_t *scratch, uint32_t *err,
                        cudaStream_t stream);
cudaError_t cell_offsets(const uint32_t *sorted_keys, uint32_t n,
                         uint32_t ncells, uint32_t *offsets,
                         cudaStream_t stream);
// The same offsets in O(n + ncells) work: every key boundary writes the run
// of cells it starts (runs longer than 64 cells are queued in `runs`, in
// chunks of at most 4096 cells, and filled by a second kernel).  `runs` holds
// offset_runs_capacity(ncells) entries; *runs_count is scratch.  Two
// kernels and one memset.
uint32_t offset_runs_capacity(uint32_t ncells);
cudaError_t cell_offsets_runs(const uint32_t *sorted_keys, uint32_t n, uint32_t ncells,
                              uint32_t *offsets, uint4 *runs, uint32_t *runs_count,
                              cudaStream_t stream);
cudaError_t find_cells(const uint32_t *offsets, uint32_t ncells,
                       int32_t *first_last, cudaStream_t stream);
cudaError_t cell_hash(const float4 *pred, uint32_t n, const SceneDesc &scene,
                      uint32_t *hash, cudaStream_t stream);
// Runs the sort's bounded look-back wait against a predecessor that never
// publishes (scratch: kSelftestWords zeroed words, the last one the flag);
// sets kDevErrLookback in *err
// after spin_limit polls.
cudaError_t wait_selftest(uint32_t *scratch, uint32_t spin_limit, uint32_t *err,
                          cudaStream_t stream);
// Number of kernel launches of one sort (histogram not included).
uint32_t sort_pass_launches(const SortPlan &plan);

// Counting sort of cell keys (paper path): the predict kernel counts every
// cell's particles into `counts` and keeps each particle's place among its
// cell's in `pos`; cell_sort_finish turns the counts into the cell offsets
// (leaving the counts zero for the next step), scatters the particles and
// puts each cell back in index order, so skeys / perm are the stable sort's.
// Layout of its scratch (32-bit words):
struct CellSortPlan {
  uint32_t n = 0, ncells = 0, tiles = 0;
  uint32_t small_cap = 0, med_cap = 0, big_cap = 0, huge_cap = 0;
  uint32_t bm_words = 0;   // words of a bitmap over the n particle indices
  uint32_t bm_stride = 0;  // words from one CTA's bitmap to the next
  size_t off_counts = 0;  // ncells: per-cell counts (zero between steps)
  size_t off_pos = 0;     // n: each particle's place among its cell's
  size_t off_ctl = 0;     // 8 control words (list counts, an error word), then the
  size_t ctl_words = 0;   //     scan's look-back words (zeroed before every step)
  size_t off_small = 0;   // cells of 2..16 particles out of index order
  size_t off_med = 0;     // cells of 17..64 particles
  size_t off_big = 0;     // cells of 65..8192 particles
  size_t off_huge = 0;    // cells of more than 8192
  size_t off_bitmap = 0;  // one bitmap of the particle indices per huge-cell CTA
  size_t words = 0;
};
CellSortPlan make_cell_sort_plan(uint32_t n, uint32_t ncells);
// The same layout (sized for n_cap particles and cells_cap cells) sorting
// n particles over ncells cells: a batch keeps one layout of its scratch
// while its scenes change.
CellSortPlan resize_cell_sort_plan(const CellSortPlan &cap, uint32_t n, uint32_t ncells);
// Zeroes the control words (and, with counts = true, the counts: once after
// allocation).
cudaError_t cell_sort_clear(const CellSortPlan &plan, uint32_t *scratch, bool counts,
                            cudaStream_t stream);
// Offsets, scatter and in-cell order after the predict kernel has counted
// (4 launches).
cudaError_t cell_sort_finish(const CellSortPlan &plan, const uint32_t *keys, uint32_t *scratch,
                             uint32_t *offsets, uint32_t *skeys, uint32_t *perm, uint32_t *err,
                             cudaStream_t stream);
uint32_t cell_sort_launches();
// The predict kernel's counting from a key array; a key outside
// [0, plan.ncells) is left out and sets kDevErrKey in *err.
cudaError_t cell_sort_count(const CellSortPlan &plan, const uint32_t *keys, uint32_t *scratch,
                            uint32_t *err, cudaStream_t stream);

// ------------------------------------------------- gather-pass launch shape --
// The gather passes of the paper equations, as tuned separately.
enum GatherKind : int {
  kKindNbr = 0,     // neighbour-list build
  kKindNbrLambda,   // list build fused with the first lambda
  kKindLambda,
  kKindDelta,
  kKindVorticity,
  kKindXsph,
  kGatherKinds
};

// Launch shape of each gather pass.  No choice changes a result bit: every
// variant computes each particle in one thread with the same operations in
// the same order.
struct GatherTuning {
  // threads per CTA, 64 << code: 128, except 256 for lambda and vorticity
  // (fastest over the 1M-particle dam break's 500 steps)
  uint8_t block[kGatherKinds] = {1, 1, 2, 1, 2, 1};
  uint8_t batch[kGatherKinds] = {0, 0, 0, 0, 0, 0};  // neighbour loads in flight: 4 << code
  // 1: one kernel builds the lists and computes the first lambda (faster over
  // the 1M-particle dam break's 500 steps: 0.893 against 0.906 ms per step)
  uint8_t fuse_first = 1;
  // 1: the gather passes stage each tile's neighbourhood in shared memory
  // (pbf_tile.cu; one 128-thread shape, fuse_first does not apply)
  uint8_t staged = 0;
  // 1: the onesweep radix sort of the cell keys instead of the counting
  // sort by cell (same permutation)
  uint8_t radix_sort = 0;
  // 1: the list build tests each row's candidates into a membership mask and
  // stores the members from it afterwards (same lists; 3% faster build, 6%
  // faster fused build on the 1M-particle dam break)
  uint8_t masked_build = 1;
};
constexpr int kBlockCodes = 3;  // 64, 128, 256
constexpr int kBatchCodes = 2;  // 4, 8

// Optional per-kind timing of gather launches (used by the tuner): an event
// pair around each launch, summed per kind by collect().
struct GatherTimer {
  static constexpr int kMax = 512;
  cudaEvent_t ev[2 * kMax] = {};
  int kind[kMax] = {};
  int used = 0;
  bool ready = false;
  cudaError_t init() {
    for (int i = 0; i < 2 * kMax; ++i) {
      const cudaError_t e = cudaEventCreate(&ev[i]);
      if (e != cudaSuccess) return e;
    }
    ready = true;
    return cudaSuccess;
  }
  void destroy() {
    for (int i = 0; i < 2 * kMax; ++i)
      if (ev[i]) cudaEventDestroy(ev[i]);
    ready = false;
  }
  // Returns the slot to close with end(), or -1 when the pool is full.
  int begin(int k, cudaStream_t st) {
    if (!ready || used >= kMax) return -1;
    kind[used] = k;
    cudaEventRecord(ev[2 * used], st);
    return used++;
  }
  void end(int slot, cudaStream_t st) {
    if (slot >= 0) cudaEventRecord(ev[2 * slot + 1], st);
  }
  cudaError_t collect(double ms[kGatherKinds], uint32_t count[kGatherKinds]) {
    for (int k = 0; k < kGatherKinds; ++k) ms[k] = 0.0, count[k] = 0;
    for (int i = 0; i < used; ++i) {
      cudaError_t e = cudaEventSynchronize(ev[2 * i + 1]);
      if (e != cudaSuccess) return e;
      float t = 0.f;
      e = cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]);
      if (e != cudaSuccess) return e;
      ms[kind[i]] += t;
      count[kind[i]] += 1;
    }
    used = 0;
    return cudaSuccess;
  }
};

// --------------------------------------------------------- device buffers --
// Everything one plain (single-scene) simulation keeps on the device.
struct DeviceState {
  // persistent particle state
  float4 *X = nullptr, *V = nullptr;   // positions (.w=|v|), velocities (.w=m)
  uint32_t *ID = nullptr;              // input index of each slot (paper)
  // step scratch
  float4 *X2 = nullptr, *V2 = nullptr; // reordered state (paper)
  uint32_t *ID2 = nullptr;
  float4 *P = nullptr, *Q = nullptr;   // predicted positions (+lambda)
  float4 *D = nullptr;                 // displacement since step start (paper)
  float4 *U = nullptr;                 // velocity and 1/rho (paper)
  float4 *W = nullptr;                 // vorticity and |omega| (paper)
  float4 *S = nullptr;                 // sum of (1/rho_j) grad W (paper, vorticity pass)
  float *R = nullptr;                  // density (paper)
  // ref-compat: P, V and lambda by sorted slot during the step (P with the
  // Jacobi ping-pong), and the XSPH velocity change by input index
  float4 *PS = nullptr, *PS2 = nullptr, *VS = nullptr, *DV = nullptr;
  float *SS = nullptr;
  uint32_t *keys = nullptr, *skeys = nullptr, *perm = nullptr;
  uint32_t *offsets = nullptr;         // ncells + 1
  uint4 *runs = nullptr;               // offset_runs_capacity(ncells) queued runs
  uint32_t *runs_count = nullptr;
  uint4 *nbr = nullptr;                // neighbour lists, 4 slots or 8 staged indices per word (paper)
  uint32_t *nbr_cnt = nullptr;         // neighbour counts (paper)
  uint32_t *nbr_max = nullptr;         // largest neighbour count of the step (paper)
  uint32_t *sort_scratch = nullptr;
  uint32_t *cell_scratch = nullptr;    // counting sort by cell (paper)
  uint32_t *err = nullptr;             // device error flag word
  SceneDesc *scenes = nullptr;         // device scene table
  float4 *io_pos = nullptr, *io_vel = nullptr; // input-order staging
  // staged cell blocks (paper): the step's work list of occupied blocks
  uint32_t *blk_list = nullptr;        // block indices (capacity blk_cap)
  uint32_t *blk_count = nullptr;       // [0] blocks in the list, [1] staged, [2] unstaged
  uint32_t blk_cap = 0;                // capacity of blk_list
  uint32_t blk_total = 0;              // blocks of the current layout (host)
  // batches only (null for a single scene)
  uint16_t *sid = nullptr;             // scene of each sorted slot
  // host-side launch shape of the gather passes, and the tuner's timer
  GatherTuning tune;
  GatherTimer *timer = nullptr;
};

// Scene of every sorted slot of a batch from its scene table (device).
cudaError_t scene_ids(const SceneDesc *scenes, uint32_t nscenes, uint32_t n, uint16_t *sid,
                      cudaStream_t st);
// dst[i] = i for i in [0, n).
cudaError_t iota_range(uint32_t *dst, uint32_t n, cudaStream_t st);

// ------------------------------------------------------- staged cell blocks
// The staged gather passes (pbf_tile.cu) work on blocks of kBlockCells^3
// cells of each scene's grid.
constexpr int kBlockCells = 4;
#ifdef __CUDACC__
#define PBF_HOST_DEVICE __host__ __device__
#else
#define PBF_HOST_DEVICE
#endif
PBF_HOST_DEVICE inline uint32_t blocks_along(int32_t cells) {
  return (uint32_t)((cells + kBlockCells - 1) / kBlockCells);
}
inline uint32_t scene_blocks(const SceneDesc &s) {
  return blocks_along(s.ncell[0]) * blocks_along(s.ncell[1]) * blocks_along(s.ncell[2]);
}
// Sets the kernels' shared-memory limits and persistent grid sizes (once per
// process); the launches below call it too.
cudaError_t tile_init();
// The step's list of occupied cell blocks (after the cell offsets), then the
// staged passes: the same outputs as the paper_* launches of the same names.
// `nscenes` scene descriptors, `blocks` = the layout's blocks in total.
cudaError_t tile_plan(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                      uint32_t nscenes, cudaStream_t st);
cudaError_t tile_nbr_build(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                           uint32_t nscenes, cudaStream_t st);
cudaError_t tile_lambda(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                        uint32_t nscenes, cudaStream_t st);
cudaError_t tile_delta(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                       uint32_t nscenes, bool last, cudaStream_t st);
cudaError_t tile_vorticity(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                           uint32_t nscenes, cudaStream_t st);
cudaError_t tile_xsph_commit(const DeviceState &d, const PaperConsts &c, const uint16_t *sid,
                             uint32_t nscenes, cudaStream_t st);

// ------------------------------------------------------- paper-mode launches
// 16-byte list words per particle for a list capacity of maxn neighbours.
inline uint32_t paper_list_words(uint32_t maxn) { return (maxn + 3u) / 4u; }
cudaError_t paper_predict_hash(const float4 *X, const float4 *V, uint32_t n,
                               const PaperConsts &c, const SceneDesc *scenes,
                               const uint16_t *sid, uint32_t *keys,
                               const SortPlan &plan, uint32_t *sort_scratch,
                               cudaStream_t st);
// The same prediction and keys, counted for the counting sort.
cudaError_t paper_predict_count(const float4 *X, const float4 *V, uint32_t n,
                                const PaperConsts &c, const SceneDesc *scenes,
                                const uint16_t *sid, uint32_t *keys,
                                const CellSortPlan &plan, uint32_t *cell_scratch,
                                cudaStream_t st);
cudaError_t paper_reorder(const uint32_t *perm, const float4 *X,
                          const float4 *V, const uint32_t *ID, uint32_t n,
                          const PaperConsts &c, float4 *X2, float4 *V2,
                          uint32_t *ID2, float4 *P, float4 *D, cudaStream_t st);
// Neighbour lists of the step (from the predicted positions P).
cudaError_t paper_nbr_build(const DeviceState &d, const PaperConsts &c,
                            const uint16_t *sid, cudaStream_t st);
// The same lists and, in the same kernel, the first lambda pass.
cudaError_t paper_nbr_lambda(const DeviceState &d, const PaperConsts &c,
                             const uint16_t *sid, cudaStream_t st);
// Launches of the first solver iteration's list build and lambda pass under
// the current tuning (1 fused or 2).
inline uint32_t paper_first_launches(const DeviceState &d) {
  return d.tune.staged ? 3u /*plan, build, lambda*/ : (d.tune.fuse_first ? 1u : 2u);
}
cudaError_t paper_lambda(const DeviceState &d, const PaperConsts &c,
                         const uint16_t *sid, cudaStream_t st);
cudaError_t paper_delta(const DeviceState &d, const PaperConsts &c,
                        const uint16_t *sid, bool last, cudaStream_t st);
cudaError_t paper_vorticity(const DeviceState &d, const PaperConsts &c,
                            const uint16_t *sid, cudaStream_t st);
cudaError_t paper_xsph_commit(const DeviceState &d, const PaperConsts &c,
                              const uint16_t *sid, cudaStream_t st);
// state <-> input order
cudaError_t gather_to_input_order(const float4 *X, const float4 *V,
                                  const uint32_t *ID, uint32_t n,
                                  float4 *out_pos, float4 *out_vel,
                                  cudaStream_t st);
cudaError_t scatter_from_input_order(const float4 *in_pos,
                                     const float4 *in_vel, const uint32_t *ID,
                                     uint32_t n, float4 *X, float4 *V,
                                     cudaStream_t st);
cudaError_t gather_scalar_to_input_order(const float *src, const uint32_t *ID,
                                         uint32_t n, float *out,
                                         cudaStream_t st);
cudaError_t iota_u32(uint32_t *dst, uint32_t n, cudaStream_t st);

// --------------------------------------------------- ref-compat launches --
cudaError_t rc_predict_hash(float4 *X, float4 *V, float4 *P, uint32_t n,
                            const RefConsts &k, const SceneDesc *scenes,
                            uint32_t *keys, const SortPlan &plan,
                            uint32_t *sort_scratch, cudaStream_t st);
// PS[m] = P[perm[m]]: the predicted positions by sorted slot.
cudaError_t rc_gather(const float4 *P, const uint32_t *perm, uint32_t n, float4 *PS,
                      cudaStream_t st);
// The passes read neighbours by sorted slot (PS, SS, VS) and write their own
// slot's values there; the last delta-p pass also writes P and V by input
// index for the commit.
cudaError_t rc_lambda(float4 *PS, float *SS, const uint32_t *offsets, uint32_t n,
                      const RefConsts &k, cudaStream_t st);
cudaError_t rc_delta(const float4 *PS, float4 *PS2, const float *SS, const uint32_t *perm,
                     const uint32_t *offsets, const float4 *X, float4 *V, float4 *P,
                     float4 *VS, uint32_t n, const RefConsts &k, const SceneDesc *scenes,
                     bool last, cudaStream_t st);
cudaError_t rc_xsph(const float4 *PS, const float4 *VS, float4 *DV, const uint32_t *perm,
                    const uint32_t *offsets, uint32_t n, const RefConsts &k,
                    cudaStream_t st);
cudaError_t rc_commit(float4 *X, float4 *V, const float4 *P, const float4 *DV,
                      uint32_t n, cudaStream_t st);

}  // namespace pbf
