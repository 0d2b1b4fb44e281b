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
//           the vorticity pass then reuses it for (p, |vorticity| / rho)
//   Q       (predicted position, lambda) as read by the delta-p pass; the
//           vorticity pass then reuses it for the XSPH sum
//   U       (velocity, 1/rho) as read by the velocity passes
//   W       (vorticity, |vorticity|)
//   S       sum of (1/rho_j) grad W over the neighbours (vorticity pass)
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
#include "pbf_paper.cuh"

namespace pbf {

namespace {


// ------------------------------------------------------------------------
// Prediction and cell key of every particle (grid-stride, whole warps
// iterate together), counted for the counting sort.
__global__ void __launch_bounds__(256)
    k_predict_count(const float4 *__restrict__ X, const float4 *__restrict__ V, uint32_t n,
                    PaperConsts c, const SceneDesc *__restrict__ scenes,
                    const uint16_t *__restrict__ sid, uint32_t *__restrict__ keys,
                    uint32_t *__restrict__ counts, uint32_t *__restrict__ pos) {
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
    count_cell_key(key, valid, k, counts, pos);
  }
}

__global__ void __launch_bounds__(256)
    k_predict_hash(const float4 *__restrict__ X, const float4 *__restrict__ V,
                   uint32_t n, PaperConsts c,
                   const SceneDesc *__restrict__ scenes,
                   const uint16_t *__restrict__ sid, uint32_t *__restrict__ keys,
                   uint32_t passes, uint32_t digit_bits, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_hist[kMaxHistWords];
  const uint32_t hist_words = passes << digit_bits;
  for (uint32_t i = threadIdx.x; i < hist_words; i += blockDim.x) s_hist[i] = 0;
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
    warp_digit_histogram(key, valid, passes, digit_bits, s_hist);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < hist_words; i += blockDim.x)
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

// Neighbour-list build from the predicted positions P (which equal the
// step-start positions the fallback recomputes).  Each member's slot is
// stored straight into its list word; the rest of the last word holds the
// particle's own slot.  kMasked: the candidates of each row are tested into
// a membership mask first and the members stored from it afterwards
// (scan_members_masked); the same lists either way.
template <int kBlock, bool kMasked>
__global__ void __launch_bounds__(kBlock)
    k_nbr_build(const float4 *__restrict__ P, NbrCtx nc, PaperConsts c,
                uint4 *__restrict__ nbr4, uint32_t *__restrict__ nbr_cnt) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = P[k];
  uint32_t *__restrict__ out = reinterpret_cast<uint32_t *>(nbr4) + 4ull * k;
  const size_t stride = 4ull * c.n;  // words from one list group to the next
  uint32_t cnt = 0;
  const auto store = [&](uint32_t j) {
    if (cnt < c.maxn) out[(size_t)(cnt >> 2) * stride + (cnt & 3u)] = j;
    ++cnt;
  };
  const SceneDesc &sc = scene_of(nc.scenes, nc.sid, k);
  if constexpr (kMasked)
    scan_members_masked(pk, nc.skeys[k], sc, nc.off, P, c, store);
  else
    scan_members(pk, nc.skeys[k], sc, nc.off, P, c, [&](uint32_t j, const Sep &) { store(j); });
  pad_list(out, stride, cnt, c.maxn, k);
  nbr_cnt[k] = cnt;
  record_count(nc.cnt_max, cnt);
}

// k_nbr_build fused with the first lambda pass: the same lists, and lambda
// summed over the members in the order the lists store them -- the bits
// k_lambda computes from the lists.  (In one kernel a warp executes the
// lambda arithmetic whenever any of its lanes has a member, so which form is
// faster depends on the scene; the tuner picks.)  kMasked: the members come
// from row masks (scan_members_masked) and each member's separation is
// evaluated again from its position, the same operations on the same values.
template <int kBlock, bool kMasked>
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
  const auto store = [&](uint32_t j) {
    if (cnt < c.maxn) out[(size_t)(cnt >> 2) * stride + (cnt & 3u)] = j;
    ++cnt;
  };
  const SceneDesc &sc = scene_of(nc.scenes, nc.sid, k);
  if constexpr (kMasked)
    scan_members_masked(pk, nc.skeys[k], sc, nc.off, P, c, [&](uint32_t j) {
      store(j);
      acc.add(separation(pk, __ldg(&P[j])), c);
    });
  else
    scan_members(pk, nc.skeys[k], sc, nc.off, P, c, [&](uint32_t j, const Sep &r) {
      store(j);
      acc.add(r, c);
    });
  pad_list(out, stride, cnt, c.maxn, k);
  nbr_cnt[k] = cnt;
  record_count(nc.cnt_max, cnt);
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
      [&](float4 pj) { lambda_pair(acc, pk, pj, c); });
  lambda_commit(k, pk, acc, c, Q, R);
}

template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock)
    k_delta(const float4 *__restrict__ Q, NbrCtx nc, PaperConsts c,
            float4 *__restrict__ D, float4 *__restrict__ P,
            const float *__restrict__ R, float4 *__restrict__ U, int last) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 qk = Q[k];
  DeltaAcc acc{0.f, 0.f, 0.f};
  // one neighbour walk per s_corr exponent form, chosen once per thread
  const auto walk = [&](auto twelve) {
    visit_neighbours<kBatch>(
        nc, k, [&](uint32_t j) { return __ldg(&Q[j]); },
        [&](float4 qj) { acc.template pair<decltype(twelve)::value>(qk, qj, c); });
  };
  if (c.scorr_n3 == 12) walk(std::true_type{});
  else walk(std::false_type{});
  delta_commit(k, acc, nc, c, D, P, R, U, last);
}

// Vorticity pass: omega_k and the sums the XSPH pass uses (pbf_paper.cuh).
template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock)
    k_vorticity(const float4 *__restrict__ P, const float4 *__restrict__ U,
                NbrCtx nc, PaperConsts c, float4 *__restrict__ Wo,
                float4 *__restrict__ PW, float4 *__restrict__ XS, float4 *__restrict__ SS) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = P[k];
  const float4 uk = U[k];
  VortAcc acc{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  visit_neighbours<kBatch>(
      nc, k, [&](uint32_t j) { return PU{__ldg(&P[j]), __ldg(&U[j])}; },
      [&](const PU &d) { acc.pair(pk, uk, d, c); });
  vort_commit(k, pk, uk, acc, Wo, PW, XS, SS);
}

// XSPH + commit: gathers (p_j, |omega_j|/rho_j) only.
template <int kBlock, int kBatch>
__global__ void __launch_bounds__(kBlock)
    k_xsph_commit(const float4 *__restrict__ PW, const float4 *__restrict__ U,
                  const float4 *__restrict__ Wv, const float4 *__restrict__ XS,
                  const float4 *__restrict__ SS, NbrCtx nc, PaperConsts c,
                  const uint32_t *__restrict__ ID2, float4 *__restrict__ X,
                  float4 *__restrict__ V, uint32_t *__restrict__ ID) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= c.n) return;
  const float4 pk = PW[k];
  XsphAcc acc{0.f, 0.f, 0.f};
  visit_neighbours<kBatch>(
      nc, k, [&](uint32_t j) { return __ldg(&PW[j]); },
      [&](const float4 &pj) { acc.pair(pk, pj, c); });
  xsph_commit(k, pk, load_own(&U[k]), load_own(&Wv[k]), load_own(&XS[k]), load_own(&SS[k]), acc,
              nc, c, ID2, X, V, ID);
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
  nc.cnt_max = d.nbr_max;
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
      X, V, n, c, scenes, sid, keys, plan.passes, plan.digit_bits,
      sort_scratch + plan.off_hist);
  return cudaGetLastError();
}

cudaError_t paper_predict_count(const float4 *X, const float4 *V, uint32_t n,
                                const PaperConsts &c, const SceneDesc *scenes,
                                const uint16_t *sid, uint32_t *keys,
                                const CellSortPlan &plan, uint32_t *cell_scratch,
                                cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_predict_count<<<min(blocks_for(n, 256), kStrideCtas), 256, 0, st>>>(
      X, V, n, c, scenes, sid, keys, cell_scratch + plan.off_counts, cell_scratch + plan.off_pos);
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
    switch (d.tune.block[KIND] * 2 + (d.tune.masked_build ? 1 : 0)) {                  \
      case 0: KERNEL<64, false><<<blocks_for(c.n, 64), 64, 0, st>>>(__VA_ARGS__); break;    \
      case 1: KERNEL<64, true><<<blocks_for(c.n, 64), 64, 0, st>>>(__VA_ARGS__); break;     \
      case 2: KERNEL<128, false><<<blocks_for(c.n, 128), 128, 0, st>>>(__VA_ARGS__); break; \
      case 3: KERNEL<128, true><<<blocks_for(c.n, 128), 128, 0, st>>>(__VA_ARGS__); break;  \
      case 4: KERNEL<256, false><<<blocks_for(c.n, 256), 256, 0, st>>>(__VA_ARGS__); break; \
      case 5: KERNEL<256, true><<<blocks_for(c.n, 256), 256, 0, st>>>(__VA_ARGS__); break;  \
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
  PBF_GATHER_LAUNCH(k_vorticity, kKindVorticity, d.P, d.U, make_ctx(d, c, sid), c, d.W, d.D, d.Q,
                    d.S);
  return cudaGetLastError();
}

cudaError_t paper_xsph_commit(const DeviceState &d, const PaperConsts &c,
                              const uint16_t *sid, cudaStream_t st) {
  PBF_GATHER_LAUNCH(k_xsph_commit, kKindXsph, d.D, d.U, d.W, d.Q, d.S, make_ctx(d, c, sid), c, d.ID2,
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
