// Launch-shape tuner of the gather passes (paper equations), shared by the
// single-scene simulation and the batch.  Host code only.
#pragma once

#include <cuda_runtime.h>

#include <limits>
#include <vector>

#include "pbf_host.hpp"

namespace pbf {

// Times every launch shape (threads per CTA x neighbour loads in flight x
// list build fused with the first lambda or not) over `trials` steps, each
// shape from the same state, and keeps for every gather pass the shape with
// the shortest launches.  Then it times whole steps of that choice against
// the staged tiles (pbf_tile.cu) from the same state and keeps the staged
// passes when their steps are more than kTuneMargin faster.  The current shapes are timed first and a pass
// moves to another shape only when that one is more than kTuneMargin
// faster: on a near-tie the pick would follow timing noise, and the
// defaults are the shapes measured fastest over a whole dam break, where
// later states separate shapes that tie on the starting lattice.  X, V and
// ID of the first n slots are saved before and restored after, so the
// caller's state is unchanged; since no shape changes a result bit, later
// steps are the ones an untuned run would take.
// `step()` launches one step eagerly on `st` and returns a pbf_status.
// per_launch_ms[k] receives the best time of kind k (0 if never launched).
constexpr double kTuneMargin = 0.01;

template <typename Step>
int paper_autotune(DeviceState &d, uint32_t n, cudaStream_t st, uint32_t trials, Step &&step,
                   double per_launch_ms[kGatherKinds]) {
  for (int k = 0; k < kGatherKinds; ++k) per_launch_ms[k] = 0.0;
  if (n == 0 || trials == 0) return PBF_OK;
  float4 *sx = nullptr, *sv = nullptr;
  uint32_t *sid = nullptr;
  GatherTimer *timer = new GatherTimer();
  int rc = PBF_OK;
  auto cuda = [&](cudaError_t e, const char *where) {
    if (e != cudaSuccess && rc == PBF_OK) rc = cuda_status(e, where);
    return rc == PBF_OK;
  };
  auto copy_state = [&](bool save) {
    const size_t b4 = (size_t)n * sizeof(float4), b1 = (size_t)n * sizeof(uint32_t);
    if (save) {
      return cuda(cudaMemcpyAsync(sx, d.X, b4, cudaMemcpyDeviceToDevice, st), "tune save") &&
             cuda(cudaMemcpyAsync(sv, d.V, b4, cudaMemcpyDeviceToDevice, st), "tune save") &&
             cuda(cudaMemcpyAsync(sid, d.ID, b1, cudaMemcpyDeviceToDevice, st), "tune save");
    }
    return cuda(cudaMemcpyAsync(d.X, sx, b4, cudaMemcpyDeviceToDevice, st), "tune restore") &&
           cuda(cudaMemcpyAsync(d.V, sv, b4, cudaMemcpyDeviceToDevice, st), "tune restore") &&
           cuda(cudaMemcpyAsync(d.ID, sid, b1, cudaMemcpyDeviceToDevice, st), "tune restore");
  };
  auto uniform = [](int block, int batch, int fuse) {
    GatherTuning t;
    for (int k = 0; k < kGatherKinds; ++k) {
      t.block[k] = (uint8_t)block;
      t.batch[k] = (uint8_t)batch;
    }
    t.fuse_first = (uint8_t)fuse;
    return t;
  };
  const GatherTuning before = d.tune;
  GatherTuning best = before;
  best.staged = 0;
  double best_ms[kGatherKinds];
  for (int k = 0; k < kGatherKinds; ++k) best_ms[k] = std::numeric_limits<double>::infinity();
  // Runs `trials` steps (one, untimed, when !timed) with shapes t from the
  // saved state; when timed, a pass takes t's shape if it is the first
  // timing of that pass (incumbent) or beats the best by the margin.
  auto trial = [&](const GatherTuning &t, bool timed, bool incumbent) {
    if (!copy_state(false)) return false;
    d.tune = t;
    d.timer = timed ? timer : nullptr;
    const uint32_t steps = timed ? trials : 1u;
    for (uint32_t i = 0; i < steps && rc == PBF_OK; ++i) rc = step();
    d.timer = nullptr;
    if (rc != PBF_OK) return false;
    if (!timed) return true;
    double ms[kGatherKinds];
    uint32_t cnt[kGatherKinds];
    if (!cuda(timer->collect(ms, cnt), "tune timing")) return false;
    for (int k = 0; k < kGatherKinds; ++k) {
      if (!cnt[k]) continue;
      const double tk = ms[k] / cnt[k];
      const bool first = best_ms[k] == std::numeric_limits<double>::infinity();
      if ((incumbent && first) || tk < best_ms[k] * (1.0 - kTuneMargin)) {
        best_ms[k] = tk;
        best.block[k] = t.block[k];
        best.batch[k] = t.batch[k];
      }
    }
    return true;
  };
  if (cuda(cudaMalloc(&sx, (size_t)n * sizeof(float4)), "tune alloc") &&
      cuda(cudaMalloc(&sv, (size_t)n * sizeof(float4)), "tune alloc") &&
      cuda(cudaMalloc(&sid, (size_t)n * sizeof(uint32_t)), "tune alloc") &&
      cuda(timer->init(), "tune events") && copy_state(true)) {
    for (int pass = 0; pass < 2 && rc == PBF_OK; ++pass) {
      // pass 0 loads every variant once (untimed); pass 1 times the current
      // shapes (split and fused) first, then every uniform shape
      const bool timed = pass == 1;
      if (timed) {
        GatherTuning cur = before;
        cur.staged = 0;
        for (int fuse = 0; fuse < 2 && rc == PBF_OK; ++fuse) {
          cur.fuse_first = (uint8_t)fuse;
          if (!trial(cur, true, true)) break;
        }
      }
      for (int fuse = 0; fuse < 2 && rc == PBF_OK; ++fuse)
        for (int bl = 0; bl < kBlockCodes && rc == PBF_OK; ++bl)
          for (int nb = 0; nb < kBatchCodes && rc == PBF_OK; ++nb)
            if (!trial(uniform(bl, nb, fuse), timed, false)) break;
    }
    if (rc == PBF_OK) {
      best.fuse_first =
          best_ms[kKindNbrLambda] < best_ms[kKindNbr] + best_ms[kKindLambda] ? 1u : 0u;
      best.staged = 0;
      for (int k = 0; k < kGatherKinds; ++k)
        per_launch_ms[k] = best_ms[k] < std::numeric_limits<double>::infinity() ? best_ms[k] : 0.0;
    }
    // whole steps: the L1-gather choice against the staged tiles
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == PBF_OK && cuda(cudaEventCreate(&e0), "tune events") &&
        cuda(cudaEventCreate(&e1), "tune events")) {
      GatherTuning staged = best;
      staged.staged = 1;
      float step_ms[2] = {0.f, 0.f};
      for (int v = 0; v < 2 && rc == PBF_OK; ++v) {
        const GatherTuning &t = v == 0 ? best : staged;
        if (!trial(t, false, false)) break;  // loads the variant's kernels
        if (!copy_state(false)) break;
        d.tune = t;
        if (!cuda(cudaEventRecord(e0, st), "tune timing")) break;
        for (uint32_t i = 0; i < trials && rc == PBF_OK; ++i) rc = step();
        if (rc != PBF_OK || !cuda(cudaEventRecord(e1, st), "tune timing") ||
            !cuda(cudaEventSynchronize(e1), "tune timing") ||
            !cuda(cudaEventElapsedTime(&step_ms[v], e0, e1), "tune timing"))
          break;
      }
      if (rc == PBF_OK && step_ms[1] < step_ms[0] * (1.0 - kTuneMargin)) best = staged;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    copy_state(false);
    cuda(cudaStreamSynchronize(st), "tune sync");
  }
  d.timer = nullptr;
  d.tune = rc == PBF_OK ? best : before;
  if (timer->ready) timer->destroy();
  delete timer;
  if (sx) cudaFree(sx);
  if (sv) cudaFree(sv);
  if (sid) cudaFree(sid);
  return rc;
}

}  // namespace pbf
