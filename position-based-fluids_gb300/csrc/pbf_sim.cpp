// The single-scene simulation object behind the C-ABI (include/pbf.h) and
// the neighbour-structure operator entry points.
//
// Reference: Simulation (src/Simulation.hpp:41-108, src/Simulation.cpp):
// construction (:34-88), init (:104-201), initCells (:203-230), step
// (:455-576), dumpData (:578-591), setWaveGenerator (Simulation.hpp:105-108).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "pbf_host.hpp"
#include "pbf_tune.hpp"

using namespace pbf;

namespace {
struct KernelTime {
  double ms = 0;
  uint64_t launches = 0;
  uint64_t groups = 0;
};
}  // namespace

struct pbf_sim {
  pbf_params prm{};
  uint32_t n = 0;
  std::vector<pbf_particle> particles;
  bool paper = true;
  // cell offsets by runs of cells (sparse grids: at least half as many
  // cells as particles) or by one binary search per cell
  bool offset_runs = false;
  bool inited = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  DeviceState d;
  PaperConsts pc{};
  RefConsts rc{};
  SceneDesc scene{};
  SortPlan plan;
  CellSortPlan cplan;  // paper mode's counting sort
  uint32_t ncells = 0;
  std::vector<void *> allocations;
  size_t device_bytes = 0;
  // CUDA graph of one step
  bool use_graph = true;
  cudaGraphExec_t graph = nullptr;
  // per-stage timing: each timed step is captured (with its boundary events
  // as event-record nodes) and launched as one graph, so the device runs it
  // back to back as an untimed step does and host enqueue gaps stay out of
  // the intervals
  bool timing = false;
  bool timed_capture = false;
  std::vector<cudaEvent_t> events;
  std::vector<int> event_stage;
  std::vector<const char *> event_name;
  std::vector<uint32_t> event_launches;
  size_t events_used = 0;
  double stage_acc[4] = {0, 0, 0, 0};
  uint32_t timed_steps = 0;
  std::map<std::string, KernelTime> kernel_times;
  float stage_ms[4] = {0, 0, 0, 0};
  bool have_times = false;
  bool stepped = false;
  bool scene_dirty = false;
  // adaptive neighbour-list capacity (paper): the largest count of each
  // step lands in page-locked memory; before launching a step the host
  // looks at the count of the step two back (the first step's right after
  // it) and grows the lists when it came within 1/8 of the capacity
  uint32_t *nbr_max_host = nullptr;
  // the copy of that count runs on a side branch of the step (forked after
  // the list build, joined at the step's end) so the solver passes do not
  // wait for it
  cudaStream_t count_stream = nullptr;
  cudaEvent_t count_fork = nullptr, count_join = nullptr;
  cudaEvent_t step_done[2] = {nullptr, nullptr};
  uint64_t launched = 0;  // steps launched since init or the last growth
  uint32_t list_grows = 0;
  // debug views
  int32_t *d_ranges = nullptr;
};

namespace {

template <typename T>
int dalloc(pbf_sim *s, T **p, size_t count) {
  void *q = nullptr;
  const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return cuda_status(e, "cudaMalloc");
  s->allocations.push_back(q);
  s->device_bytes += bytes;
  *p = static_cast<T *>(q);
  return PBF_OK;
}

void free_all(pbf_sim *s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  for (cudaEvent_t &e : s->step_done) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  if (s->nbr_max_host) cudaFreeHost(s->nbr_max_host);
  s->nbr_max_host = nullptr;
  if (s->count_fork) cudaEventDestroy(s->count_fork);
  if (s->count_join) cudaEventDestroy(s->count_join);
  if (s->count_stream) cudaStreamDestroy(s->count_stream);
  s->count_fork = s->count_join = nullptr;
  s->count_stream = nullptr;
  for (cudaEvent_t e : s->events) cudaEventDestroy(e);
  s->events.clear();
  for (void *p : s->allocations) cudaFree(p);
  s->allocations.clear();
  if (s->stream) cudaStreamDestroy(s->stream);
  s->stream = nullptr;
}

#define PBF_TRY(expr)                                  \
  do {                                                 \
    const cudaError_t e_ = (expr);                     \
    if (e_ != cudaSuccess) return cuda_status(e_, #expr); \
  } while (0)

#define PBF_TRY_STATUS(expr)      \
  do {                            \
    const int s_ = (expr);        \
    if (s_ != PBF_OK) return s_;  \
  } while (0)

// Records a boundary after a launch when timing is on: `stage` is one of the
// four reported stages (-1 = start of step), `name` the kernel (or kernel
// group) that just ran and `launches` how many launches that group was.
int mark(pbf_sim *s, int stage, const char *name, uint32_t launches,
         size_t *next) {
  if (!s->timing) return PBF_OK;
  if (*next >= s->events.size()) {
    cudaEvent_t e;
    PBF_TRY(cudaEventCreate(&e));
    s->events.push_back(e);
    s->event_stage.push_back(stage);
    s->event_name.push_back(name);
    s->event_launches.push_back(launches);
  }
  s->event_stage[*next] = stage;
  s->event_name[*next] = name;
  s->event_launches[*next] = launches;
  if (s->timed_capture)
    PBF_TRY(cudaEventRecordWithFlags(s->events[*next], s->stream, cudaEventRecordExternal));
  else
    PBF_TRY(cudaEventRecord(s->events[*next], s->stream));
  ++*next;
  return PBF_OK;
}

cudaError_t step_offsets(pbf_sim *s) {
  DeviceState &d = s->d;
  if (s->offset_runs)
    return cell_offsets_runs(d.skeys, s->n, s->ncells, d.offsets, d.runs, d.runs_count, s->stream);
  return cell_offsets(d.skeys, s->n, s->ncells, d.offsets, s->stream);
}

// Copies the step's largest neighbour count (complete once the list build
// has run) to page-locked host memory on the side stream; join_count_copy
// at the end of the step makes the step wait for it.
cudaError_t fork_count_copy(pbf_sim *s) {
  cudaError_t e = cudaEventRecord(s->count_fork, s->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s->count_stream, s->count_fork, 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->nbr_max_host, s->d.nbr_max, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                        s->count_stream);
  if (e == cudaSuccess) e = cudaEventRecord(s->count_join, s->count_stream);
  return e;
}

cudaError_t join_count_copy(pbf_sim *s) {
  return cudaStreamWaitEvent(s->stream, s->count_join, 0);
}

int launch_step(pbf_sim *s) {
  DeviceState &d = s->d;
  const cudaStream_t st = s->stream;
  const uint32_t n = s->n;
  const uint32_t passes = s->plan.passes;
  size_t ev = 0;
  s->events_used = 0;
  PBF_TRY_STATUS(mark(s, -1, "start", 0, &ev));
  if (s->paper && !d.tune.radix_sort) {
    // counting sort by cell: the counts, the offsets, the scatter and the
    // order within each cell
    PBF_TRY(cell_sort_clear(s->cplan, d.cell_scratch, false, st));
    PBF_TRY(cudaMemsetAsync(d.nbr_max, 0, sizeof(uint32_t), st));
    PBF_TRY(paper_predict_count(d.X, d.V, n, s->pc, d.scenes, nullptr, d.keys, s->cplan,
                                d.cell_scratch, st));
    PBF_TRY_STATUS(mark(s, 0, "predict_hash", 1, &ev));
    PBF_TRY(cell_sort_finish(s->cplan, d.keys, d.cell_scratch, d.offsets, d.skeys, d.perm, d.err,
                             st));
    PBF_TRY_STATUS(mark(s, 0, "cell_sort", cell_sort_launches(), &ev));
  } else if (s->paper) {
    PBF_TRY(sort_clear(s->plan, d.sort_scratch, st));
    PBF_TRY(cudaMemsetAsync(d.nbr_max, 0, sizeof(uint32_t), st));
    PBF_TRY(paper_predict_hash(d.X, d.V, n, s->pc, d.scenes, nullptr, d.keys,
                               s->plan, d.sort_scratch, st));
    PBF_TRY_STATUS(mark(s, 0, "predict_hash", 1, &ev));
    PBF_TRY(sort_scan(s->plan, d.sort_scratch, st));
    PBF_TRY(sort_passes(s->plan, d.keys, nullptr, d.skeys, d.perm,
                        d.sort_scratch, d.err, st));
    PBF_TRY_STATUS(mark(s, 0, "sort_onesweep", 1 + passes, &ev));
    PBF_TRY(step_offsets(s));
    PBF_TRY_STATUS(mark(s, 0, "cell_offsets", 1, &ev));
  } else {
    PBF_TRY(sort_clear(s->plan, d.sort_scratch, st));
  }
  if (s->paper) {
    PBF_TRY(paper_reorder(d.perm, d.X, d.V, d.ID, n, s->pc, d.X2, d.V2, d.ID2,
                          d.P, d.D, st));
    PBF_TRY_STATUS(mark(s, 0, "reorder", 1, &ev));
    const uint32_t iters = s->prm.solver_iterations;
    if (d.tune.staged) {
      PBF_TRY(tile_plan(d, s->pc, nullptr, 1, st));
      PBF_TRY_STATUS(mark(s, 0, "tile_plan", 1, &ev));
      for (uint32_t it = 0; it < iters; ++it) {
        if (it == 0) {
          PBF_TRY(tile_nbr_build(d, s->pc, nullptr, 1, st));
          PBF_TRY(fork_count_copy(s));
          PBF_TRY_STATUS(mark(s, 1, "nbr_build", 1, &ev));
        }
        PBF_TRY(tile_lambda(d, s->pc, nullptr, 1, st));
        PBF_TRY_STATUS(mark(s, 1, "lambda", 1, &ev));
        PBF_TRY(tile_delta(d, s->pc, nullptr, 1, it + 1 == iters, st));
        PBF_TRY_STATUS(mark(s, 2, "delta", 1, &ev));
      }
      PBF_TRY(tile_vorticity(d, s->pc, nullptr, 1, st));
      PBF_TRY_STATUS(mark(s, 3, "vorticity", 1, &ev));
      PBF_TRY(tile_xsph_commit(d, s->pc, nullptr, 1, st));
      PBF_TRY_STATUS(mark(s, 3, "xsph_commit", 1, &ev));
      PBF_TRY(join_count_copy(s));
    } else {
      for (uint32_t it = 0; it < iters; ++it) {
        if (it == 0 && d.tune.fuse_first) {
          PBF_TRY(paper_nbr_lambda(d, s->pc, nullptr, st));
          PBF_TRY(fork_count_copy(s));
          PBF_TRY_STATUS(mark(s, 1, "nbr_lambda", 1, &ev));
        } else {
          if (it == 0) {
            PBF_TRY(paper_nbr_build(d, s->pc, nullptr, st));
            PBF_TRY(fork_count_copy(s));
            PBF_TRY_STATUS(mark(s, 1, "nbr_build", 1, &ev));
          }
          PBF_TRY(paper_lambda(d, s->pc, nullptr, st));
          PBF_TRY_STATUS(mark(s, 1, "lambda", 1, &ev));
        }
        PBF_TRY(paper_delta(d, s->pc, nullptr, it + 1 == iters, st));
        PBF_TRY_STATUS(mark(s, 2, "delta", 1, &ev));
      }
      PBF_TRY(paper_vorticity(d, s->pc, nullptr, st));
      PBF_TRY_STATUS(mark(s, 3, "vorticity", 1, &ev));
      PBF_TRY(paper_xsph_commit(d, s->pc, nullptr, st));
      PBF_TRY_STATUS(mark(s, 3, "xsph_commit", 1, &ev));
      PBF_TRY(join_count_copy(s));
    }
  } else {
    PBF_TRY(rc_predict_hash(d.X, d.V, d.P, n, s->rc, d.scenes, d.keys, s->plan,
                            d.sort_scratch, st));
    PBF_TRY_STATUS(mark(s, 0, "rc_predict_hash", 1, &ev));
    PBF_TRY(sort_scan(s->plan, d.sort_scratch, st));
    PBF_TRY(sort_passes(s->plan, d.keys, nullptr, d.skeys, d.perm,
                        d.sort_scratch, d.err, st));
    PBF_TRY_STATUS(mark(s, 0, "sort_onesweep", 1 + passes, &ev));
    PBF_TRY(step_offsets(s));
    PBF_TRY_STATUS(mark(s, 0, "cell_offsets", 1, &ev));
    PBF_TRY(rc_gather(d.P, d.perm, n, d.PS, st));
    PBF_TRY_STATUS(mark(s, 0, "rc_gather", 1, &ev));
    float4 *cur = d.PS, *alt = d.PS2;
    const uint32_t iters = s->prm.solver_iterations;
    for (uint32_t it = 0; it < iters; ++it) {
      PBF_TRY(rc_lambda(cur, d.SS, d.offsets, n, s->rc, st));
      PBF_TRY_STATUS(mark(s, 1, "rc_lambda", 1, &ev));
      PBF_TRY(rc_delta(cur, alt, d.SS, d.perm, d.offsets, d.X, d.V, d.P, d.VS, n, s->rc,
                       d.scenes, it + 1 == iters, st));
      PBF_TRY_STATUS(mark(s, 2, "rc_delta", 1, &ev));
      std::swap(cur, alt);
    }
    PBF_TRY(rc_xsph(cur, d.VS, d.DV, d.perm, d.offsets, n, s->rc, st));
    PBF_TRY_STATUS(mark(s, 3, "rc_xsph", 1, &ev));
    PBF_TRY(rc_commit(d.X, d.V, d.P, d.DV, n, st));
    PBF_TRY_STATUS(mark(s, 3, "rc_commit", 1, &ev));
  }
  s->events_used = ev;
  return PBF_OK;
}

int upload_scene(pbf_sim *s) {
  PBF_TRY(cudaMemcpyAsync(s->d.scenes, &s->scene, sizeof(SceneDesc),
                          cudaMemcpyHostToDevice, s->stream));
  s->scene_dirty = false;
  return PBF_OK;
}

int check_device_error(pbf_sim *s) {
  uint32_t flag = 0;
  PBF_TRY(cudaMemcpyAsync(&flag, s->d.err, sizeof flag, cudaMemcpyDeviceToHost,
                          s->stream));
  PBF_TRY(cudaStreamSynchronize(s->stream));
  if (flag) {
    PBF_TRY(cudaMemsetAsync(s->d.err, 0, sizeof(uint32_t), s->stream));
    PBF_TRY(cudaStreamSynchronize(s->stream));
    set_error_message("device error flag " + std::to_string(flag));
    return PBF_ERR_DEVICE;
  }
  return PBF_OK;
}

int build_graph(pbf_sim *s) {
  if (s->graph) return PBF_OK;
  cudaGraph_t g = nullptr;
  PBF_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  const bool was_timing = s->timing;
  s->timing = false;
  const int rc = launch_step(s);
  s->timing = was_timing;
  const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc != PBF_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
  const cudaError_t ie = cudaGraphInstantiate(&s->graph, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    s->graph = nullptr;
    return cuda_status(ie, "cudaGraphInstantiate");
  }
  return PBF_OK;
}

// One step with its stage boundaries, captured and launched as a graph.
int launch_timed_step(pbf_sim *s) {
  // the boundary events exist before the capture (one per mark of a step:
  // at most 8 outside the solver loop, 2 per iteration)
  const size_t marks = 16 + 2 * (size_t)s->prm.solver_iterations;
  while (s->events.size() < marks) {
    cudaEvent_t e;
    PBF_TRY(cudaEventCreate(&e));
    s->events.push_back(e);
    s->event_stage.push_back(-1);
    s->event_name.push_back("");
    s->event_launches.push_back(0);
  }
  cudaGraph_t g = nullptr;
  PBF_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  s->timed_capture = true;
  const int rc = launch_step(s);
  s->timed_capture = false;
  const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc != PBF_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
  cudaGraphExec_t x = nullptr;
  cudaError_t le = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (le == cudaSuccess) le = cudaGraphLaunch(x, s->stream);
  if (x) cudaGraphExecDestroy(x);  // released once the launch completes
  if (le != cudaSuccess) return cuda_status(le, "timed step graph");
  return PBF_OK;
}

// Accumulates the stage and per-kernel times of the step just launched.
int collect_times(pbf_sim *s) {
  if (s->events_used < 2) return PBF_OK;
  PBF_TRY(cudaEventSynchronize(s->events[s->events_used - 1]));
  for (size_t q = 1; q < s->events_used; ++q) {
    float ms = 0;
    PBF_TRY(cudaEventElapsedTime(&ms, s->events[q - 1], s->events[q]));
    const int st = s->event_stage[q];
    if (st >= 0 && st < 4) s->stage_acc[st] += ms;
    KernelTime &kt = s->kernel_times[s->event_name[q]];
    kt.ms += ms;
    kt.launches += s->event_launches[q];
    kt.groups += 1;
  }
  s->timed_steps += 1;
  for (int st = 0; st < 4; ++st) s->stage_ms[st] = (float)(s->stage_acc[st] / s->timed_steps);
  s->have_times = true;
  return PBF_OK;
}

bool ready(const pbf_sim *s) { return s && s->inited; }

// Largest list capacity (pbf_params.max_neighbours range).
constexpr uint32_t kMaxListCapacity = 1024;

// Before a paper-mode step: the largest neighbour count of a recent step
// (the first step's right after it, later the step two back, which leaves
// one step queued on the device while the host waits) against the list
// capacity.  When it came within 1/8 of the capacity the lists grow to 1.5x
// that count (multiple of 8, at most 1024) before the step is launched, so a
// scene whose sets outgrow the lists re-derives them from the cells in at
// most the steps already queued.
int adapt_lists(pbf_sim *s) {
  if (!s->paper || !s->prm.grow_lists || s->launched == 0) return PBF_OK;
  const uint64_t wait_for = s->launched >= 2 ? s->launched - 2 : 0;
  PBF_TRY(cudaEventSynchronize(s->step_done[wait_for & 1]));
  const uint32_t mx = *reinterpret_cast<volatile uint32_t *>(s->nbr_max_host);
  const uint32_t cap = s->pc.maxn;
  if (cap >= kMaxListCapacity || mx <= cap - cap / 8) return PBF_OK;
  const uint32_t grown = std::min(kMaxListCapacity, ((mx + mx / 2 + 7) / 8) * 8);
  if (grown <= cap) return PBF_OK;
  PBF_TRY(cudaStreamSynchronize(s->stream));
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  DeviceState &d = s->d;
  const size_t old_bytes = (size_t)paper_list_words(cap) * s->n * sizeof(uint4);
  const size_t new_bytes = (size_t)paper_list_words(grown) * s->n * sizeof(uint4);
  void *q = nullptr;
  PBF_TRY(cudaMalloc(&q, std::max<size_t>(new_bytes, 16)));
  for (void *&a : s->allocations)
    if (a == d.nbr) {
      cudaFree(a);
      a = q;
    }
  d.nbr = static_cast<uint4 *>(q);
  s->device_bytes += new_bytes - std::max<size_t>(old_bytes, 16);
  s->pc.maxn = grown;
  s->launched = 0;
  ++s->list_grows;
  return PBF_OK;
}

}  // namespace

extern "C" {

int pbf_create(const pbf_params *params, const pbf_particle *particles,
               uint32_t n, pbf_sim **out) {
  if (!params || !out || (!particles && n)) return PBF_ERR_INVALID;
  *out = nullptr;
  const int v = validate_params(*params, n);
  if (v != PBF_OK) return v;
  std::unique_ptr<pbf_sim> s(new pbf_sim());
  s->prm = *params;
  s->n = n;
  s->particles.assign(particles, particles + n);
  s->paper = params->mode == PBF_MODE_PAPER;
  s->ncells = (uint32_t)grid_cells(*params);
  s->scene = make_scene(*params);
  s->rc = make_ref_consts(*params);
  s->rc.n = n;
  s->pc = make_paper_consts(*params, n);
  s->plan = make_sort_plan(n, bits_for(s->ncells));
  s->cplan = make_cell_sort_plan(n, s->ncells);
  *out = s.release();
  return PBF_OK;
}

int pbf_init(pbf_sim *s) {
  if (!s) return PBF_ERR_INVALID;
  if (s->inited) return PBF_ERR_STATE;
  PBF_TRY(cudaGetDevice(&s->device));
  PBF_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  DeviceState &d = s->d;
  const size_t n = s->n;
  int rc = PBF_OK;
  auto A = [&](auto **p, size_t count) {
    if (rc == PBF_OK) rc = dalloc(s, p, count);
  };
  A(&d.X, n);
  A(&d.V, n);
  A(&d.P, n);
  A(&d.keys, n);
  A(&d.skeys, n);
  A(&d.perm, n);
  A(&d.offsets, (size_t)s->ncells + 1);
  s->offset_runs = (uint64_t)s->ncells * 2u >= (uint64_t)n;
  if (s->offset_runs) {
    A(&d.runs, offset_runs_capacity(s->ncells));
    A(&d.runs_count, 1);
  }
  A(&d.sort_scratch, s->plan.words);
  A(&d.err, 1);
  A(&d.scenes, 1);
  A(&d.io_pos, n);
  A(&d.io_vel, n);
  if (s->paper) {
    A(&d.ID, n);
    A(&d.ID2, n);
    A(&d.X2, n);
    A(&d.V2, n);
    A(&d.Q, n);
    A(&d.D, n);
    A(&d.U, n);
    A(&d.W, n);
    A(&d.S, n);
    A(&d.R, n);
    A(&d.nbr_cnt, n);
    A(&d.nbr_max, 1);
    A(&d.cell_scratch, s->cplan.words);
    A(&d.nbr, (size_t)paper_list_words(s->pc.maxn) * n);
    d.blk_total = d.blk_cap = scene_blocks(s->scene);
    A(&d.blk_list, d.blk_cap);
    A(&d.blk_count, 3);
  } else {
    A(&d.PS, n);
    A(&d.PS2, n);
    A(&d.VS, n);
    A(&d.DV, n);
    A(&d.SS, n);
  }
  if (rc == PBF_OK && s->paper) {
    cudaError_t te = tile_init();
    if (te == cudaSuccess) te = cudaMallocHost(&s->nbr_max_host, sizeof(uint32_t));
    for (cudaEvent_t &e : s->step_done)
      if (te == cudaSuccess) te = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (te == cudaSuccess) te = cudaStreamCreateWithFlags(&s->count_stream, cudaStreamNonBlocking);
    if (te == cudaSuccess) te = cudaEventCreateWithFlags(&s->count_fork, cudaEventDisableTiming);
    if (te == cudaSuccess) te = cudaEventCreateWithFlags(&s->count_join, cudaEventDisableTiming);
    if (te != cudaSuccess) rc = cuda_status(te, "pbf_init");
    else *s->nbr_max_host = 0;
  }
  if (rc != PBF_OK) {
    free_all(s);
    return rc;
  }
  // Initial state in the dumpData layout (src/Simulation.cpp:120-134).
  std::vector<float4> pos(n), vel(n);
  for (size_t i = 0; i < n; ++i) {
    const pbf_particle &p = s->particles[i];
    pos[i] = make_float4(p.x[0], p.x[1], p.x[2], 0.0f);
    vel[i] = make_float4(p.v[0], p.v[1], p.v[2], p.m);
  }
  PBF_TRY(cudaMemsetAsync(d.err, 0, sizeof(uint32_t), s->stream));
  if (s->paper) PBF_TRY(cell_sort_clear(s->cplan, d.cell_scratch, true, s->stream));
  PBF_TRY(cudaMemsetAsync(d.P, 0, n * sizeof(float4), s->stream));
  PBF_TRY(cudaMemsetAsync(d.offsets, 0, ((size_t)s->ncells + 1) * sizeof(uint32_t),
                          s->stream));
  PBF_TRY(cudaMemcpyAsync(d.X, pos.data(), n * sizeof(float4),
                          cudaMemcpyHostToDevice, s->stream));
  PBF_TRY(cudaMemcpyAsync(d.V, vel.data(), n * sizeof(float4),
                          cudaMemcpyHostToDevice, s->stream));
  if (s->paper) PBF_TRY(iota_u32(d.ID, s->n, s->stream));
  PBF_TRY_STATUS(upload_scene(s));
  PBF_TRY(cudaStreamSynchronize(s->stream));
  s->inited = true;
  return PBF_OK;
}

int pbf_init_cells(pbf_sim *s) { return ready(s) ? PBF_OK : PBF_ERR_STATE; }

int pbf_step(pbf_sim *s, uint32_t nsteps) {
  if (!ready(s)) return PBF_ERR_STATE;
  for (uint32_t k = 0; k < nsteps; ++k) {
    if (s->scene_dirty) PBF_TRY_STATUS(upload_scene(s));
    PBF_TRY_STATUS(adapt_lists(s));
    if (s->timing) {
      PBF_TRY_STATUS(s->use_graph ? launch_timed_step(s) : launch_step(s));
      PBF_TRY_STATUS(collect_times(s));
    } else if (s->use_graph) {
      PBF_TRY_STATUS(build_graph(s));
      PBF_TRY(cudaGraphLaunch(s->graph, s->stream));
    } else {
      PBF_TRY_STATUS(launch_step(s));
    }
    if (s->paper) {
      PBF_TRY(cudaEventRecord(s->step_done[s->launched & 1], s->stream));
      ++s->launched;
    }
    s->stepped = true;
  }
  return PBF_OK;
}

int pbf_list_capacity(const pbf_sim *s, uint32_t *capacity, uint32_t *grows) {
  if (!s || !capacity) return PBF_ERR_INVALID;
  *capacity = s->pc.maxn;
  if (grows) *grows = s->list_grows;
  return PBF_OK;
}

int pbf_sync(pbf_sim *s) {
  if (!ready(s)) return PBF_ERR_STATE;
  return check_device_error(s);
}

int pbf_set_state_async(pbf_sim *s, const float *pos4, const float *vel4) {
  if (!ready(s) || !pos4 || !vel4) return ready(s) ? PBF_ERR_INVALID : PBF_ERR_STATE;
  DeviceState &d = s->d;
  const size_t bytes = (size_t)s->n * sizeof(float4);
  if (s->paper) {
    PBF_TRY(cudaMemcpyAsync(d.io_pos, pos4, bytes, cudaMemcpyHostToDevice, s->stream));
    PBF_TRY(cudaMemcpyAsync(d.io_vel, vel4, bytes, cudaMemcpyHostToDevice, s->stream));
    PBF_TRY(scatter_from_input_order(d.io_pos, d.io_vel, d.ID, s->n, d.X, d.V,
                                     s->stream));
  } else {
    PBF_TRY(cudaMemcpyAsync(d.X, pos4, bytes, cudaMemcpyHostToDevice, s->stream));
    PBF_TRY(cudaMemcpyAsync(d.V, vel4, bytes, cudaMemcpyHostToDevice, s->stream));
  }
  return PBF_OK;
}

int pbf_dump_data_async(pbf_sim *s, float *pos4, float *vel4) {
  if (!ready(s) || !pos4 || !vel4) return ready(s) ? PBF_ERR_INVALID : PBF_ERR_STATE;
  DeviceState &d = s->d;
  const size_t bytes = (size_t)s->n * sizeof(float4);
  const float4 *sp = d.X, *sv = d.V;
  if (s->paper) {
    PBF_TRY(gather_to_input_order(d.X, d.V, d.ID, s->n, d.io_pos, d.io_vel,
                                  s->stream));
    sp = d.io_pos;
    sv = d.io_vel;
  }
  PBF_TRY(cudaMemcpyAsync(pos4, sp, bytes, cudaMemcpyDeviceToHost, s->stream));
  PBF_TRY(cudaMemcpyAsync(vel4, sv, bytes, cudaMemcpyDeviceToHost, s->stream));
  return PBF_OK;
}

int pbf_set_state(pbf_sim *s, const float *pos4, const float *vel4) {
  PBF_TRY_STATUS(pbf_set_state_async(s, pos4, vel4));
  PBF_TRY(cudaStreamSynchronize(s->stream));
  return PBF_OK;
}

int pbf_dump_data(pbf_sim *s, float *pos4, float *vel4) {
  PBF_TRY_STATUS(pbf_dump_data_async(s, pos4, vel4));
  return check_device_error(s);
}

int pbf_host_alloc(size_t bytes, void **out) {
  if (!out) return PBF_ERR_INVALID;
  PBF_TRY(cudaMallocHost(out, bytes ? bytes : 16));
  return PBF_OK;
}

int pbf_host_free(void *ptr) {
  if (ptr) PBF_TRY(cudaFreeHost(ptr));
  return PBF_OK;
}

int pbf_set_wave(pbf_sim *s, float value) {
  if (!s) return PBF_ERR_INVALID;
  s->scene.wave = value;
  s->scene_dirty = true;
  return PBF_OK;
}

int pbf_get_num_particles(const pbf_sim *s, uint32_t *n) {
  if (!s || !n) return PBF_ERR_INVALID;
  *n = s->n;
  return PBF_OK;
}

int pbf_get_sizes(const pbf_sim *s, float min4[4], float max4[4]) {
  if (!s || !min4 || !max4) return PBF_ERR_INVALID;
  min4[0] = s->prm.x_min;
  min4[1] = s->prm.y_min;
  min4[2] = s->prm.z_min;
  min4[3] = 0.0f;
  max4[0] = s->prm.x_max;
  max4[1] = s->prm.y_max;
  max4[2] = s->prm.z_max;
  max4[3] = 0.0f;
  return PBF_OK;
}

int pbf_get_stream(const pbf_sim *s, void **stream) {
  if (!s || !stream) return PBF_ERR_INVALID;
  if (!s->inited) return PBF_ERR_STATE;
  *stream = (void *)s->stream;
  return PBF_OK;
}

int pbf_set_stage_timing(pbf_sim *s, int enable) {
  if (!s) return PBF_ERR_INVALID;
  s->timing = enable != 0;
  s->kernel_times.clear();
  for (double &a : s->stage_acc) a = 0;
  s->timed_steps = 0;
  s->have_times = false;
  return PBF_OK;
}

int pbf_kernel_times(pbf_sim *s, uint32_t cap, char *names, float *total_ms,
                     uint32_t *launches, uint32_t *count) {
  if (!s || !count) return PBF_ERR_INVALID;
  uint32_t q = 0;
  for (const auto &kv : s->kernel_times) {
    if (q < cap) {
      if (names) {
        std::strncpy(names + 32 * (size_t)q, kv.first.c_str(), 31);
        names[32 * (size_t)q + 31] = '\0';
      }
      if (total_ms) total_ms[q] = (float)kv.second.ms;
      if (launches) launches[q] = (uint32_t)kv.second.launches;
    }
    ++q;
  }
  *count = q;
  return PBF_OK;
}

int pbf_stage_times(pbf_sim *s, float ms[4]) {
  if (!s || !ms) return PBF_ERR_INVALID;
  if (!s->have_times) return PBF_ERR_STATE;
  std::memcpy(ms, s->stage_ms, sizeof s->stage_ms);
  return PBF_OK;
}

int pbf_set_graph(pbf_sim *s, int enable) {
  if (!s) return PBF_ERR_INVALID;
  s->use_graph = enable != 0;
  return PBF_OK;
}

int pbf_launches_per_step(const pbf_sim *s, uint32_t *launches) {
  if (!s || !launches) return PBF_ERR_INVALID;
  const uint32_t it = s->prm.solver_iterations;
  const uint32_t sort = s->paper && !s->d.tune.radix_sort
                            ? cell_sort_launches()
                            : 1u /*scan*/ + s->plan.passes + (s->offset_runs ? 2u : 1u) /*offsets*/;
  if (s->paper)
    *launches = 1u /*predict+hash*/ + sort + 1u /*reorder*/ + paper_first_launches(s->d) +
                2u * it - 1u + 2u;
  else
    *launches = 1u + sort + 1u /*gather*/ + 2u * it + 2u;
  return PBF_OK;
}

int pbf_render(pbf_sim *s, const pbf_camera *cam, uint32_t width, uint32_t height,
               uint8_t *rgb) {
  if (!ready(s)) return s ? PBF_ERR_STATE : PBF_ERR_INVALID;
  if (!cam || !rgb) return PBF_ERR_INVALID;
  return render_particles(s->d.X, s->paper ? s->d.ID : nullptr, s->n, s->prm, *cam, width,
                          height, rgb, s->stream);
}

int pbf_autotune(pbf_sim *s, uint32_t trial_steps, pbf_tuning *out) {
  if (!ready(s)) return s ? PBF_ERR_STATE : PBF_ERR_INVALID;
  if (trial_steps < 1 || trial_steps > 32) return PBF_ERR_INVALID;
  double ms[kGatherKinds] = {0, 0, 0, 0, 0, 0};
  if (s->paper) {
    const bool timing = s->timing;
    s->timing = false;
    const int rc = paper_autotune(s->d, s->n, s->stream, trial_steps,
                                  [&]() { return launch_step(s); }, ms);
    s->timing = timing;
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
    if (rc != PBF_OK) return rc;
    PBF_TRY_STATUS(check_device_error(s));
  }
  if (out) to_pbf_tuning(s->d.tune, ms, out);
  return PBF_OK;
}

int pbf_get_tuning(const pbf_sim *s, pbf_tuning *out) {
  if (!s || !out) return PBF_ERR_INVALID;
  to_pbf_tuning(s->d.tune, nullptr, out);
  return PBF_OK;
}

int pbf_set_tuning(pbf_sim *s, const pbf_tuning *t) {
  if (!s || !t) return PBF_ERR_INVALID;
  PBF_TRY_STATUS(to_gather_tuning(*t, &s->d.tune));
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  return PBF_OK;
}

int pbf_get_density(pbf_sim *s, float *density) {
  if (!ready(s) || !density) return ready(s) ? PBF_ERR_INVALID : PBF_ERR_STATE;
  const size_t n = s->n;
  if (s->paper) {
    float *tmp = reinterpret_cast<float *>(s->d.io_pos);
    PBF_TRY(gather_scalar_to_input_order(s->d.R, s->d.ID, s->n, tmp, s->stream));
    PBF_TRY(cudaMemcpyAsync(density, tmp, n * sizeof(float),
                            cudaMemcpyDeviceToHost, s->stream));
    PBF_TRY(cudaStreamSynchronize(s->stream));
  } else {
    std::vector<float4> p(n);
    PBF_TRY(cudaMemcpyAsync(p.data(), s->d.P, n * sizeof(float4),
                            cudaMemcpyDeviceToHost, s->stream));
    PBF_TRY(cudaStreamSynchronize(s->stream));
    for (size_t i = 0; i < n; ++i) density[i] = p[i].w;
  }
  return PBF_OK;
}

int pbf_neighbour_stats(pbf_sim *s, uint32_t *max_count, uint32_t *overflow) {
  if (!ready(s) || !max_count || !overflow) return ready(s) ? PBF_ERR_INVALID : PBF_ERR_STATE;
  if (!s->paper || !s->stepped) return PBF_ERR_STATE;
  std::vector<uint32_t> cnt(s->n);
  PBF_TRY(cudaMemcpyAsync(cnt.data(), s->d.nbr_cnt, (size_t)s->n * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, s->stream));
  PBF_TRY(cudaStreamSynchronize(s->stream));
  uint32_t mx = 0, over = 0;
  for (uint32_t c : cnt) {
    mx = c > mx ? c : mx;
    over += c > s->pc.maxn ? 1u : 0u;
  }
  *max_count = mx;
  *overflow = over;
  return PBF_OK;
}

int pbf_tile_stats(pbf_sim *s, uint32_t *staged, uint32_t *unstaged) {
  if (!ready(s) || !staged || !unstaged) return ready(s) ? PBF_ERR_INVALID : PBF_ERR_STATE;
  if (!s->paper || !s->stepped) return PBF_ERR_STATE;
  uint32_t st[3] = {0u, 0u, 0u};
  if (s->d.tune.staged) {
    PBF_TRY(cudaMemcpyAsync(st, s->d.blk_count, sizeof st, cudaMemcpyDeviceToHost, s->stream));
    PBF_TRY(cudaStreamSynchronize(s->stream));
  }
  *staged = st[1];
  *unstaged = st[2];
  return PBF_OK;
}

int pbf_get_cells(pbf_sim *s, uint32_t *hash, uint32_t *perm, int32_t *ranges) {
  if (!ready(s)) return PBF_ERR_STATE;
  if (!s->stepped) return PBF_ERR_STATE;
  const size_t n = s->n;
  std::vector<uint32_t> skeys(n), p(n), id(n);
  PBF_TRY(cudaMemcpyAsync(skeys.data(), s->d.skeys, n * 4, cudaMemcpyDeviceToHost, s->stream));
  PBF_TRY(cudaMemcpyAsync(p.data(), s->paper ? s->d.ID : s->d.perm, n * 4,
                          cudaMemcpyDeviceToHost, s->stream));
  if (!s->paper && hash)
    PBF_TRY(cudaMemcpyAsync(hash, s->d.keys, n * 4, cudaMemcpyDeviceToHost, s->stream));
  if (ranges) {
    if (!s->d_ranges) PBF_TRY_STATUS(dalloc(s, &s->d_ranges, 2 * (size_t)s->ncells));
    PBF_TRY(find_cells(s->d.offsets, s->ncells, s->d_ranges, s->stream));
    PBF_TRY(cudaMemcpyAsync(ranges, s->d_ranges, (size_t)s->ncells * 8,
                            cudaMemcpyDeviceToHost, s->stream));
  }
  PBF_TRY(cudaStreamSynchronize(s->stream));
  if (s->paper && hash)
    for (size_t q = 0; q < n; ++q) hash[p[q]] = skeys[q];
  if (perm) std::memcpy(perm, p.data(), n * 4);
  return PBF_OK;
}

int pbf_destroy(pbf_sim *s) {
  if (!s) return PBF_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
  return PBF_OK;
}

/* ------------------------------------------------------------ operators */
int pbf_op_cell_hash(const pbf_params *params, const float *d_pred4, uint32_t n,
                     uint32_t *d_hash, void *stream) {
  if (!params || (n && (!d_pred4 || !d_hash))) return PBF_ERR_INVALID;
  if (grid_cells(*params) == 0 || grid_cells(*params) > (1ull << 31)) return PBF_ERR_INVALID;
  const SceneDesc sc = make_scene(*params);
  PBF_TRY(cell_hash(reinterpret_cast<const float4 *>(d_pred4), n, sc, d_hash,
                    (cudaStream_t)stream));
  return PBF_OK;
}

size_t pbf_op_sort_scratch_bytes(uint32_t n, uint32_t key_bits) {
  return make_sort_plan(n, key_bits).words * sizeof(uint32_t);
}

int pbf_op_sort_pairs(const uint32_t *d_keys_in, const uint32_t *d_vals_in,
                      uint32_t n, uint32_t key_bits, uint32_t *d_keys_out,
                      uint32_t *d_vals_out, void *d_scratch,
                      size_t scratch_bytes, void *stream) {
  if (n == 0) return PBF_OK;
  if (!d_keys_in || !d_keys_out || !d_vals_out || !d_scratch) return PBF_ERR_INVALID;
  if (key_bits < 1 || key_bits > 32 || n >= (1u << 30)) return PBF_ERR_INVALID;
  const SortPlan plan = make_sort_plan(n, key_bits);
  if (scratch_bytes < plan.words * sizeof(uint32_t)) return PBF_ERR_INVALID;
  uint32_t *scratch = static_cast<uint32_t *>(d_scratch);
  uint32_t *err = scratch + plan.off_counter + 31;
  const cudaStream_t st = (cudaStream_t)stream;
  PBF_TRY(sort_clear(plan, scratch, st));
  PBF_TRY(sort_histogram(plan, d_keys_in, scratch, st));
  PBF_TRY(sort_scan(plan, scratch, st));
  PBF_TRY(sort_passes(plan, d_keys_in, d_vals_in, d_keys_out, d_vals_out,
                      scratch, err, st));
  return PBF_OK;
}

int pbf_op_sort_status(const void *d_scratch, uint32_t n, uint32_t key_bits,
                       void *stream) {
  if (!d_scratch) return PBF_ERR_INVALID;
  if (n == 0) return PBF_OK;
  const SortPlan plan = make_sort_plan(n, key_bits);
  uint32_t flag = 0;
  const uint32_t *err = static_cast<const uint32_t *>(d_scratch) + plan.off_counter + 31;
  PBF_TRY(cudaMemcpyAsync(&flag, err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  PBF_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  if (flag) {
    set_error_message("radix sort look-back wait gave up");
    return PBF_ERR_DEVICE;
  }
  return PBF_OK;
}

size_t pbf_op_sort_cells_scratch_bytes(uint32_t n, uint32_t ncells) {
  return make_cell_sort_plan(n, ncells).words * sizeof(uint32_t);
}

int pbf_op_sort_cells(const uint32_t *d_keys, uint32_t n, uint32_t ncells, uint32_t *d_offsets,
                      uint32_t *d_sorted_keys, uint32_t *d_perm, void *d_scratch,
                      size_t scratch_bytes, void *stream) {
  if (ncells == 0 || !d_offsets || !d_scratch) return PBF_ERR_INVALID;
  if (n && (!d_keys || !d_sorted_keys || !d_perm)) return PBF_ERR_INVALID;
  if (n >= (1u << 30)) return PBF_ERR_INVALID;
  const CellSortPlan plan = make_cell_sort_plan(n, ncells);
  if (scratch_bytes < plan.words * sizeof(uint32_t)) return PBF_ERR_INVALID;
  uint32_t *scratch = static_cast<uint32_t *>(d_scratch);
  const cudaStream_t st = (cudaStream_t)stream;
  // the control words hold the error word (ctl[3]); the counts start at zero
  PBF_TRY(cell_sort_clear(plan, scratch, true, st));
  PBF_TRY(cell_sort_count(plan, d_keys, scratch, scratch + plan.off_ctl + 3, st));
  PBF_TRY(cell_sort_finish(plan, d_keys, scratch, d_offsets, d_sorted_keys, d_perm,
                           scratch + plan.off_ctl + 3, st));
  return PBF_OK;
}

int pbf_op_sort_cells_status(const void *d_scratch, uint32_t n, uint32_t ncells, void *stream) {
  if (!d_scratch || ncells == 0) return PBF_ERR_INVALID;
  const CellSortPlan plan = make_cell_sort_plan(n, ncells);
  uint32_t flag = 0;
  const uint32_t *err = static_cast<const uint32_t *>(d_scratch) + plan.off_ctl + 3;
  PBF_TRY(cudaMemcpyAsync(&flag, err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  PBF_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  if (flag) {
    set_error_message(flag & kDevErrKey ? "cell sort: a key not below ncells"
                                        : "cell sort look-back wait gave up");
    return PBF_ERR_DEVICE;
  }
  return PBF_OK;
}

int pbf_op_cell_offsets(const uint32_t *d_sorted_keys, uint32_t n,
                        uint32_t ncells, uint32_t *d_offsets, void *stream) {
  if (!d_offsets || (n && !d_sorted_keys) || ncells == 0) return PBF_ERR_INVALID;
  PBF_TRY(cell_offsets(d_sorted_keys, n, ncells, d_offsets, (cudaStream_t)stream));
  return PBF_OK;
}

int pbf_selftest_bounded_wait(uint32_t spin_limit, uint32_t *device_flag) {
  if (spin_limit == 0 || spin_limit > (1u << 26) || !device_flag) return PBF_ERR_INVALID;
  cudaStream_t st = nullptr;
  uint32_t *buf = nullptr;
  int rc = PBF_OK;
  auto cuda = [&](cudaError_t e, const char *where) {
    if (e != cudaSuccess && rc == PBF_OK) rc = cuda_status(e, where);
    return rc == PBF_OK;
  };
  *device_flag = 0;
  if (cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "selftest") &&
      cuda(cudaMalloc(&buf, kSelftestWords * sizeof(uint32_t)), "selftest") &&
      cuda(cudaMemsetAsync(buf, 0, kSelftestWords * sizeof(uint32_t), st), "selftest") &&
      cuda(wait_selftest(buf, spin_limit, buf + kSelftestWords - 1, st), "selftest") &&
      cuda(cudaMemcpyAsync(device_flag, buf + kSelftestWords - 1, sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, st), "selftest"))
    cuda(cudaStreamSynchronize(st), "selftest");
  if (buf) cudaFree(buf);
  if (st) cudaStreamDestroy(st);
  if (rc != PBF_OK) return rc;
  if (*device_flag) {
    set_error_message("device error flag " + std::to_string(*device_flag));
    return PBF_ERR_DEVICE;
  }
  return PBF_OK;
}

int pbf_op_find_cells(const uint32_t *d_offsets, uint32_t ncells,
                      int32_t *d_first_last, void *stream) {
  if (!d_offsets || !d_first_last) return PBF_ERR_INVALID;
  PBF_TRY(find_cells(d_offsets, ncells, d_first_last, (cudaStream_t)stream));
  return PBF_OK;
}

}  // extern "C"
