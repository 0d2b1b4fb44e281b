// Batched scenes: many independent PBF scenes in one set of device arrays,
// advanced by one launch per kernel (include/pbf.h, pbf_batch_*).
//
// Layout: scenes occupy consecutive particle ranges [p_begin, p_end) of the
// sorted state and consecutive key ranges [cell_base, cell_base + cells).
// Because every key of scene s is below every key of scene s+1, the stable
// sort keeps each scene's particles inside its range, in the order the scene
// alone would have, and every kernel works on one particle per thread with
// neighbours from the particle's own scene.  A scene therefore runs exactly
// the operations it runs alone, whatever else is in the batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "pbf_host.hpp"
#include "pbf_tune.hpp"

using namespace pbf;

namespace {

#define PBF_TRY(expr)                                      \
  do {                                                     \
    const cudaError_t e_ = (expr);                         \
    if (e_ != cudaSuccess) return cuda_status(e_, #expr);  \
  } while (0)

#define PBF_TRY_STATUS(expr)     \
  do {                           \
    const int s_ = (expr);       \
    if (s_ != PBF_OK) return s_; \
  } while (0)

struct SceneRec {
  uint32_t id;
  uint32_t n;
  uint32_t cells;
  SceneDesc desc;  // box, grid and clamp bounds; bases filled at layout time
};

size_t bytes_per_particle(uint32_t maxn) {
  return 10 * sizeof(float4)                  // X V X2 V2 P Q D U W S
         + 6 * sizeof(uint32_t)               // ID ID2 keys skeys perm nbr_cnt
         + sizeof(float)                      // R
         + (size_t)paper_list_words(maxn) * 16  // lists
         + sizeof(uint16_t)                   // sid
         + 2 * sizeof(float4);                // io staging
}

}  // namespace

struct pbf_batch {
  pbf_params solver{};
  PaperConsts pc{};
  uint32_t max_scenes = 0, max_particles = 0, max_cells = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  DeviceState d;
  std::vector<void *> allocations;
  std::vector<SceneRec> scenes;
  uint32_t next_id = 0;
  uint32_t n_total = 0, cells_total = 0;
  SortPlan plan;
  CellSortPlan cplan_cap, cplan;  // counting sort: layout at capacity, sizes of the layout
  bool dirty = true;
  // a step (or the tuner's trial steps) ran on the current layout, so the
  // neighbour lists and counts belong to it
  bool stepped_on_layout = false;
  cudaGraphExec_t graph = nullptr;
  bool graph_stale = false;
  std::vector<SceneDesc> table;
};

namespace {

template <typename T>
int balloc(pbf_batch *b, T **p, size_t count) {
  void *q = nullptr;
  const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count * sizeof(T), 16));
  if (e != cudaSuccess) return cuda_status(e, "cudaMalloc");
  b->allocations.push_back(q);
  *p = static_cast<T *>(q);
  return PBF_OK;
}

void release(pbf_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  for (void *p : b->allocations) cudaFree(p);
  b->allocations.clear();
  if (b->stream) cudaStreamDestroy(b->stream);
  b->stream = nullptr;
}

int find_scene(const pbf_batch *b, uint32_t id) {
  for (size_t i = 0; i < b->scenes.size(); ++i)
    if (b->scenes[i].id == id) return (int)i;
  return -1;
}

// Recomputes bases, uploads the scene table and scene ids.
int apply_layout(pbf_batch *b) {
  DeviceState &d = b->d;
  b->table.resize(b->scenes.size());
  uint32_t p = 0, c = 0, blocks = 0;
  for (size_t i = 0; i < b->scenes.size(); ++i) {
    SceneRec &s = b->scenes[i];
    s.desc.p_begin = p;
    s.desc.p_end = p + s.n;
    s.desc.cell_base = c;
    s.desc.block_base = blocks;
    b->table[i] = s.desc;
    p += s.n;
    c += s.cells;
    blocks += scene_blocks(s.desc);
  }
  b->n_total = p;
  b->cells_total = c;
  d.blk_total = blocks;
  b->pc.n = p;
  b->plan = make_sort_plan(p, bits_for(std::max<uint32_t>(c, 1)));
  b->cplan = resize_cell_sort_plan(b->cplan_cap, p, c);
  if (!b->scenes.empty()) {
    PBF_TRY(cudaMemcpyAsync(d.scenes, b->table.data(), b->table.size() * sizeof(SceneDesc),
                            cudaMemcpyHostToDevice, b->stream));
    PBF_TRY(scene_ids(d.scenes, (uint32_t)b->scenes.size(), p, d.sid, b->stream));
  }
  b->graph_stale = true;  // same kernels, new sizes: updated in place at the next step
  b->dirty = false;
  b->stepped_on_layout = false;
  return PBF_OK;
}

int launch_batch_step(pbf_batch *b) {
  DeviceState &d = b->d;
  const cudaStream_t st = b->stream;
  const uint32_t n = b->n_total;
  const PaperConsts &pc = b->pc;
  if (!d.tune.radix_sort) {
    PBF_TRY(cell_sort_clear(b->cplan, d.cell_scratch, false, st));
    PBF_TRY(paper_predict_count(d.X, d.V, n, pc, d.scenes, d.sid, d.keys, b->cplan,
                                d.cell_scratch, st));
    PBF_TRY(cell_sort_finish(b->cplan, d.keys, d.cell_scratch, d.offsets, d.skeys, d.perm, d.err,
                             st));
  } else {
    PBF_TRY(sort_clear(b->plan, d.sort_scratch, st));
    PBF_TRY(paper_predict_hash(d.X, d.V, n, pc, d.scenes, d.sid, d.keys, b->plan,
                               d.sort_scratch, st));
    PBF_TRY(sort_scan(b->plan, d.sort_scratch, st));
    PBF_TRY(sort_passes(b->plan, d.keys, nullptr, d.skeys, d.perm, d.sort_scratch, d.err, st));
    PBF_TRY(cell_offsets_runs(d.skeys, n, b->cells_total, d.offsets, d.runs, d.runs_count, st));
  }
  PBF_TRY(paper_reorder(d.perm, d.X, d.V, d.ID, n, pc, d.X2, d.V2, d.ID2, d.P, d.D, st));
  const uint32_t iters = b->solver.solver_iterations;
  if (d.tune.staged) {
    PBF_TRY(tile_plan(d, pc, d.sid, (uint32_t)b->scenes.size(), st));
    for (uint32_t it = 0; it < iters; ++it) {
      if (it == 0) PBF_TRY(tile_nbr_build(d, pc, d.sid, (uint32_t)b->scenes.size(), st));
      PBF_TRY(tile_lambda(d, pc, d.sid, (uint32_t)b->scenes.size(), st));
      PBF_TRY(tile_delta(d, pc, d.sid, (uint32_t)b->scenes.size(), it + 1 == iters, st));
    }
    PBF_TRY(tile_vorticity(d, pc, d.sid, (uint32_t)b->scenes.size(), st));
    PBF_TRY(tile_xsph_commit(d, pc, d.sid, (uint32_t)b->scenes.size(), st));
    return PBF_OK;
  }
  for (uint32_t it = 0; it < iters; ++it) {
    if (it == 0 && d.tune.fuse_first) {
      PBF_TRY(paper_nbr_lambda(d, pc, d.sid, st));
    } else {
      if (it == 0) PBF_TRY(paper_nbr_build(d, pc, d.sid, st));
      PBF_TRY(paper_lambda(d, pc, d.sid, st));
    }
    PBF_TRY(paper_delta(d, pc, d.sid, it + 1 == iters, st));
  }
  PBF_TRY(paper_vorticity(d, pc, d.sid, st));
  PBF_TRY(paper_xsph_commit(d, pc, d.sid, st));
  return PBF_OK;
}

}  // namespace

namespace pbf {

int batch_check_scene(const pbf_batch *b, const pbf_params &scene, uint32_t n,
                      pbf_params *merged_out, uint64_t *cells_out) {
  // The batch's solver settings with this scene's box, grid and walls.
  pbf_params merged = b->solver;
  merged.x_min = scene.x_min; merged.x_max = scene.x_max;
  merged.y_min = scene.y_min; merged.y_max = scene.y_max;
  merged.z_min = scene.z_min; merged.z_max = scene.z_max;
  merged.x_n = scene.x_n; merged.y_n = scene.y_n; merged.z_n = scene.z_n;
  merged.wall_margin = scene.wall_margin;
  {
    const int v = validate_params(merged, n);
    if (v != PBF_OK) return v;
  }
  const float h = params_h(b->solver);
  const float ext[3] = {merged.x_max - merged.x_min, merged.y_max - merged.y_min,
                        merged.z_max - merged.z_min};
  const float nc[3] = {merged.x_n, merged.y_n, merged.z_n};
  for (int a = 0; a < 3; ++a)
    if (ext[a] / nc[a] < h * (1.0f - 1e-5f)) {
      set_error_message("scene cells must be at least the batch's h long");
      return PBF_ERR_INVALID;
    }
  // Clamp bounds from this scene's box; wall margin default from the batch h.
  merged.wall_margin = scene.wall_margin < 0.0f ? 0.25f * h : scene.wall_margin;
  if (merged_out) *merged_out = merged;
  if (cells_out) *cells_out = grid_cells(merged);
  return PBF_OK;
}

void batch_capacity(const pbf_batch *b, uint32_t *scenes, uint32_t *particles,
                    uint32_t *cells) {
  *scenes = b->max_scenes;
  *particles = b->max_particles;
  *cells = b->max_cells;
}

}  // namespace pbf

extern "C" {

size_t pbf_batch_device_bytes(const pbf_params *solver, uint32_t max_scenes,
                              uint32_t max_particles, uint32_t max_cells) {
  if (!solver) return 0;
  const PaperConsts pc = make_paper_consts(*solver, max_particles);
  return (size_t)max_particles * bytes_per_particle(pc.maxn) +
         ((size_t)max_cells + 1) * sizeof(uint32_t) +
         (size_t)max_cells * sizeof(uint32_t) + 3 * sizeof(uint32_t) +  // cell-block list
         (size_t)offset_runs_capacity(max_cells) * sizeof(uint4) + sizeof(uint32_t) +
         sort_words_max(max_particles) * sizeof(uint32_t) +
         make_cell_sort_plan(max_particles, max_cells).words * sizeof(uint32_t) +
         (size_t)max_scenes * sizeof(SceneDesc) + 64;
}

int pbf_batch_create(const pbf_params *solver, uint32_t max_scenes, uint32_t max_particles,
                     uint32_t max_cells, pbf_batch **out) {
  if (!solver || !out) return PBF_ERR_INVALID;
  *out = nullptr;
  if (solver->mode != PBF_MODE_PAPER) {
    set_error_message("batches run the paper equations");
    return PBF_ERR_INVALID;
  }
  if (max_scenes == 0 || max_scenes > 65535 || max_particles == 0 ||
      max_particles >= (1u << 30) || max_cells == 0 || max_cells > (1u << 31)) {
    set_error_message("batch capacities out of range");
    return PBF_ERR_INVALID;
  }
  {
    const int v = validate_params(*solver, 1);
    if (v != PBF_OK) return v;
  }
  std::unique_ptr<pbf_batch> b(new pbf_batch());
  b->solver = *solver;
  b->pc = make_paper_consts(*solver, 0);
  b->max_scenes = max_scenes;
  b->max_particles = max_particles;
  b->max_cells = max_cells;
  cudaError_t e = cudaGetDevice(&b->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamCreate");
  DeviceState &d = b->d;
  const size_t M = max_particles;
  int rc = PBF_OK;
  auto A = [&](auto **p, size_t count) {
    if (rc == PBF_OK) rc = balloc(b.get(), p, count);
  };
  A(&d.X, M); A(&d.V, M); A(&d.X2, M); A(&d.V2, M); A(&d.P, M); A(&d.Q, M);
  A(&d.D, M); A(&d.U, M); A(&d.W, M); A(&d.S, M);
  A(&d.ID, M); A(&d.ID2, M); A(&d.keys, M); A(&d.skeys, M); A(&d.perm, M);
  A(&d.nbr_cnt, M); A(&d.R, M); A(&d.sid, M);
  A(&d.nbr, (size_t)paper_list_words(b->pc.maxn) * M);
  // every cell block holds at least one cell
  d.blk_cap = max_cells;
  A(&d.blk_list, d.blk_cap);
  A(&d.blk_count, 3);
  A(&d.io_pos, M); A(&d.io_vel, M);
  A(&d.offsets, (size_t)max_cells + 1);
  A(&d.runs, offset_runs_capacity(max_cells));
  A(&d.runs_count, 1);
  A(&d.sort_scratch, sort_words_max(max_particles));
  b->cplan_cap = make_cell_sort_plan(max_particles, max_cells);
  b->cplan = resize_cell_sort_plan(b->cplan_cap, 0, 0);
  A(&d.cell_scratch, b->cplan_cap.words);
  A(&d.scenes, max_scenes);
  A(&d.err, 1);
  if (rc == PBF_OK) {
    const cudaError_t te = tile_init();
    if (te != cudaSuccess) rc = cuda_status(te, "tile_init");
  }
  if (rc != PBF_OK) {
    release(b.get());
    return rc;
  }
  e = cudaMemsetAsync(d.err, 0, sizeof(uint32_t), b->stream);
  if (e == cudaSuccess) e = cell_sort_clear(b->cplan_cap, d.cell_scratch, true, b->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(d.offsets, 0, ((size_t)max_cells + 1) * sizeof(uint32_t), b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    release(b.get());
    return cuda_status(e, "pbf_batch_create");
  }
  *out = b.release();
  return PBF_OK;
}


int pbf_batch_add_scene(pbf_batch *b, const pbf_params *scene, const pbf_particle *particles,
                        uint32_t n, uint32_t *scene_id) {
  if (!b || !scene || !particles || !scene_id || n == 0) return PBF_ERR_INVALID;
  pbf_params merged;
  uint64_t cells = 0;
  PBF_TRY_STATUS(batch_check_scene(b, *scene, n, &merged, &cells));
  if (b->scenes.size() + 1 > b->max_scenes || (uint64_t)b->n_total + n > b->max_particles ||
      (uint64_t)b->cells_total + cells > b->max_cells) {
    set_error_message("batch capacity exceeded");
    return PBF_ERR_BUDGET;
  }
  SceneRec rec;
  rec.id = b->next_id++;
  rec.n = n;
  rec.cells = (uint32_t)cells;
  rec.desc = make_scene(merged);
  const uint32_t p0 = b->n_total;
  std::vector<float4> pos(n), vel(n);
  for (uint32_t i = 0; i < n; ++i) {
    const pbf_particle &q = particles[i];
    pos[i] = make_float4(q.x[0], q.x[1], q.x[2], 0.0f);
    vel[i] = make_float4(q.v[0], q.v[1], q.v[2], q.m);
  }
  PBF_TRY(cudaMemcpyAsync(b->d.X + p0, pos.data(), n * sizeof(float4), cudaMemcpyHostToDevice,
                          b->stream));
  PBF_TRY(cudaMemcpyAsync(b->d.V + p0, vel.data(), n * sizeof(float4), cudaMemcpyHostToDevice,
                          b->stream));
  PBF_TRY(iota_range(b->d.ID + p0, n, b->stream));
  PBF_TRY(cudaStreamSynchronize(b->stream));  // host arrays go out of scope
  b->scenes.push_back(rec);
  b->n_total += n;
  b->cells_total += rec.cells;
  b->dirty = true;
  *scene_id = rec.id;
  return PBF_OK;
}

int pbf_batch_remove_scene(pbf_batch *b, uint32_t scene_id) {
  if (!b) return PBF_ERR_INVALID;
  const int i = find_scene(b, scene_id);
  if (i < 0) return PBF_ERR_NOT_FOUND;
  if (b->dirty) PBF_TRY_STATUS(apply_layout(b));
  const SceneRec rec = b->scenes[i];
  const uint32_t pb = rec.desc.p_begin, pe = rec.desc.p_end;
  const uint32_t tail = b->n_total - pe;
  if (tail) {
    // Move the later scenes down through the scratch arrays (the ranges may
    // overlap).
    DeviceState &d = b->d;
    const cudaStream_t st = b->stream;
    PBF_TRY(cudaMemcpyAsync(d.X2, d.X + pe, tail * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    PBF_TRY(cudaMemcpyAsync(d.V2, d.V + pe, tail * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    PBF_TRY(cudaMemcpyAsync(d.ID2, d.ID + pe, tail * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    PBF_TRY(cudaMemcpyAsync(d.X + pb, d.X2, tail * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    PBF_TRY(cudaMemcpyAsync(d.V + pb, d.V2, tail * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    PBF_TRY(cudaMemcpyAsync(d.ID + pb, d.ID2, tail * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  }
  b->scenes.erase(b->scenes.begin() + i);
  b->n_total -= rec.n;
  b->cells_total -= rec.cells;
  b->dirty = true;
  return PBF_OK;
}

int pbf_batch_step(pbf_batch *b, uint32_t nsteps) {
  if (!b) return PBF_ERR_INVALID;
  if (b->dirty) PBF_TRY_STATUS(apply_layout(b));
  if (b->n_total == 0) return PBF_OK;
  if (!b->graph || b->graph_stale) {
    cudaGraph_t g = nullptr;
    PBF_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = launch_batch_step(b);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != PBF_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
    // A layout change keeps the kernels and only changes their arguments and
    // grid sizes, so the executable graph is usually updated in place; a
    // different topology (another number of radix passes) re-instantiates.
    bool updated = false;
    if (b->graph) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(b->graph, g, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
      }
    }
    cudaError_t ie = cudaSuccess;
    if (!updated) ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      b->graph = nullptr;
      return cuda_status(ie, "cudaGraphInstantiate");
    }
    b->graph_stale = false;
  }
  for (uint32_t k = 0; k < nsteps; ++k) PBF_TRY(cudaGraphLaunch(b->graph, b->stream));
  if (nsteps > 0) b->stepped_on_layout = true;
  return PBF_OK;
}

int pbf_batch_sync(pbf_batch *b) {
  if (!b) return PBF_ERR_INVALID;
  uint32_t flag = 0;
  PBF_TRY(cudaMemcpyAsync(&flag, b->d.err, sizeof flag, cudaMemcpyDeviceToHost, b->stream));
  PBF_TRY(cudaStreamSynchronize(b->stream));
  if (flag) {
    PBF_TRY(cudaMemsetAsync(b->d.err, 0, sizeof(uint32_t), b->stream));
    PBF_TRY(cudaStreamSynchronize(b->stream));
    set_error_message("device error flag " + std::to_string(flag));
    return PBF_ERR_DEVICE;
  }
  return PBF_OK;
}

int pbf_batch_dump_scene(pbf_batch *b, uint32_t scene_id, float *pos4, float *vel4) {
  if (!b || !pos4 || !vel4) return PBF_ERR_INVALID;
  const int i = find_scene(b, scene_id);
  if (i < 0) return PBF_ERR_NOT_FOUND;
  if (b->dirty) PBF_TRY_STATUS(apply_layout(b));
  const SceneRec &s = b->scenes[i];
  const uint32_t pb = s.desc.p_begin;
  DeviceState &d = b->d;
  PBF_TRY(gather_to_input_order(d.X + pb, d.V + pb, d.ID + pb, s.n, d.io_pos, d.io_vel,
                                b->stream));
  PBF_TRY(cudaMemcpyAsync(pos4, d.io_pos, s.n * sizeof(float4), cudaMemcpyDeviceToHost,
                          b->stream));
  PBF_TRY(cudaMemcpyAsync(vel4, d.io_vel, s.n * sizeof(float4), cudaMemcpyDeviceToHost,
                          b->stream));
  return pbf_batch_sync(b);
}

int pbf_batch_set_wave(pbf_batch *b, uint32_t scene_id, float value) {
  if (!b) return PBF_ERR_INVALID;
  const int i = find_scene(b, scene_id);
  if (i < 0) return PBF_ERR_NOT_FOUND;
  b->scenes[i].desc.wave = value;
  if (!b->dirty) {
    b->table[i].wave = value;
    PBF_TRY(cudaMemcpyAsync(b->d.scenes + i, &b->table[i], sizeof(SceneDesc),
                            cudaMemcpyHostToDevice, b->stream));
    PBF_TRY(cudaStreamSynchronize(b->stream));
  }
  return PBF_OK;
}

int pbf_batch_info(const pbf_batch *b, uint32_t *scenes, uint32_t *particles, uint32_t *cells) {
  if (!b) return PBF_ERR_INVALID;
  if (scenes) *scenes = (uint32_t)b->scenes.size();
  if (particles) *particles = b->n_total;
  if (cells) *cells = b->cells_total;
  return PBF_OK;
}

int pbf_batch_get_stream(const pbf_batch *b, void **stream) {
  if (!b || !stream) return PBF_ERR_INVALID;
  *stream = (void *)b->stream;
  return PBF_OK;
}

int pbf_batch_launches_per_step(const pbf_batch *b, uint32_t *launches) {
  if (!b || !launches) return PBF_ERR_INVALID;
  const SortPlan plan = make_sort_plan(std::max<uint32_t>(b->n_total, 1),
                                       bits_for(std::max<uint32_t>(b->cells_total, 1)));
  // predict + hash, the sort (counting: 4 launches; radix: scan, digit
  // passes, two for the offsets), reorder, the solver, the velocity passes
  const uint32_t sort = b->d.tune.radix_sort ? 1u + plan.passes + 2u : cell_sort_launches();
  *launches = 1u + sort + 1u + paper_first_launches(b->d) +
              2u * b->solver.solver_iterations - 1u + 2u;
  return PBF_OK;
}

int pbf_batch_neighbour_stats(pbf_batch *b, uint32_t *max_count, uint32_t *overflow) {
  if (!b || !max_count || !overflow) return PBF_ERR_INVALID;
  // the lists belong to the current layout only after a step ran on it
  if (b->dirty || !b->stepped_on_layout) return PBF_ERR_STATE;
  std::vector<uint32_t> cnt(b->n_total);
  if (b->n_total) {
    PBF_TRY(cudaMemcpyAsync(cnt.data(), b->d.nbr_cnt, (size_t)b->n_total * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, b->stream));
    PBF_TRY(cudaStreamSynchronize(b->stream));
  }
  uint32_t mx = 0, over = 0;
  for (uint32_t c : cnt) {
    mx = c > mx ? c : mx;
    over += c > b->pc.maxn ? 1u : 0u;
  }
  *max_count = mx;
  *overflow = over;
  return PBF_OK;
}

int pbf_batch_autotune(pbf_batch *b, uint32_t trial_steps, pbf_tuning *out) {
  if (!b || trial_steps < 1 || trial_steps > 32) return PBF_ERR_INVALID;
  if (b->dirty) PBF_TRY_STATUS(apply_layout(b));
  double ms[kGatherKinds] = {0, 0, 0, 0, 0, 0};
  if (b->n_total > 0) {
    PBF_TRY_STATUS(paper_autotune(b->d, b->n_total, b->stream, trial_steps,
                                  [&]() { return launch_batch_step(b); }, ms));
    b->stepped_on_layout = true;  // the trial steps built lists on this layout
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    PBF_TRY_STATUS(pbf_batch_sync(b));
  }
  if (out) to_pbf_tuning(b->d.tune, ms, out);
  return PBF_OK;
}

int pbf_batch_get_tuning(const pbf_batch *b, pbf_tuning *out) {
  if (!b || !out) return PBF_ERR_INVALID;
  to_pbf_tuning(b->d.tune, nullptr, out);
  return PBF_OK;
}

int pbf_batch_set_tuning(pbf_batch *b, const pbf_tuning *t) {
  if (!b || !t) return PBF_ERR_INVALID;
  PBF_TRY_STATUS(to_gather_tuning(*t, &b->d.tune));
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  return PBF_OK;
}

int pbf_batch_render_scene(pbf_batch *b, uint32_t scene_id, const pbf_camera *cam,
                           uint32_t width, uint32_t height, uint8_t *rgb) {
  if (!b || !cam || !rgb) return PBF_ERR_INVALID;
  const int i = find_scene(b, scene_id);
  if (i < 0) return PBF_ERR_NOT_FOUND;
  if (b->dirty) PBF_TRY_STATUS(apply_layout(b));
  const SceneRec &s = b->scenes[i];
  const uint32_t pb = s.desc.p_begin;
  pbf_params box = b->solver;
  box.x_min = s.desc.gmin[0]; box.y_min = s.desc.gmin[1]; box.z_min = s.desc.gmin[2];
  box.x_max = s.desc.gmin[0] + s.desc.clen[0] * (float)s.desc.ncell[0];
  box.y_max = s.desc.gmin[1] + s.desc.clen[1] * (float)s.desc.ncell[1];
  box.z_max = s.desc.gmin[2] + s.desc.clen[2] * (float)s.desc.ncell[2];
  return render_particles(b->d.X + pb, b->d.ID + pb, s.n, box, *cam, width, height, rgb,
                          b->stream);
}

int pbf_batch_destroy(pbf_batch *b) {
  if (!b) return PBF_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  release(b);
  delete b;
  return PBF_OK;
}

}  // extern "C"
