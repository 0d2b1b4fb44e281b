// Served scenes: a request loop with continuous batching over one batch
// (include/pbf.h, pbf_server_*).
//
// Each turn of pbf_server_poll retires the requests whose steps are done,
// admits queued requests first-fit in arrival order while the batch's
// preallocated capacities (derived from the HBM budget) hold them, and
// enqueues the next chunk of batched steps without waiting for it.  A chunk
// never runs past the step count of any active request, so a request sees
// exactly its own steps; because a scene's arithmetic in a batch does not
// depend on the other scenes, its result is bitwise the one it has alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <deque>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "pbf_host.hpp"

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

struct Request {
  pbf_params prm{};
  std::vector<pbf_particle> particles;  // released at admission
  uint32_t n = 0, steps = 0, steps_done = 0;
  uint32_t cells = 0;
  int state = PBF_REQ_QUEUED;
  uint32_t scene = 0;                   // batch scene id while active
  std::vector<float> pos, vel;          // final state once done
};

}  // namespace

struct pbf_server {
  pbf_batch *batch = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t chunk_done = nullptr;
  bool in_flight = false;
  uint32_t chunk = 0;
  uint32_t max_chunk = 0;
  uint32_t max_scenes = 0, max_particles = 0, max_cells = 0;
  uint64_t device_bytes = 0;
  uint64_t next_id = 1;
  std::unordered_map<uint64_t, Request> reqs;
  std::deque<uint64_t> queue;    // arrival order
  std::vector<uint64_t> active;  // admission order
  uint32_t active_particles = 0, active_cells = 0;
  pbf_server_stats stats{};
};

namespace {

// Retires finished requests: final state to host, scene out of the batch.
// On an error the failing request and every one after it stay active, so
// the active list always matches the scenes in the batch.
int retire(pbf_server *s, std::vector<uint64_t> &done) {
  std::vector<uint64_t> keep;
  keep.reserve(s->active.size());
  int rc = PBF_OK;
  for (uint64_t id : s->active) {
    Request &r = s->reqs[id];
    if (rc != PBF_OK || r.steps_done < r.steps) {
      keep.push_back(id);
      continue;
    }
    r.pos.assign((size_t)r.n * 4, 0.0f);
    r.vel.assign((size_t)r.n * 4, 0.0f);
    rc = pbf_batch_dump_scene(s->batch, r.scene, r.pos.data(), r.vel.data());
    if (rc == PBF_OK) rc = pbf_batch_remove_scene(s->batch, r.scene);
    if (rc != PBF_OK) {
      keep.push_back(id);
      continue;
    }
    r.state = PBF_REQ_DONE;
    s->active_particles -= r.n;
    s->active_cells -= r.cells;
    s->stats.completed++;
    done.push_back(id);
  }
  s->active.swap(keep);
  return rc;
}

// Admits queued requests, first fit in arrival order.
int admit(pbf_server *s) {
  for (auto it = s->queue.begin(); it != s->queue.end();) {
    Request &r = s->reqs[*it];
    const bool fits = s->active.size() + 1 <= s->max_scenes &&
                      (uint64_t)s->active_particles + r.n <= s->max_particles &&
                      (uint64_t)s->active_cells + r.cells <= s->max_cells;
    if (!fits) {
      ++it;
      continue;
    }
    PBF_TRY_STATUS(pbf_batch_add_scene(s->batch, &r.prm, r.particles.data(), r.n, &r.scene));
    r.state = PBF_REQ_ACTIVE;
    std::vector<pbf_particle>().swap(r.particles);
    s->active.push_back(*it);
    s->active_particles += r.n;
    s->active_cells += r.cells;
    s->stats.admitted++;
    it = s->queue.erase(it);
  }
  return PBF_OK;
}

int launch_chunk(pbf_server *s) {
  if (s->active.empty()) return PBF_OK;
  uint32_t k = s->max_chunk;
  for (uint64_t id : s->active) {
    const Request &r = s->reqs[id];
    k = std::min(k, r.steps - r.steps_done);
  }
  uint32_t per_step = 0;
  PBF_TRY_STATUS(pbf_batch_launches_per_step(s->batch, &per_step));
  PBF_TRY_STATUS(pbf_batch_step(s->batch, k));
  PBF_TRY(cudaEventRecord(s->chunk_done, s->stream));
  s->in_flight = true;
  s->chunk = k;
  s->stats.batch_steps += k;
  s->stats.launches += (uint64_t)k * per_step;
  s->stats.particle_steps += (uint64_t)k * s->active_particles;
  return PBF_OK;
}

}  // namespace

extern "C" {

int pbf_server_create(const pbf_params *solver, uint64_t hbm_budget_bytes, uint32_t max_scenes,
                      float cells_per_particle, uint32_t max_chunk, pbf_server **out) {
  if (!solver || !out || max_scenes == 0 || max_scenes > 65535 || max_chunk == 0 ||
      !(cells_per_particle >= 1.0f) || cells_per_particle > 64.0f)
    return PBF_ERR_INVALID;
  *out = nullptr;
  // Largest particle capacity whose batch fits the budget.
  auto cells_for = [&](uint64_t p) {
    return (uint64_t)((double)p * cells_per_particle + 0.5);
  };
  auto bytes_for = [&](uint64_t p) {
    const uint64_t c = cells_for(p);
    if (c >= (1ull << 31)) return UINT64_MAX;
    return (uint64_t)pbf_batch_device_bytes(solver, max_scenes, (uint32_t)p, (uint32_t)c);
  };
  uint64_t lo = 0, hi = (1ull << 30) - 1;
  while (lo < hi) {
    const uint64_t mid = (lo + hi + 1) / 2;
    if (bytes_for(mid) <= hbm_budget_bytes) lo = mid;
    else hi = mid - 1;
  }
  if (lo < 1024) {
    set_error_message("HBM budget holds no useful batch");
    return PBF_ERR_BUDGET;
  }
  std::unique_ptr<pbf_server> s(new pbf_server());
  s->max_chunk = max_chunk;
  s->max_scenes = max_scenes;
  s->max_particles = (uint32_t)lo;
  s->max_cells = (uint32_t)cells_for(lo);
  s->device_bytes = bytes_for(lo);
  PBF_TRY_STATUS(pbf_batch_create(solver, max_scenes, s->max_particles, s->max_cells, &s->batch));
  void *st = nullptr;
  pbf_batch_get_stream(s->batch, &st);
  s->stream = (cudaStream_t)st;
  const cudaError_t e = cudaEventCreateWithFlags(&s->chunk_done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    pbf_batch_destroy(s->batch);
    return cuda_status(e, "cudaEventCreate");
  }
  *out = s.release();
  return PBF_OK;
}

int pbf_server_submit(pbf_server *s, const pbf_params *scene, const pbf_particle *particles,
                      uint32_t n, uint32_t steps, uint64_t *request_id) {
  if (!s || !scene || !particles || !request_id || n == 0 || steps == 0)
    return PBF_ERR_INVALID;
  Request r;
  uint64_t cells = 0;
  PBF_TRY_STATUS(batch_check_scene(s->batch, *scene, n, nullptr, &cells));
  if (n > s->max_particles || cells > s->max_cells) {
    set_error_message("request exceeds the server's capacity");
    return PBF_ERR_BUDGET;
  }
  r.prm = *scene;
  r.particles.assign(particles, particles + n);
  r.n = n;
  r.steps = steps;
  r.cells = (uint32_t)cells;
  const uint64_t id = s->next_id++;
  s->reqs.emplace(id, std::move(r));
  s->queue.push_back(id);
  s->stats.submitted++;
  *request_id = id;
  return PBF_OK;
}

int pbf_server_poll(pbf_server *s, int wait, uint64_t *completed, uint32_t cap,
                    uint32_t *ncompleted, int *busy) {
  if (!s || !ncompleted || !busy || (cap && !completed)) return PBF_ERR_INVALID;
  *ncompleted = 0;
  if (s->in_flight) {
    if (!wait) {
      const cudaError_t q = cudaEventQuery(s->chunk_done);
      if (q == cudaErrorNotReady) {
        *busy = 1;
        return PBF_OK;
      }
      if (q != cudaSuccess) return cuda_status(q, "cudaEventQuery");
    }
    PBF_TRY_STATUS(pbf_batch_sync(s->batch));
    s->in_flight = false;
    for (uint64_t id : s->active) s->reqs[id].steps_done += s->chunk;
  }
  std::vector<uint64_t> done;
  PBF_TRY_STATUS(retire(s, done));
  PBF_TRY_STATUS(admit(s));
  PBF_TRY_STATUS(launch_chunk(s));
  for (size_t i = 0; i < done.size() && i < cap; ++i) completed[i] = done[i];
  *ncompleted = (uint32_t)done.size();
  *busy = (!s->queue.empty() || !s->active.empty()) ? 1 : 0;
  return PBF_OK;
}

int pbf_server_request_info(const pbf_server *s, uint64_t request_id, int *state, uint32_t *n,
                            uint32_t *steps_done) {
  if (!s) return PBF_ERR_INVALID;
  const auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return PBF_ERR_NOT_FOUND;
  if (state) *state = it->second.state;
  if (n) *n = it->second.n;
  if (steps_done) *steps_done = it->second.steps_done;
  return PBF_OK;
}

int pbf_server_result(pbf_server *s, uint64_t request_id, float *pos4, float *vel4) {
  if (!s || !pos4 || !vel4) return PBF_ERR_INVALID;
  const auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return PBF_ERR_NOT_FOUND;
  Request &r = it->second;
  if (r.state != PBF_REQ_DONE) return PBF_ERR_STATE;
  std::copy(r.pos.begin(), r.pos.end(), pos4);
  std::copy(r.vel.begin(), r.vel.end(), vel4);
  s->reqs.erase(it);
  return PBF_OK;
}

int pbf_server_stats_get(const pbf_server *s, pbf_server_stats *out) {
  if (!s || !out) return PBF_ERR_INVALID;
  *out = s->stats;
  out->queued = (uint32_t)s->queue.size();
  out->active = (uint32_t)s->active.size();
  out->active_particles = s->active_particles;
  out->active_cells = s->active_cells;
  out->max_particles = s->max_particles;
  out->max_cells = s->max_cells;
  out->max_scenes = s->max_scenes;
  out->device_bytes = s->device_bytes;
  return PBF_OK;
}

int pbf_server_destroy(pbf_server *s) {
  if (!s) return PBF_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->chunk_done) cudaEventDestroy(s->chunk_done);
  pbf_batch_destroy(s->batch);
  delete s;
  return PBF_OK;
}

}  // extern "C"
