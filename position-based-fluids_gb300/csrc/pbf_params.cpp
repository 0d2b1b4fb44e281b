// Parameter defaults, validation and derived solver constants.
//
// Reference: the constants src/main.cpp:149-168 bakes into the OpenCL
// program; the solver settings the kernels hard-code (relaxation 1e4 at
// compute_scaling.cl:16, XSPH c = 0.01 at apply_vorticity_and_viscosity.cl:103,
// gravity -9.81 at predict_positions.cl:8, 4 iterations at
// src/Simulation.cpp:503).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "pbf_host.hpp"

namespace pbf {

namespace {
thread_local std::string g_last_error;
}

void set_error_message(const std::string &msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char *where) {
  if (e == cudaSuccess) return PBF_OK;
  set_error_message(std::string(where) + ": " + cudaGetErrorName(e) + " (" +
                    cudaGetErrorString(e) + ")");
  return e == cudaErrorMemoryAllocation ? PBF_ERR_OOM : PBF_ERR_CUDA;
}

float baked6(double v) {
  // ostream << showpoint at the default precision is printf's "%#g".
  char buf[64];
  std::snprintf(buf, sizeof buf, "%#g", v);
  return std::strtof(buf, nullptr);
}

float params_h(const pbf_params &p) { return (p.x_max - p.x_min) / p.x_n; }

uint64_t grid_cells(const pbf_params &p) {
  return (uint64_t)p.x_n * (uint64_t)p.y_n * (uint64_t)p.z_n;
}

RefConsts make_ref_consts(const pbf_params &p) {
  RefConsts k;
  k.min[0] = baked6(p.x_min);
  k.max[0] = baked6(p.x_max);
  k.min[1] = baked6(p.y_min);
  k.max[1] = baked6(p.y_max);
  k.min[2] = baked6(p.z_min);
  k.max[2] = baked6(p.z_max);
  k.ncell[0] = baked6(p.x_n);
  k.ncell[1] = baked6(p.y_n);
  k.ncell[2] = baked6(p.z_n);
  k.clen[0] = baked6((p.x_max - p.x_min) / p.x_n);
  k.clen[1] = baked6((p.y_max - p.y_min) / p.y_n);
  k.clen[2] = baked6((p.z_max - p.z_min) / p.z_n);
  k.dt = baked6(p.time_step_length);
  k.rest_density = baked6(p.rest_density);
  const float h = params_h(p);
  k.h = baked6(h);
  k.h2 = baked6(std::pow((double)h, 2.0));
  k.poly6 = baked6(315.0f / (64.0f * M_PI * std::pow((double)h, 9.0)));
  k.spiky = baked6(45.0f / (M_PI * std::pow((double)h, 6.0)));
  return k;
}

PaperConsts make_paper_consts(const pbf_params &p, uint32_t n) {
  PaperConsts c;
  const double h = params_h(p);
  c.dt = p.time_step_length;
  c.gy = p.gravity_y;
  c.h = (float)h;
  c.h2 = (float)(h * h);
  c.poly6 = (float)(315.0 / (64.0 * M_PI * std::pow(h, 9)));
  c.spiky = (float)(45.0 / (M_PI * std::pow(h, 6)));
  c.w_self = (float)(315.0 / (64.0 * M_PI * std::pow(h, 3)));
  c.rho0 = p.rest_density;
  c.inv_rho0 = (float)(1.0 / (double)p.rest_density);
  c.relax_eps = p.relax_eps;
  // s_corr is added to lambda (units of area): the paper's dimensionless k
  // is applied in units of h^2.
  c.scorr_k = (float)((double)p.scorr_k * h * h);
  const double dq = (double)p.scorr_dq * h;
  c.inv_scorr_den = (float)(1.0 / (h * h - dq * dq));
  c.scorr_n3 = 3 * p.scorr_n;
  c.xsph_c = p.xsph_c;
  c.vort_eps = p.vort_eps;
  c.n = n;
  // Lists are stored in groups of eight entries.
  c.maxn = p.max_neighbours < 8 ? 8u : (p.max_neighbours / 8u) * 8u;
  return c;
}

SceneDesc make_scene(const pbf_params &p) {
  SceneDesc s;
  std::memset(&s, 0, sizeof s);
  const float mn[3] = {p.x_min, p.y_min, p.z_min};
  const float mx[3] = {p.x_max, p.y_max, p.z_max};
  const float nc[3] = {p.x_n, p.y_n, p.z_n};
  const bool ref = p.mode == PBF_MODE_REF_COMPAT;
  const RefConsts rk = make_ref_consts(p);
  const float h = params_h(p);
  const float margin = p.wall_margin < 0.0f ? 0.25f * h : p.wall_margin;
  for (int a = 0; a < 3; ++a) {
    s.gmin[a] = ref ? rk.min[a] : mn[a];
    s.clen[a] = ref ? rk.clen[a] : (mx[a] - mn[a]) / nc[a];
    s.ncell[a] = (int32_t)nc[a];
    s.lo[a] = mn[a] + margin;
    s.hi[a] = mx[a] - margin;
  }
  s.cell_base = 0;
  s.wave = 0.0f;
  return s;
}

int validate_params(const pbf_params &p, uint32_t n) {
  if (n == 0) {
    set_error_message("no particles");
    return PBF_ERR_INVALID;
  }
  if (p.mode != PBF_MODE_REF_COMPAT && p.mode != PBF_MODE_PAPER) {
    set_error_message("unknown mode");
    return PBF_ERR_INVALID;
  }
  const float nc[3] = {p.x_n, p.y_n, p.z_n};
  const float ext[3] = {p.x_max - p.x_min, p.y_max - p.y_min, p.z_max - p.z_min};
  for (int a = 0; a < 3; ++a) {
    if (!(nc[a] >= 1.0f) || nc[a] != std::floor(nc[a]) || nc[a] > 65536.0f) {
      set_error_message("cell counts must be whole numbers in [1, 65536]");
      return PBF_ERR_INVALID;
    }
    if (!(ext[a] > 0.0f)) {
      set_error_message("empty box");
      return PBF_ERR_INVALID;
    }
  }
  const uint64_t cells = grid_cells(p);
  if (cells > (1ull << 31)) {
    set_error_message("more than 2^31 cells");
    return PBF_ERR_INVALID;
  }
  if (n >= (1u << 30)) {
    set_error_message("more than 2^30 - 1 particles");
    return PBF_ERR_INVALID;
  }
  if (!(p.time_step_length > 0.0f) || !(p.rest_density > 0.0f)) {
    set_error_message("time step and rest density must be positive");
    return PBF_ERR_INVALID;
  }
  if (p.solver_iterations < 1 || p.solver_iterations > 64) {
    set_error_message("solver_iterations must be in [1, 64]");
    return PBF_ERR_INVALID;
  }
  if (p.mode == PBF_MODE_PAPER) {
    const float h = params_h(p);
    for (int a = 0; a < 3; ++a) {
      if (ext[a] / nc[a] < h * (1.0f - 1e-5f)) {
        set_error_message("paper mode needs cells at least h long on every axis");
        return PBF_ERR_INVALID;
      }
    }
    if (p.max_neighbours < 1 || p.max_neighbours > 1024) {
      set_error_message("max_neighbours must be in [1, 1024]");
      return PBF_ERR_INVALID;
    }
    if (!(p.scorr_dq >= 0.0f && p.scorr_dq < 1.0f) || p.scorr_n < 0 || p.scorr_n > 10) {
      set_error_message("scorr_dq must be in [0,1) and scorr_n in [0,10]");
      return PBF_ERR_INVALID;
    }
    const float margin = p.wall_margin < 0.0f ? 0.25f * h : p.wall_margin;
    for (int a = 0; a < 3; ++a)
      if (!(2.0f * margin < ext[a])) {
        set_error_message("wall margin leaves no room in the box");
        return PBF_ERR_INVALID;
      }
  }
  return PBF_OK;
}

}  // namespace pbf

extern "C" {

int pbf_abi_version(void) { return PBF_ABI_VERSION; }

const char *pbf_status_string(int status) {
  switch (status) {
    case PBF_OK: return "ok";
    case PBF_ERR_INVALID: return "invalid argument";
    case PBF_ERR_OOM: return "out of memory";
    case PBF_ERR_CUDA: return "CUDA error";
    case PBF_ERR_DEVICE: return "device error flag set (a bounded wait gave up)";
    case PBF_ERR_IO: return "I/O error";
    case PBF_ERR_BUDGET: return "HBM budget exceeded";
    case PBF_ERR_STATE: return "call out of order";
    case PBF_ERR_NOT_FOUND: return "not found";
    default: return "unknown status";
  }
}

const char *pbf_last_error_message(void) {
  return pbf::g_last_error.c_str();
}

void pbf_params_default(pbf_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->time_step_length = 1.0f / 120.0f;
  p->time_end = 1.0f;
  p->cl_workgroup_1dsize = 0;
  p->x_min = p->y_min = p->z_min = 0.0f;
  p->x_max = p->y_max = p->z_max = 1.0f;
  p->x_n = p->y_n = p->z_n = 10.0f;
  p->rest_density = 8000.0f;
  p->mode = PBF_MODE_PAPER;
  p->solver_iterations = 4;
  p->relax_eps = 600.0f;
  p->scorr_k = 0.1f;
  p->scorr_dq = 0.2f;
  p->scorr_n = 4;
  p->xsph_c = 0.01f;
  p->vort_eps = 0.0005f;
  p->gravity_y = -9.81f;
  p->wall_margin = -1.0f; /* resolved to h/4 */
  p->max_neighbours = 128;
  p->grow_lists = 1;
}

}  // extern "C"

namespace pbf {

void to_pbf_tuning(const GatherTuning &g, const double trial_ms[kGatherKinds], pbf_tuning *out) {
  for (int k = 0; k < kGatherKinds; ++k) {
    out->threads[k] = 64u << g.block[k];
    out->batch[k] = 4u << g.batch[k];
    out->trial_ms[k] = trial_ms ? (float)trial_ms[k] : 0.0f;
  }
  out->fuse_first = g.fuse_first;
  out->staged = g.staged;
  out->radix_sort = g.radix_sort;
  out->masked_build = g.masked_build;
}

int to_gather_tuning(const pbf_tuning &t, GatherTuning *out) {
  GatherTuning g;
  for (int k = 0; k < kGatherKinds; ++k) {
    int bl = -1, nb = -1;
    for (int c = 0; c < kBlockCodes; ++c)
      if (t.threads[k] == (64u << c)) bl = c;
    for (int c = 0; c < kBatchCodes; ++c)
      if (t.batch[k] == (4u << c)) nb = c;
    if (bl < 0 || nb < 0) {
      set_error_message("tuning: threads must be 64, 128 or 256 and batch 4 or 8");
      return PBF_ERR_INVALID;
    }
    g.block[k] = (uint8_t)bl;
    g.batch[k] = (uint8_t)nb;
  }
  if (t.fuse_first > 1) {
    set_error_message("tuning: fuse_first must be 0 or 1");
    return PBF_ERR_INVALID;
  }
  g.fuse_first = (uint8_t)t.fuse_first;
  if (t.staged > 1) {
    set_error_message("tuning: staged must be 0 or 1");
    return PBF_ERR_INVALID;
  }
  g.staged = (uint8_t)t.staged;
  if (t.radix_sort > 1) {
    set_error_message("tuning: radix_sort must be 0 or 1");
    return PBF_ERR_INVALID;
  }
  g.radix_sort = (uint8_t)t.radix_sort;
  if (t.masked_build > 1) {
    set_error_message("tuning: masked_build must be 0 or 1");
    return PBF_ERR_INVALID;
  }
  g.masked_build = (uint8_t)t.masked_build;
  *out = g;
  return PBF_OK;
}

}  // namespace pbf
