/*
 * TEST INFRASTRUCTURE (oracle) -- never linked into the product library.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it, and only as the oracle results are compared against or as the timed
 * CPU baseline.
 *
 * CPU restatement of the position-based-fluids step of the reference
 * (MrMagne/position-based-fluids).  See pbf_oracle.h for the C-ABI.
 *
 * Pinning: the float instantiation of the REF_COMPAT step is checked, bit for
 * bit, against the reference's own kernels compiled from their .cl sources
 * (oracle/ref_launch.cpp), on the reference's scenario files.
 */
#include "pbf_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <vector>

namespace {

/* ------------------------------------------------------------------------ */
/* REF_COMPAT constants: src/main.cpp:149-168 streams each value with
 * std::showpoint at the default precision (printf "%#g"), appends "f", and
 * the OpenCL compiler reads the text back as a float literal.             */
float baked(double v) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%#g", v);
  return std::strtof(buf, nullptr);
}

struct RefK {
  float min[3], max[3], ncell[3], clen[3];
  float dt, rd, h, h2, poly6, spiky;
};

RefK derive(const oracle_config &c) {
  RefK k;
  k.min[0] = baked(c.x_min);
  k.max[0] = baked(c.x_max);
  k.min[1] = baked(c.y_min);
  k.max[1] = baked(c.y_max);
  k.min[2] = baked(c.z_min);
  k.max[2] = baked(c.z_max);
  k.ncell[0] = baked(c.x_n);
  k.ncell[1] = baked(c.y_n);
  k.ncell[2] = baked(c.z_n);
  k.clen[0] = baked((c.x_max - c.x_min) / c.x_n);
  k.clen[1] = baked((c.y_max - c.y_min) / c.y_n);
  k.clen[2] = baked((c.z_max - c.z_min) / c.z_n);
  k.dt = baked(c.timestep_length);
  k.rd = baked(c.rest_density);
  const float h = (c.x_max - c.x_min) / c.x_n; /* main.cpp:164 */
  k.h = baked(h);
  k.h2 = baked(std::pow((double)h, 2.0));
  k.poly6 = baked(315.0f / (64.0f * M_PI * std::pow((double)h, 9.0)));
  k.spiky = baked(45.0f / (M_PI * std::pow((double)h, 6.0)));
  return k;
}

bool valid_grid(const oracle_config *c, uint32_t *ncells) {
  if (!c) return false;
  const double nx = c->x_n, ny = c->y_n, nz = c->z_n;
  if (!(nx >= 1 && ny >= 1 && nz >= 1)) return false;
  const double total = nx * ny * nz;
  if (total > 4294967295.0) return false;
  *ncells = (uint32_t)total;
  return true;
}

/* Cell of one axis: (int) truncation of (p - min) / cell_length as in
 * src/kernels/update_cells.cl:10-15, clamped to the grid.  The reference
 * indexes out of bounds for positions outside the grid; inside the grid the
 * clamp never fires. */
template <typename T>
inline int axis_cell(T p, float mn, float cl, float ncell) {
  int c = (int)((p - (T)mn) / (T)cl);
  const int hi = (int)ncell - 1;
  return c < 0 ? 0 : (c > hi ? hi : c);
}

/* Linear cell index in the reference's float arithmetic (NUMBER_OF_CELLS_*
 * are float literals, update_cells.cl:13-15); exact while C < 2^24. */
inline uint32_t linear_cell(int cx, int cy, int cz, const float *ncell) {
  const float f = (float)cx + (float)cy * ncell[0] +
                  (float)cz * ncell[0] * ncell[1];
  return (uint32_t)f;
}

template <typename T>
struct V4 {
  T x, y, z, w;
};

/* ------------------------------------------------------------------------ */
/* REF_COMPAT step, restating src/kernels/*.cl in the order of
 * src/Simulation.cpp:455-576.  Arithmetic follows the kernels' expression
 * trees operator by operator.                                              */
template <typename T>
struct RefCompat {
  RefK k;
  uint32_t n = 0, ncells = 0;
  int threads = 1;
  std::vector<V4<T>> x, v, p, dlt, dv;
  std::vector<T> s;
  std::vector<int> cells, list;

  /* predict_positions.cl:8-9 */
  void predict() {
    const T dt = (T)k.dt;
#pragma omp parallel for num_threads(threads)
    for (long i = 0; i < (long)n; ++i) {
      v[i].x = v[i].x + dt * (T)0.0f;
      v[i].y = v[i].y + dt * (T)(-9.81f);
      v[i].z = v[i].z + dt * (T)0.0f;
      p[i].x = x[i].x + dt * v[i].x;
      p[i].y = x[i].y + dt * v[i].y;
      p[i].z = x[i].z + dt * v[i].z;
    }
  }

  /* init_cells_old.cl + update_cells.cl launched in ascending work-item
   * order: each atomic_xchg pushes a new list head. */
  void build_cells() {
    std::fill(cells.begin(), cells.end(), -1);
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t c = linear_cell(axis_cell(p[i].x, k.min[0], k.clen[0], k.ncell[0]),
                                     axis_cell(p[i].y, k.min[1], k.clen[1], k.ncell[1]),
                                     axis_cell(p[i].z, k.min[2], k.clen[2], k.ncell[2]),
                                     k.ncell);
      list[i] = cells[c];
      cells[c] = (int)i;
    }
  }

  /* Visit the particles of the 27 cells around the *current* cell of i in the
   * kernels' loop order (x outer, z inner), e.g. compute_scaling.cl:20-88. */
  template <typename F>
  void for_neighbours(uint32_t i, F &&f) const {
    const V4<T> &pi = p[i];
    int cc[3];
    cc[0] = (int)((pi.x - (T)k.min[0]) / (T)k.clen[0]);
    cc[1] = (int)((pi.y - (T)k.min[1]) / (T)k.clen[1]);
    cc[2] = (int)((pi.z - (T)k.min[2]) / (T)k.clen[2]);
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          const int n0 = cc[0] + dx, n1 = cc[1] + dy, n2 = cc[2] + dz;
          if (n0 < 0 || (float)n0 >= k.ncell[0] || n1 < 0 ||
              (float)n1 >= k.ncell[1] || n2 < 0 || (float)n2 >= k.ncell[2])
            continue;
          const uint32_t ci = linear_cell(n0, n1, n2, k.ncell);
          for (int j = cells[ci]; j != -1; j = list[j]) {
            if ((int)i != j) f(j);
          }
        }
  }

  /* compute_scaling.cl:11-140 */
  void compute_scaling() {
    const T h = k.h, h2 = k.h2, poly6 = k.poly6, spiky = k.spiky, rd = k.rd;
#pragma omp parallel for num_threads(threads)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      T dens = 0, gsum = 0, gvx = 0, gvy = 0, gvz = 0;
      const V4<T> pi = p[i];
      for_neighbours(i, [&](int j) {
        const T rx = pi.x - p[j].x, ry = pi.y - p[j].y, rz = pi.z - p[j].z;
        const T r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > (T)0 && r2 < h2) {
          const T rl = std::sqrt(r2);
          const T gx = rx / rl * spiky * (h - rl) * (h - rl);
          const T gy = ry / rl * spiky * (h - rl) * (h - rl);
          const T gz = rz / rl * spiky * (h - rl) * (h - rl);
          const T poly = poly6 * (h2 - r2) * (h2 - r2) * (h2 - r2);
          dens += poly;
          gsum += std::sqrt(gx * gx + gy * gy + gz * gz);
          gvx += gx;
          gvy += gy;
          gvz += gz;
        }
      });
      gsum += std::sqrt(gvx * gvx + gvy * gvy + gvz * gvz);
      p[i].w = dens;
      const T c = dens / rd - (T)1.0f;
      s[i] = (T)(-1.0f) * c / (gsum * gsum / (rd * rd) + (T)10000.0f);
    }
  }

  /* compute_delta.cl:13-152 (linked-cell branch; s_corr not applied) */
  void compute_delta(T wave) {
    const T h = k.h, h2 = k.h2, spiky = k.spiky, rd = k.rd;
    const T mnx = k.min[0], mny = k.min[1], mnz = k.min[2];
    const T mxx = k.max[0], mxy = k.max[1], mxz = k.max[2];
#pragma omp parallel for num_threads(threads)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      T sx = 0, sy = 0, sz = 0;
      const V4<T> pi = p[i];
      for_neighbours(i, [&](int j) {
        const T rx = pi.x - p[j].x, ry = pi.y - p[j].y, rz = pi.z - p[j].z;
        const T r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > (T)0 && r2 < h2) {
          const T rl = std::sqrt(r2);
          const T gx = (T)(-1.0f) * rx / rl * spiky * (h - rl) * (h - rl);
          const T gy = (T)(-1.0f) * ry / rl * spiky * (h - rl) * (h - rl);
          const T gz = (T)(-1.0f) * rz / rl * spiky * (h - rl) * (h - rl);
          const T sc = s[i] + s[j];
          sx += sc * gx;
          sy += sc * gy;
          sz += sc * gz;
        }
      });
      T fx = pi.x + sx / rd, fy = pi.y + sy / rd, fz = pi.z + sz / rd;
      if ((fx - h) < (mnx + wave)) fx = mnx + wave + h;
      else if ((fx + h) > mxx) fx = mxx - h;
      if ((fy - h) < mny) fy = mny + h;
      else if ((fy + h) > mxy) fy = mxy - h;
      if ((fz - h) < mnz) fz = mnz + h;
      else if ((fz + h) > mxz) fz = mxz - h;
      dlt[i].x = fx - pi.x;
      dlt[i].y = fy - pi.y;
      dlt[i].z = fz - pi.z;
    }
  }

  /* update_predicted.cl:7 */
  void update_predicted() {
#pragma omp parallel for num_threads(threads)
    for (long i = 0; i < (long)n; ++i) {
      p[i].x = p[i].x + dlt[i].x;
      p[i].y = p[i].y + dlt[i].y;
      p[i].z = p[i].z + dlt[i].z;
    }
  }

  /* update_velocities.cl:8 */
  void update_velocities() {
    const T dt = k.dt;
#pragma omp parallel for num_threads(threads)
    for (long i = 0; i < (long)n; ++i) {
      v[i].x = (p[i].x - x[i].x) / dt;
      v[i].y = (p[i].y - x[i].y) / dt;
      v[i].z = (p[i].z - x[i].z) / dt;
    }
  }

  /* apply_vorticity_and_viscosity.cl:12-104 (XSPH only) */
  void viscosity() {
    const T h2 = k.h2, poly6 = k.poly6;
#pragma omp parallel for num_threads(threads)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      T sx = 0, sy = 0, sz = 0;
      const V4<T> pi = p[i];
      for_neighbours(i, [&](int j) {
        const T rx = pi.x - p[j].x, ry = pi.y - p[j].y, rz = pi.z - p[j].z;
        const T r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > (T)0 && r2 < h2) {
          const T vx = v[j].x - v[i].x, vy = v[j].y - v[i].y,
                  vz = v[j].z - v[i].z;
          const T poly = poly6 * (h2 - r2) * (h2 - r2) * (h2 - r2);
          const T inv = (T)1.0f / p[j].w;
          sx += inv * vx * poly;
          sy += inv * vy * poly;
          sz += inv * vz * poly;
        }
      });
      dv[i].x = (T)0.01f * sx;
      dv[i].y = (T)0.01f * sy;
      dv[i].z = (T)0.01f * sz;
    }
  }

  /* update_positions.cl:9-12 */
  void update_positions() {
#pragma omp parallel for num_threads(threads)
    for (long i = 0; i < (long)n; ++i) {
      x[i].x = p[i].x;
      x[i].y = p[i].y;
      x[i].z = p[i].z;
      v[i].x += dv[i].x;
      v[i].y += dv[i].y;
      v[i].z += dv[i].z;
      x[i].w = std::sqrt(v[i].x * v[i].x + v[i].y * v[i].y + v[i].z * v[i].z);
    }
  }

  void step(T wave) {
    predict();
    build_cells();
    for (int it = 0; it < 4; ++it) { /* Simulation.cpp:503 */
      compute_scaling();
      compute_delta(wave);
      update_predicted();
    }
    update_velocities();
    viscosity();
    update_positions();
  }
};

template <typename T>
int refcompat_steps(const oracle_config *cfg, uint32_t n, T *pos4, T *vel4,
                    uint32_t steps, T wave, int threads, T *pred_out,
                    T *scaling_out) {
  RefCompat<T> s;
  if (!valid_grid(cfg, &s.ncells) || n == 0 || !pos4 || !vel4) return 1;
  s.k = derive(*cfg);
  s.n = n;
  s.threads = threads > 0 ? threads : omp_get_max_threads();
  s.x.assign(n, V4<T>{0, 0, 0, 0});
  s.v = s.x;
  s.p = s.x;
  s.dlt = s.x;
  s.dv = s.x;
  s.s.assign(n, (T)0);
  s.cells.assign(s.ncells, -1);
  s.list.assign(n, -1);
  for (uint32_t i = 0; i < n; ++i) {
    s.x[i] = V4<T>{pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], pos4[4 * i + 3]};
    s.v[i] = V4<T>{vel4[4 * i], vel4[4 * i + 1], vel4[4 * i + 2], vel4[4 * i + 3]};
  }
  for (uint32_t t = 0; t < steps; ++t) s.step(wave);
  for (uint32_t i = 0; i < n; ++i) {
    pos4[4 * i] = s.x[i].x;
    pos4[4 * i + 1] = s.x[i].y;
    pos4[4 * i + 2] = s.x[i].z;
    pos4[4 * i + 3] = s.x[i].w;
    vel4[4 * i] = s.v[i].x;
    vel4[4 * i + 1] = s.v[i].y;
    vel4[4 * i + 2] = s.v[i].z;
    vel4[4 * i + 3] = s.v[i].w;
    if (pred_out) {
      pred_out[4 * i] = s.p[i].x;
      pred_out[4 * i + 1] = s.p[i].y;
      pred_out[4 * i + 2] = s.p[i].z;
      pred_out[4 * i + 3] = s.p[i].w;
    }
    if (scaling_out) scaling_out[i] = s.s[i];
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* PBF_PAPER in double.  Macklin & Mueller, "Position Based Fluids", ACM TOG
 * 32(4), 2013, Algorithm 1, with number densities (unit mass) as in the
 * reference, and these choices where the paper leaves room:
 *   rho_i     = W(0) + sum_j W_poly6(r_ij)                     (self term)
 *   g_ij      = grad_i W_spiky(p_i - p_j) = -S (h-r)^2 r_vec/r
 *   lambda_i  = -(rho_i/rho0 - 1) / ((|sum_j g_ij|^2 + sum_j |g_ij|^2)/rho0^2
 *                                     + eps)
 *   dp_i      = (1/rho0) sum_j (lambda_i + lambda_j + s_corr_ij) g_ij,
 *   s_corr_ij = -k h^2 (W_poly6(r_ij) / W_poly6(dq h))^n
 *               (s_corr is added to lambda, which has units of area; the
 *               paper's dimensionless k is taken in units of h^2.  Read as
 *               k m^2 at h = 0.1 m it outweighs lambda a thousandfold and a
 *               resting block flies apart within 20 steps.)
 *   collision = clamp to [min + margin (+wave on x-min), max - margin]
 *   v_i       = (p_i - x_i) / dt
 *   omega_i   = sum_j (1/rho_j) g_ij x (v_j - v_i)
 *   eta_i     = sum_j (1/rho_j) (|omega_j| - |omega_i|) g_ij,  N = eta/|eta|
 *   v_i      += dt * eps_v (N x omega_i) + c sum_j (1/rho_j)(v_j - v_i) W_ij
 * with N_i = { j != i : 0 < |p_i - p_j| < h } taken from the predicted
 * positions at the start of the step (paper, Algorithm 1 line 6) and every
 * kernel evaluated at the current positions with W = 0 beyond h.  rho_j in
 * the velocity terms is the density of the last lambda pass.            */
template <typename T>
struct Paper {
  oracle_paper_params prm;
  uint32_t n = 0;
  int threads = 1;
  T h, h2, poly6c, spikyc, rho_self, dq2, cl[3];
  std::vector<T> x, v, m, pw, d, p, lam, rho, dpx, vel, om, omn;
  std::vector<uint32_t> nbr_off, nbr;

  void setup() {
    h = (T)prm.h;
    h2 = h * h;
    poly6c = 315.0 / (64.0 * M_PI * std::pow(h, 9));
    spikyc = 45.0 / (M_PI * std::pow(h, 6));
    rho_self = poly6c * h2 * h2 * h2;
    const T dq = (T)prm.scorr_dq * h;
    dq2 = dq * dq;
    for (int a = 0; a < 3; ++a)
      cl[a] = ((T)prm.box_max[a] - (T)prm.box_min[a]) / (T)prm.n_cells[a];
  }

  int cell_axis(T q, int a) const {
    int c = (int)std::floor((q - (T)prm.box_min[a]) / cl[a]);
    return c < 0 ? 0 : (c >= prm.n_cells[a] ? prm.n_cells[a] - 1 : c);
  }

  void build_neighbours() {
    const int nx = prm.n_cells[0], ny = prm.n_cells[1], nz = prm.n_cells[2];
    const size_t C = (size_t)nx * ny * nz;
    std::vector<uint32_t> cnt(C + 1, 0), key(n), order(n);
    for (uint32_t i = 0; i < n; ++i) {
      const int cx = cell_axis(p[3 * i], 0), cy = cell_axis(p[3 * i + 1], 1),
                cz = cell_axis(p[3 * i + 2], 2);
      key[i] = (uint32_t)(cx + (size_t)nx * (cy + (size_t)ny * cz));
      cnt[key[i] + 1]++;
    }
    for (size_t c = 0; c < C; ++c) cnt[c + 1] += cnt[c];
    std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
    for (uint32_t i = 0; i < n; ++i) order[fill[key[i]]++] = i;
    std::vector<std::vector<uint32_t>> lists(n);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      const int cx = cell_axis(p[3 * i], 0), cy = cell_axis(p[3 * i + 1], 1),
                cz = cell_axis(p[3 * i + 2], 2);
      std::vector<uint32_t> &L = lists[i];
      for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            const int ax = cx + dx, ay = cy + dy, az = cz + dz;
            if (ax < 0 || ay < 0 || az < 0 || ax >= nx || ay >= ny || az >= nz)
              continue;
            const size_t c = ax + (size_t)nx * (ay + (size_t)ny * az);
            for (uint32_t q = cnt[c]; q < cnt[c + 1]; ++q) {
              const uint32_t j = order[q];
              if (j == i) continue;
              const T rx = p[3 * i] - p[3 * j], ry = p[3 * i + 1] - p[3 * j + 1],
                           rz = p[3 * i + 2] - p[3 * j + 2];
              const T r2 = rx * rx + ry * ry + rz * rz;
              if (r2 > 0.0 && r2 < h2) L.push_back(j);
            }
          }
      std::sort(L.begin(), L.end());
    }
    nbr_off.assign(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) nbr_off[i + 1] = nbr_off[i] + (uint32_t)lists[i].size();
    nbr.resize(nbr_off[n]);
    for (uint32_t i = 0; i < n; ++i)
      std::copy(lists[i].begin(), lists[i].end(), nbr.begin() + nbr_off[i]);
  }

  /* g_ij and r^2 at the current positions; false if r >= h or r == 0. */
  bool grad(uint32_t i, uint32_t j, T g[3], T *r2o) const {
    const T rx = p[3 * i] - p[3 * j], ry = p[3 * i + 1] - p[3 * j + 1],
                 rz = p[3 * i + 2] - p[3 * j + 2];
    const T r2 = rx * rx + ry * ry + rz * rz;
    *r2o = r2;
    if (!(r2 > 0.0 && r2 < h2)) return false;
    const T r = std::sqrt(r2);
    const T f = -spikyc * (h - r) * (h - r) / r;
    g[0] = f * rx;
    g[1] = f * ry;
    g[2] = f * rz;
    return true;
  }

  void lambda_pass() {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      // Density summed with a compensation term (Fast2Sum: the running sum
      // starts at W(0), the largest term), so that C = rho/rho0 - 1, a small
      // difference of large numbers, keeps its precision.
      T dens = rho_self, dens_lo = 0, G[3] = {0, 0, 0}, S = 0;
      for (uint32_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
        const uint32_t j = nbr[q];
        T g[3], r2;
        if (!grad(i, j, g, &r2)) continue;
        const T t = h2 - r2;
        const T w = poly6c * t * t * t;
        const T sum = dens + w;
        dens_lo += w - (sum - dens);
        dens = sum;
        G[0] += g[0];
        G[1] += g[1];
        G[2] += g[2];
        S += g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
      }
      const T rho0 = (T)prm.rest_density;
      const T C = ((dens - rho0) + dens_lo) / rho0;
      dens += dens_lo;
      const T den = (G[0] * G[0] + G[1] * G[1] + G[2] * G[2] + S) / (rho0 * rho0);
      lam[i] = -C / (den + (T)prm.relax_eps);
      rho[i] = dens;
    }
  }

  void delta_pass(T wave) {
    const T dn = (h2 - dq2);
    const int sn = prm.scorr_n;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      T s[3] = {0, 0, 0};
      for (uint32_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
        const uint32_t j = nbr[q];
        T g[3], r2;
        if (!grad(i, j, g, &r2)) continue;
        const T ratio = std::pow((h2 - r2) / dn, 3.0 * sn);
        const T sc = -(T)prm.scorr_k * h2 * ratio;
        const T w = lam[i] + lam[j] + sc;
        s[0] += w * g[0];
        s[1] += w * g[1];
        s[2] += w * g[2];
      }
      for (int a = 0; a < 3; ++a) {
        const T dnew = d[3 * i + a] + s[a] / (T)prm.rest_density;
        T q = x[3 * i + a] + dnew;
        const T lo = (T)(prm.box_min[a] + prm.wall_margin) + (a == 0 ? (T)wave : (T)0);
        const T hi = (T)(prm.box_max[a] - prm.wall_margin);
        if (q < lo) q = lo;
        else if (q > hi) q = hi;
        dpx[3 * i + a] = q - x[3 * i + a];
      }
    }
    d.swap(dpx);
    for (size_t q = 0; q < (size_t)3 * n; ++q) p[q] = x[q] + d[q];
  }

  void velocity_pass() {
    const T dt = (T)prm.dt;
    for (size_t q = 0; q < (size_t)3 * n; ++q) vel[q] = d[q] / dt;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      T w[3] = {0, 0, 0};
      for (uint32_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
        const uint32_t j = nbr[q];
        T g[3], r2;
        if (!grad(i, j, g, &r2)) continue;
        const T vj = 1.0 / rho[j];
        const T u[3] = {vel[3 * j] - vel[3 * i], vel[3 * j + 1] - vel[3 * i + 1],
                             vel[3 * j + 2] - vel[3 * i + 2]};
        w[0] += vj * (g[1] * u[2] - g[2] * u[1]);
        w[1] += vj * (g[2] * u[0] - g[0] * u[2]);
        w[2] += vj * (g[0] * u[1] - g[1] * u[0]);
      }
      om[3 * i] = w[0];
      om[3 * i + 1] = w[1];
      om[3 * i + 2] = w[2];
      omn[i] = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    }
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (long li = 0; li < (long)n; ++li) {
      const uint32_t i = (uint32_t)li;
      T eta[3] = {0, 0, 0}, xs[3] = {0, 0, 0};
      for (uint32_t q = nbr_off[i]; q < nbr_off[i + 1]; ++q) {
        const uint32_t j = nbr[q];
        T g[3], r2;
        if (!grad(i, j, g, &r2)) continue;
        const T vj = 1.0 / rho[j];
        const T dw = vj * (omn[j] - omn[i]);
        eta[0] += dw * g[0];
        eta[1] += dw * g[1];
        eta[2] += dw * g[2];
        const T t = h2 - r2;
        const T W = poly6c * t * t * t * vj;
        xs[0] += W * (vel[3 * j] - vel[3 * i]);
        xs[1] += W * (vel[3 * j + 1] - vel[3 * i + 1]);
        xs[2] += W * (vel[3 * j + 2] - vel[3 * i + 2]);
      }
      const T el = std::sqrt(eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
      T N[3] = {0, 0, 0};
      if (el > 0.0) {
        N[0] = eta[0] / el;
        N[1] = eta[1] / el;
        N[2] = eta[2] / el;
      }
      const T *o = &om[3 * i];
      const T ve = (T)prm.vort_eps, dt = (T)prm.dt, c = (T)prm.xsph_c;
      const T f[3] = {ve * (N[1] * o[2] - N[2] * o[1]),
                      ve * (N[2] * o[0] - N[0] * o[2]),
                      ve * (N[0] * o[1] - N[1] * o[0])};
      for (int a = 0; a < 3; ++a)
        dpx[3 * i + a] = vel[3 * i + a] + dt * f[a] + c * xs[a];
    }
  }

  void step(T wave) {
    const T dt = (T)prm.dt;
    for (uint32_t i = 0; i < n; ++i) {
      v[3 * i + 1] += dt * (T)prm.gravity_y;
      for (int a = 0; a < 3; ++a) {
        d[3 * i + a] = dt * v[3 * i + a];
        p[3 * i + a] = x[3 * i + a] + d[3 * i + a];
      }
    }
    build_neighbours();
    for (int it = 0; it < prm.iterations; ++it) {
      lambda_pass();
      delta_pass(wave);
    }
    velocity_pass();
    for (uint32_t i = 0; i < n; ++i) {
      T s2 = 0;
      for (int a = 0; a < 3; ++a) {
        x[3 * i + a] = p[3 * i + a];
        v[3 * i + a] = dpx[3 * i + a];
        s2 += v[3 * i + a] * v[3 * i + a];
      }
      pw[i] = std::sqrt(s2);
    }
  }
};

}  // namespace

extern "C" {

int oracle_ref_constants(const oracle_config *cfg, float *out18) {
  if (!cfg || !out18) return 1;
  const RefK k = derive(*cfg);
  const float vals[18] = {k.min[0], k.max[0], k.min[1], k.max[1], k.min[2],
                          k.max[2], k.ncell[0], k.ncell[1], k.ncell[2],
                          k.clen[0], k.clen[1], k.clen[2], k.dt, k.rd, k.h,
                          k.h2, k.poly6, k.spiky};
  for (int i = 0; i < 18; ++i) out18[i] = vals[i];
  return 0;
}

int oracle_cell_hash(const oracle_config *cfg, const float *pred4, uint32_t n,
                     uint32_t *hash_out) {
  uint32_t nc;
  if (!valid_grid(cfg, &nc) || (!pred4 && n) || (!hash_out && n)) return 1;
  const RefK k = derive(*cfg);
  for (uint32_t i = 0; i < n; ++i)
    hash_out[i] = linear_cell(axis_cell(pred4[4 * i], k.min[0], k.clen[0], k.ncell[0]),
                              axis_cell(pred4[4 * i + 1], k.min[1], k.clen[1], k.ncell[1]),
                              axis_cell(pred4[4 * i + 2], k.min[2], k.clen[2], k.ncell[2]),
                              k.ncell);
  return 0;
}

int oracle_sort_cells(const uint32_t *hash, uint32_t n,
                      uint32_t *sorted_hash_out, uint32_t *perm_out) {
  if (n && (!hash || !sorted_hash_out || !perm_out)) return 1;
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(),
                   [&](uint32_t a, uint32_t b) { return hash[a] < hash[b]; });
  for (uint32_t q = 0; q < n; ++q) {
    perm_out[q] = idx[q];
    sorted_hash_out[q] = hash[idx[q]];
  }
  return 0;
}

int oracle_find_cells(const uint32_t *sorted_hash, uint32_t n,
                      uint32_t ncells, int32_t *first_last_out) {
  if (!first_last_out || (n && !sorted_hash)) return 1;
  for (uint32_t c = 0; c < ncells; ++c) {
    first_last_out[2 * c] = -1;
    first_last_out[2 * c + 1] = -1;
  }
  for (uint32_t q = 0; q < n; ++q) {
    const uint32_t c = sorted_hash[q];
    if (c >= ncells) return 2;
    if (q == 0 || sorted_hash[q - 1] != c) first_last_out[2 * c] = (int32_t)q;
    if (q == n - 1 || sorted_hash[q + 1] != c) first_last_out[2 * c + 1] = (int32_t)q;
  }
  return 0;
}

int oracle_refcompat_steps_f32(const oracle_config *cfg, uint32_t n,
                               float *pos4, float *vel4, uint32_t steps,
                               float wave, int threads, float *predicted4_out,
                               float *scaling_out) {
  return refcompat_steps<float>(cfg, n, pos4, vel4, steps, wave, threads,
                                predicted4_out, scaling_out);
}

int oracle_refcompat_steps_f64(const oracle_config *cfg, uint32_t n,
                               double *pos4, double *vel4, uint32_t steps,
                               double wave, int threads) {
  return refcompat_steps<double>(cfg, n, pos4, vel4, steps, wave, threads,
                                 nullptr, nullptr);
}

}  // extern "C"

namespace {

template <typename T>
int paper_steps(const oracle_paper_params *prm, uint32_t n, double *pos4,
                double *vel4, uint32_t steps, double wave, int threads,
                double *density_out, double *lambda_out,
                uint32_t *nbr_count_out) {
  if (!prm || !pos4 || !vel4 || n == 0) return 1;
  for (int a = 0; a < 3; ++a)
    if (prm->n_cells[a] < 1 || !(prm->box_max[a] > prm->box_min[a])) return 1;
  if (!(prm->h > 0) || !(prm->dt > 0) || !(prm->rest_density > 0) ||
      prm->iterations < 0)
    return 1;
  Paper<T> s;
  s.prm = *prm;
  s.n = n;
  s.threads = threads > 0 ? threads : omp_get_max_threads();
  s.setup();
  s.x.assign(3 * (size_t)n, 0);
  s.v = s.x;
  s.d = s.x;
  s.p = s.x;
  s.dpx = s.x;
  s.vel = s.x;
  s.om = s.x;
  s.m.assign(n, 0);
  s.pw.assign(n, 0);
  s.lam.assign(n, 0);
  s.rho.assign(n, s.rho_self);
  s.omn.assign(n, 0);
  for (uint32_t i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a) {
      s.x[3 * i + a] = pos4[4 * i + a];
      s.v[3 * i + a] = vel4[4 * i + a];
    }
    s.pw[i] = pos4[4 * i + 3];
    s.m[i] = vel4[4 * i + 3];
  }
  for (uint32_t t = 0; t < steps; ++t) s.step((T)wave);
  for (uint32_t i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a) {
      pos4[4 * i + a] = s.x[3 * i + a];
      vel4[4 * i + a] = s.v[3 * i + a];
    }
    pos4[4 * i + 3] = s.pw[i];
    vel4[4 * i + 3] = s.m[i];
    if (density_out) density_out[i] = s.rho[i];
    if (lambda_out) lambda_out[i] = s.lam[i];
    if (nbr_count_out) nbr_count_out[i] = s.nbr_off[i + 1] - s.nbr_off[i];
  }
  return 0;
}

}  // namespace

extern "C" {

int oracle_paper_steps_f64(const oracle_paper_params *prm, uint32_t n,
                           double *pos4, double *vel4, uint32_t steps,
                           double wave, int threads, double *density_out,
                           double *lambda_out, uint32_t *nbr_count_out) {
  return paper_steps<double>(prm, n, pos4, vel4, steps, wave, threads,
                             density_out, lambda_out, nbr_count_out);
}

int oracle_paper_steps_f32(const oracle_paper_params *prm, uint32_t n,
                           double *pos4, double *vel4, uint32_t steps,
                           double wave, int threads, double *density_out,
                           double *lambda_out, uint32_t *nbr_count_out) {
  return paper_steps<float>(prm, n, pos4, vel4, steps, wave, threads,
                            density_out, lambda_out, nbr_count_out);
}

}  // extern "C"
