// C++ host interface over the C-ABI; see Simulation.hpp.
#include "Simulation.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <numeric>
#include <thread>

namespace pbf {

void check(int status, const char *what) {
  if (status == PBF_OK) return;
  std::string msg = std::string(what) + ": " + pbf_status_string(status);
  const char *detail = pbf_last_error_message();
  if (detail && *detail) msg += std::string(" (") + detail + ")";
  throw std::runtime_error(msg);
}

ConfigParameters ConfigReader::read(const std::string &filename) const {
  ConfigParameters p;
  pbf_params_default(&p);
  check(pbf_read_config(filename.c_str(), &p), "ConfigReader::read");
  return p;
}

std::vector<Particle> PartReader::read(const std::string &filename) const {
  pbf_particle *buf = nullptr;
  uint32_t n = 0;
  check(pbf_read_particles(filename.c_str(), &buf, &n), "PartReader::read");
  std::vector<Particle> out(buf, buf + n);
  pbf_free(buf);
  return out;
}

std::string DataLoader::path(const char *kind, const std::string &name) const {
  char buf[4096];
  check(pbf_data_path(root_.c_str(), kind, name.c_str(), buf, sizeof buf),
        "DataLoader");
  return buf;
}
std::string DataLoader::getPathForScenario(const std::string &s) const { return path("scenario", s); }
std::string DataLoader::getPathForKernel(const std::string &s) const { return path("kernel", s); }
std::string DataLoader::getPathForShader(const std::string &s) const { return path("shader", s); }
std::string DataLoader::getPathForTexture(const std::string &s) const { return path("texture", s); }

Simulation::Simulation(const ConfigParameters &parameters,
                       const std::vector<Particle> &particles)
    : params_(parameters), n_((uint32_t)particles.size()) {
  check(pbf_create(&params_, particles.data(), n_, &sim_), "Simulation");
}

Simulation::~Simulation() { pbf_destroy(sim_); }

void Simulation::init() { check(pbf_init(sim_), "Simulation::init"); }

void Simulation::initCells() {
  check(pbf_init_cells(sim_), "Simulation::initCells");
}

void Simulation::step() {
  // The reference blocks on the queue once per step (Simulation.cpp:573).
  check(pbf_step(sim_, 1), "Simulation::step");
  check(pbf_sync(sim_), "Simulation::step");
}

void Simulation::dumpData(Float4 *&positions, Float4 *&velocities) {
  positions_.resize(n_);
  velocities_.resize(n_);
  check(pbf_dump_data(sim_, &positions_[0].s[0], &velocities_[0].s[0]),
        "Simulation::dumpData");
  positions = positions_.data();
  velocities = velocities_.data();
}

void Simulation::setWaveGenerator(const double value) {
  check(pbf_set_wave(sim_, (float)value), "Simulation::setWaveGenerator");
}

namespace {

// Two pinned buffer pairs; a snapshot copies the state into the next pair
// (waiting for that pair's previous file to be written) and hands the file
// write to a thread.
class SnapshotWriter {
 public:
  SnapshotWriter(pbf_sim *sim, uint32_t n) : sim_(sim), n_(n) {}
  ~SnapshotWriter() { finish(); for (auto &s : slots_) release(s); }

  void take(const std::string &path, bool vtk) {
    Slot &s = slots_[next_];
    next_ ^= 1;
    if (s.writer.joinable()) s.writer.join();
    check(s.status, "Runner snapshot");
    if (!s.pos) {
      void *p = nullptr, *v = nullptr;
      check(pbf_host_alloc((size_t)n_ * 16, &p), "Runner snapshot");
      check(pbf_host_alloc((size_t)n_ * 16, &v), "Runner snapshot");
      s.pos = static_cast<float *>(p);
      s.vel = static_cast<float *>(v);
    }
    check(pbf_dump_data_async(sim_, s.pos, s.vel), "Runner snapshot");
    check(pbf_sync(sim_), "Runner snapshot");
    s.writer = std::thread([&s, path, vtk, n = n_]() {
      if (vtk) {
        s.status = pbf_write_vtk(path.c_str(), s.pos, s.vel, n);
        return;
      }
      std::vector<pbf_particle> ps(n);
      for (uint32_t k = 0; k < n; ++k) {
        pbf_particle &q = ps[k];
        q.m = s.vel[4 * (size_t)k + 3];
        for (int a = 0; a < 3; ++a) {
          q.x[a] = s.pos[4 * (size_t)k + a];
          q.v[a] = s.vel[4 * (size_t)k + a];
          q.a[a] = 0.0f;
        }
      }
      s.status = pbf_write_particles(path.c_str(), ps.data(), n);
    });
  }

  void finish() {
    for (auto &s : slots_)
      if (s.writer.joinable()) s.writer.join();
  }
  void check_written() {
    for (auto &s : slots_) check(s.status, "Runner snapshot");
  }

 private:
  struct Slot {
    float *pos = nullptr, *vel = nullptr;
    std::thread writer;
    int status = PBF_OK;
  };
  static void release(Slot &s) {
    if (s.pos) pbf_host_free(s.pos);
    if (s.vel) pbf_host_free(s.vel);
    s.pos = s.vel = nullptr;
  }
  pbf_sim *sim_;
  uint32_t n_;
  Slot slots_[2];
  int next_ = 0;
};

std::string frame_name(const char *base, const char *fallback, uint32_t frame, const char *ext) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%05u", frame);
  return std::string(base[0] ? base : fallback) + buf + ext;
}

}  // namespace

std::vector<double> Runner::run(const ConfigParameters &parameters,
                                Simulation &simulation, bool waves,
                                bool quiet) const {
  simulation.init();
  simulation.initCells();
  SnapshotWriter snapshots(simulation.handle(), simulation.getNumberParticles());
  uint64_t step_count = 0;
  const Float4 lo = simulation.getSizesMin(), hi = simulation.getSizesMax();
  float time = 0.0f, wave = 0.0f;
  std::vector<double> times;
  do {
    const auto t0 = std::chrono::steady_clock::now();
    simulation.step();
    time += parameters.time_step_length;
    if (waves) {
      // src/Runner.cpp:91-104
      const float push = (hi.s[0] - lo.s[0]) / 3.0f;
      const float freq = 1.0f, start = (float)(-M_PI / 2.0);
      const float value = std::sin(2.0f * (float)M_PI * freq * wave + start) *
                              push / 2.0f + push / 2.0f;
      simulation.setWaveGenerator(value);
      wave += parameters.time_step_length;
    }
    const auto t1 = std::chrono::steady_clock::now();
    times.push_back(std::chrono::duration<double>(t1 - t0).count());
    ++step_count;
    if (parameters.part_out_freq && step_count % parameters.part_out_freq == 0)
      snapshots.take(frame_name(parameters.part_out_name_base, "part",
                                (uint32_t)(step_count / parameters.part_out_freq), ".in"),
                     false);
    if (parameters.vtk_out_freq && step_count % parameters.vtk_out_freq == 0)
      snapshots.take(frame_name(parameters.vtk_out_name_base, "vtk",
                                (uint32_t)(step_count / parameters.vtk_out_freq), ".vtk"),
                     true);
  } while (time <= parameters.time_end);
  snapshots.finish();
  snapshots.check_written();
  if (!quiet && !times.empty()) {
    const double sum = std::accumulate(times.begin(), times.end(), 0.0);
    const double mean = sum / times.size();
    const double sq = std::inner_product(times.begin(), times.end(), times.begin(), 0.0);
    const double stdev = std::sqrt(std::max(0.0, sq / times.size() - mean * mean));
    std::vector<double> s = times;
    std::sort(s.begin(), s.end());
    const size_t m = s.size();
    const double median = m % 2 ? s[m / 2] : (s[m / 2 - 1] + s[m / 2]) / 2;
    std::cout << "mean: " << mean << "\nmedian: " << median << "\nstd: " << stdev
              << std::endl;
  }
  return times;
}

}  // namespace pbf
