// C++ host interface of the GB300 position-based-fluids step, shaped like
// the reference's so that its callers port line for line:
//   ConfigParameters / ConfigReader  (src/Parameters.hpp, src/io/ConfigReader.*)
//   Particle / PartReader            (src/Particle.hpp, src/io/PartReader.*)
//   DataLoader                       (src/DataLoader.*)
//   Simulation                       (src/Simulation.hpp:41-108)
//   Runner                           (src/Runner.*), headless
// Everything here sits on the C-ABI of include/pbf.h; errors surface as
// std::runtime_error, as the reference's readers and cl::Error did.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pbf.h"

namespace pbf {

using ConfigParameters = pbf_params;
using Particle = pbf_particle;

// The reference's cl_float4: four floats addressed as .s[0..3].
struct Float4 {
  float s[4];
};

class ConfigReader {
 public:
  // Starts from pbf_params_default, then applies the file.
  ConfigParameters read(const std::string &filename) const;
};

class PartReader {
 public:
  std::vector<Particle> read(const std::string &filename) const;
};

class DataLoader {
 public:
  // The reference derives the root from the executable's directory
  // (macOS only); here it is explicit.
  explicit DataLoader(std::string root) : root_(std::move(root)) {}
  std::string getPathForScenario(const std::string &scenario) const;
  std::string getPathForKernel(const std::string &kernel) const;
  std::string getPathForShader(const std::string &shader) const;
  std::string getPathForTexture(const std::string &texture) const;

 private:
  std::string path(const char *kind, const std::string &name) const;
  std::string root_;
};

class Simulation {
 public:
  // The OpenCL kernel map, context, device and GL buffer of the reference
  // constructor have no counterpart: the kernels are compiled in and the
  // positions live in a device buffer read back by dumpData.
  Simulation(const ConfigParameters &parameters,
             const std::vector<Particle> &particles);
  ~Simulation();
  Simulation(const Simulation &) = delete;
  Simulation &operator=(const Simulation &) = delete;

  void init();
  void initCells();
  void step();
  // Copies current positions and velocities into arrays owned by this
  // object; the pointers stay valid until the next dumpData or destruction.
  void dumpData(Float4 *&positions, Float4 *&velocities);

  uint32_t getNumberParticles() const { return n_; }
  float getSizeXmin() const { return params_.x_min; }
  float getSizeXmax() const { return params_.x_max; }
  float getSizeYmin() const { return params_.y_min; }
  float getSizeYmax() const { return params_.y_max; }
  float getSizeZmin() const { return params_.z_min; }
  float getSizeZmax() const { return params_.z_max; }
  Float4 getSizesMin() const { return {{params_.x_min, params_.y_min, params_.z_min, 0.0f}}; }
  Float4 getSizesMax() const { return {{params_.x_max, params_.y_max, params_.z_max, 0.0f}}; }
  void setWaveGenerator(const double value);

  pbf_sim *handle() const { return sim_; }

 private:
  ConfigParameters params_;
  uint32_t n_ = 0;
  pbf_sim *sim_ = nullptr;
  std::vector<Float4> positions_, velocities_;
};

class Runner {
 public:
  // Runner::run (src/Runner.cpp:24-160) without the window: init,
  // initCells, step until time_end (optionally with the sinusoidal wave
  // wall of src/Runner.cpp:91-104), then mean/median/std of the per-step
  // wall times.  Returns the per-step times in seconds.
  //
  // Snapshots: every part_out_freq steps the state is written as
  // <part_out_name_base><frame>.in (the scenario format) and every
  // vtk_out_freq steps as <vtk_out_name_base><frame>.vtk; frames count from
  // 1, five digits.  The copy from the device goes into one of two pinned
  // buffers and a host thread writes the file while stepping goes on.
  std::vector<double> run(const ConfigParameters &parameters,
                          Simulation &simulation, bool waves = false,
                          bool quiet = false) const;
};

// Throws std::runtime_error with the library's message for a failed status.
void check(int status, const char *what);

}  // namespace pbf
