// Headless runner: the reference's main() (src/main.cpp:40-189) without the
// window, the OpenCL setup or the renderer.
//
//   pbf_run <scenario.par> [--root DIR] [--waves] [--out positions.txt]
//
// Reads the .par file (and the .in file it names, looked up next to the
// .par unless --root gives a DataLoader root), runs Runner::run until
// time_end and prints mean/median/std of the per-step times.  --out writes
// the final state as an .in file (the reference's PartReader format).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "Simulation.hpp"

int main(int argc, char **argv) {
  if (argc < 2) {
    std::cerr << "usage: pbf_run <scenario.par> [--root DIR] [--waves] [--out FILE]\n";
    return 2;
  }
  std::string par = argv[1], root, out;
  bool waves = false;
  for (int i = 2; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--root") && i + 1 < argc) root = argv[++i];
    else if (!std::strcmp(argv[i], "--waves")) waves = true;
    else if (!std::strcmp(argv[i], "--out") && i + 1 < argc) out = argv[++i];
  }
  try {
    pbf::ConfigReader config_reader;
    pbf::ConfigParameters parameters = config_reader.read(par);
    std::string part_file;
    if (!root.empty()) {
      part_file = pbf::DataLoader(root).getPathForScenario(parameters.part_input_file);
    } else {
      const size_t slash = par.find_last_of('/');
      part_file = (slash == std::string::npos ? std::string() : par.substr(0, slash + 1)) +
                  parameters.part_input_file;
    }
    pbf::PartReader part_reader;
    std::vector<pbf::Particle> particles = part_reader.read(part_file);
    pbf::Simulation simulation(parameters, particles);
    pbf::Runner runner;
    runner.run(parameters, simulation, waves);
    if (!out.empty()) {
      pbf::Float4 *pos = nullptr, *vel = nullptr;
      simulation.dumpData(pos, vel);
      std::ofstream f(out);
      f << particles.size() << "\n";
      for (size_t i = 0; i < particles.size(); ++i) {
        f << vel[i].s[3] << " " << pos[i].s[0] << " " << pos[i].s[1] << " "
          << pos[i].s[2] << " " << vel[i].s[0] << " " << vel[i].s[1] << " "
          << vel[i].s[2] << "\n";
      }
    }
  } catch (const std::exception &e) {
    std::cerr << "Error caught: " << e.what() << std::endl;
    return 1;
  }
  return 0;
}
