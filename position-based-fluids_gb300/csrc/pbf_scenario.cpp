// Scenario layer: the .par / .in readers, data-path resolution and the
// seeded lattice generator.
//
// Reference: ConfigReader::read (src/io/ConfigReader.cpp:19-91),
// PartReader::read (src/io/PartReader.cpp:21-95), DataLoader
// (src/DataLoader.cpp:7-31), tools/gen_grid.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "pbf_host.hpp"

namespace {

void copy_string(char *dst, size_t cap, const std::string &s) {
  std::strncpy(dst, s.c_str(), cap - 1);
  dst[cap - 1] = '\0';
}

uint64_t splitmix64(uint64_t *state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int pbf_read_config(const char *path, pbf_params *out) {
  if (!path || !out) return PBF_ERR_INVALID;
  std::ifstream ifs(path);
  if (!ifs) {
    pbf::set_error_message(std::string("could not open parameter file ") + path);
    return PBF_ERR_IO;
  }
  std::string line;
  size_t line_number = 0;
  while (std::getline(ifs, line)) {
    ++line_number;
    if (line.empty()) continue;
    std::istringstream ss(line);
    std::string key;
    if (!(ss >> key)) continue;
    bool ok = true;
    if (key == "part_input_file") {
      std::string v;
      ok = bool(ss >> v);
      if (ok) copy_string(out->part_input_file, sizeof out->part_input_file, v);
    } else if (key == "timestep_length") ok = bool(ss >> out->time_step_length);
    else if (key == "time_end") ok = bool(ss >> out->time_end);
    else if (key == "part_out_freq") ok = bool(ss >> out->part_out_freq);
    else if (key == "part_out_name_base") {
      std::string v;
      ok = bool(ss >> v);
      if (ok) copy_string(out->part_out_name_base, sizeof out->part_out_name_base, v);
    } else if (key == "vtk_out_freq") ok = bool(ss >> out->vtk_out_freq);
    else if (key == "vtk_out_name_base") {
      std::string v;
      ok = bool(ss >> v);
      if (ok) copy_string(out->vtk_out_name_base, sizeof out->vtk_out_name_base, v);
    } else if (key == "cl_workgroup_1dsize") ok = bool(ss >> out->cl_workgroup_1dsize);
    else if (key == "x_min") ok = bool(ss >> out->x_min);
    else if (key == "x_max") ok = bool(ss >> out->x_max);
    else if (key == "y_min") ok = bool(ss >> out->y_min);
    else if (key == "y_max") ok = bool(ss >> out->y_max);
    else if (key == "z_min") ok = bool(ss >> out->z_min);
    else if (key == "z_max") ok = bool(ss >> out->z_max);
    else if (key == "x_n") ok = bool(ss >> out->x_n);
    else if (key == "y_n") ok = bool(ss >> out->y_n);
    else if (key == "z_n") ok = bool(ss >> out->z_n);
    else if (key == "restdensity") ok = bool(ss >> out->rest_density);
    /* extension keys */
    else if (key == "mode") {
      std::string v;
      ok = bool(ss >> v);
      if (ok) {
        if (v == "ref_compat" || v == "0") out->mode = PBF_MODE_REF_COMPAT;
        else if (v == "paper" || v == "1") out->mode = PBF_MODE_PAPER;
        else ok = false;
      }
    } else if (key == "solver_iterations") ok = bool(ss >> out->solver_iterations);
    else if (key == "relax_eps") ok = bool(ss >> out->relax_eps);
    else if (key == "scorr_k") ok = bool(ss >> out->scorr_k);
    else if (key == "scorr_dq") ok = bool(ss >> out->scorr_dq);
    else if (key == "scorr_n") ok = bool(ss >> out->scorr_n);
    else if (key == "xsph_c") ok = bool(ss >> out->xsph_c);
    else if (key == "vort_eps") ok = bool(ss >> out->vort_eps);
    else if (key == "gravity_y") ok = bool(ss >> out->gravity_y);
    else if (key == "wall_margin") ok = bool(ss >> out->wall_margin);
    else if (key == "max_neighbours") ok = bool(ss >> out->max_neighbours);
    else {
      std::cerr << "Unknown parameter " << key << std::endl
                << "Leaving it out." << std::endl;
      continue;
    }
    if (!ok) {
      pbf::set_error_message("could not parse value of " + key + " in line " +
                             std::to_string(line_number));
      return PBF_ERR_IO;
    }
  }
  return PBF_OK;
}

int pbf_read_particles(const char *path, pbf_particle **out, uint32_t *n) {
  if (!path || !out || !n) return PBF_ERR_INVALID;
  *out = nullptr;
  *n = 0;
  std::ifstream ifs(path);
  if (!ifs) {
    pbf::set_error_message(std::string("could not open particle file ") + path);
    return PBF_ERR_IO;
  }
  std::string line;
  if (!std::getline(ifs, line)) {
    pbf::set_error_message("could not parse number of particles");
    return PBF_ERR_IO;
  }
  size_t count = 0;
  {
    std::istringstream ssn(line);
    if (!(ssn >> count)) {
      pbf::set_error_message("could not parse number of particles");
      return PBF_ERR_IO;
    }
  }
  if (count >= (1u << 30)) {
    pbf::set_error_message("particle count too large");
    return PBF_ERR_IO;
  }
  std::vector<pbf_particle> ps;
  ps.reserve(count);
  for (size_t k = 0; k < count; ++k) {
    if (!std::getline(ifs, line)) {
      std::cerr << "Error parsing particle in line " << (k + 2) << std::endl;
      break;
    }
    std::istringstream ss(line);
    pbf_particle p;
    std::memset(&p, 0, sizeof p);
    if (!(ss >> p.m)) {
      std::cerr << "Error parsing particle mass in line " << (k + 2) << std::endl;
      break;
    }
    bool ok = true;
    for (int a = 0; a < 3 && ok; ++a) ok = bool(ss >> p.x[a]);
    for (int a = 0; a < 3 && ok; ++a) ok = bool(ss >> p.v[a]);
    if (!ok) {
      std::cerr << "Error parsing particle position/velocity in line " << (k + 2)
                << std::endl;
      break;
    }
    ps.push_back(p);
  }
  if (ps.empty()) {
    *n = 0;
    return PBF_OK;
  }
  pbf_particle *buf = static_cast<pbf_particle *>(std::malloc(ps.size() * sizeof(pbf_particle)));
  if (!buf) return PBF_ERR_OOM;
  std::memcpy(buf, ps.data(), ps.size() * sizeof(pbf_particle));
  *out = buf;
  *n = (uint32_t)ps.size();
  return PBF_OK;
}

void pbf_free(void *ptr) { std::free(ptr); }

int pbf_data_path(const char *root, const char *kind, const char *name,
                  char *out, size_t cap) {
  if (!root || !kind || !name || !out || cap == 0) return PBF_ERR_INVALID;
  std::string sub;
  const std::string k(kind);
  if (k == "scenario") sub = "scenarios";
  else if (k == "kernel") sub = "kernels";
  else if (k == "shader") sub = "shaders";
  else if (k == "texture") sub = "textures";
  else return PBF_ERR_INVALID;
  const std::string path = std::string(root) + "/data/" + sub + "/" + name;
  if (path.size() + 1 > cap) return PBF_ERR_INVALID;
  std::memcpy(out, path.c_str(), path.size() + 1);
  return PBF_OK;
}

int pbf_generate_block(const float origin[3], uint32_t nx, uint32_t ny,
                       uint32_t nz, float spacing, float jitter, float mass,
                       uint64_t seed, pbf_particle *out) {
  if (!origin || !out || nx == 0 || ny == 0 || nz == 0) return PBF_ERR_INVALID;
  if ((uint64_t)nx * ny * nz >= (1ull << 30)) return PBF_ERR_INVALID;
  uint64_t state = seed;
  size_t q = 0;
  // Lattice order of tools/gen_grid.py: x outermost, z innermost.
  for (uint32_t ix = 0; ix < nx; ++ix)
    for (uint32_t iy = 0; iy < ny; ++iy)
      for (uint32_t iz = 0; iz < nz; ++iz, ++q) {
        pbf_particle &p = out[q];
        std::memset(&p, 0, sizeof p);
        p.m = mass;
        const uint32_t idx[3] = {ix, iy, iz};
        for (int a = 0; a < 3; ++a) {
          const double u = (double)(splitmix64(&state) >> 11) * (1.0 / 9007199254740992.0);
          const double off = (2.0 * u - 1.0) * (double)jitter;
          p.x[a] = (float)((double)origin[a] + (double)idx[a] * (double)spacing + off);
        }
      }
  return PBF_OK;
}

}  // extern "C"
