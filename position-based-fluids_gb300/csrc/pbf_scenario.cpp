// Scenario layer: the .par / .in readers and writers, a binary particle
// format for large scenes, VTK output, data-path resolution and the seeded
// lattice generator.
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

// Binary particle file: "PBFB", u32 version 1, u64 count, then count
// pbf_particle records (10 little-endian float32 each: m, x, v, a).
constexpr char kBinMagic[4] = {'P', 'B', 'F', 'B'};
constexpr uint32_t kBinVersion = 1;

int read_particles_bin(std::ifstream &ifs, pbf_particle **out, uint32_t *n) {
  uint32_t version = 0;
  uint64_t count = 0;
  if (!ifs.read(reinterpret_cast<char *>(&version), 4) ||
      !ifs.read(reinterpret_cast<char *>(&count), 8) || version != kBinVersion ||
      count >= (1u << 30)) {
    pbf::set_error_message("bad binary particle header");
    return PBF_ERR_IO;
  }
  if (count == 0) return PBF_OK;
  pbf_particle *buf = static_cast<pbf_particle *>(std::malloc(count * sizeof(pbf_particle)));
  if (!buf) return PBF_ERR_OOM;
  if (!ifs.read(reinterpret_cast<char *>(buf), (std::streamsize)(count * sizeof(pbf_particle)))) {
    std::free(buf);
    pbf::set_error_message("binary particle file is short");
    return PBF_ERR_IO;
  }
  *out = buf;
  *n = (uint32_t)count;
  return PBF_OK;
}

// Big-endian copy of a float (legacy VTK binary data is big-endian).
void put_be(std::vector<char> &buf, float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  const char b[4] = {(char)(u >> 24), (char)(u >> 16), (char)(u >> 8), (char)u};
  buf.insert(buf.end(), b, b + 4);
}
void put_be(std::vector<char> &buf, int32_t v) {
  const uint32_t u = (uint32_t)v;
  const char b[4] = {(char)(u >> 24), (char)(u >> 16), (char)(u >> 8), (char)u};
  buf.insert(buf.end(), b, b + 4);
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
    else if (key == "grow_lists") ok = bool(ss >> out->grow_lists);
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
  {
    std::ifstream bin(path, std::ios::binary);
    char magic[4] = {0, 0, 0, 0};
    if (bin && bin.read(magic, 4) && std::memcmp(magic, kBinMagic, 4) == 0)
      return read_particles_bin(bin, out, n);
  }
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

int pbf_write_particles(const char *path, const pbf_particle *p, uint32_t n) {
  if (!path || (n && !p)) return PBF_ERR_INVALID;
  FILE *f = std::fopen(path, "w");
  if (!f) {
    pbf::set_error_message(std::string("could not open ") + path);
    return PBF_ERR_IO;
  }
  std::fprintf(f, "%u\n", n);
  for (uint32_t k = 0; k < n; ++k)
    std::fprintf(f, "%.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", p[k].m, p[k].x[0], p[k].x[1],
                 p[k].x[2], p[k].v[0], p[k].v[1], p[k].v[2]);
  const bool ok = std::fclose(f) == 0;
  return ok ? PBF_OK : PBF_ERR_IO;
}

int pbf_write_particles_bin(const char *path, const pbf_particle *p, uint32_t n) {
  if (!path || (n && !p)) return PBF_ERR_INVALID;
  std::ofstream f(path, std::ios::binary);
  if (!f) {
    pbf::set_error_message(std::string("could not open ") + path);
    return PBF_ERR_IO;
  }
  const uint64_t count = n;
  f.write(kBinMagic, 4);
  f.write(reinterpret_cast<const char *>(&kBinVersion), 4);
  f.write(reinterpret_cast<const char *>(&count), 8);
  if (n) f.write(reinterpret_cast<const char *>(p), (std::streamsize)n * sizeof(pbf_particle));
  return f ? PBF_OK : PBF_ERR_IO;
}

int pbf_write_config(const char *path, const pbf_params *p) {
  if (!path || !p) return PBF_ERR_INVALID;
  FILE *f = std::fopen(path, "w");
  if (!f) {
    pbf::set_error_message(std::string("could not open ") + path);
    return PBF_ERR_IO;
  }
  const char *mode = p->mode == PBF_MODE_REF_COMPAT ? "ref_compat" : "paper";
  if (p->part_input_file[0]) std::fprintf(f, "part_input_file       %s\n", p->part_input_file);
  std::fprintf(f,
               "time_end              %.9g\n"
               "timestep_length       %.9g\n"
               "x_min                 %.9g\n"
               "x_max                 %.9g\n"
               "y_min                 %.9g\n"
               "y_max                 %.9g\n"
               "z_min                 %.9g\n"
               "z_max                 %.9g\n"
               "x_n                   %.9g\n"
               "y_n                   %.9g\n"
               "z_n                   %.9g\n"
               "restdensity           %.9g\n"
               "part_out_freq         %u\n"
               "part_out_name_base    %s\n"
               "vtk_out_freq          %u\n"
               "vtk_out_name_base     %s\n"
               "mode                  %s\n"
               "solver_iterations     %u\n"
               "relax_eps             %.9g\n"
               "scorr_k               %.9g\n"
               "scorr_dq              %.9g\n"
               "scorr_n               %d\n"
               "xsph_c                %.9g\n"
               "vort_eps              %.9g\n"
               "gravity_y             %.9g\n"
               "wall_margin           %.9g\n"
               "max_neighbours        %u\n"
               "grow_lists            %u\n",
               p->time_end, p->time_step_length, p->x_min, p->x_max,
               p->y_min, p->y_max, p->z_min, p->z_max, p->x_n, p->y_n, p->z_n,
               p->rest_density, p->part_out_freq,
               p->part_out_name_base[0] ? p->part_out_name_base : "part",
               p->vtk_out_freq, p->vtk_out_name_base[0] ? p->vtk_out_name_base : "vtk", mode,
               p->solver_iterations, p->relax_eps, p->scorr_k, p->scorr_dq, p->scorr_n,
               p->xsph_c, p->vort_eps, p->gravity_y, p->wall_margin, p->max_neighbours,
               p->grow_lists);
  return std::fclose(f) == 0 ? PBF_OK : PBF_ERR_IO;
}

int pbf_write_vtk(const char *path, const float *pos4, const float *vel4, uint32_t n) {
  if (!path || (n && (!pos4 || !vel4))) return PBF_ERR_INVALID;
  std::vector<char> buf;
  const std::string head = "# vtk DataFile Version 3.0\nposition-based-fluids particles\n"
                           "BINARY\nDATASET POLYDATA\nPOINTS " + std::to_string(n) + " float\n";
  buf.insert(buf.end(), head.begin(), head.end());
  buf.reserve(buf.size() + (size_t)n * 36 + 256);
  for (uint32_t k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) put_be(buf, pos4[4 * (size_t)k + a]);
  const std::string verts = "\nVERTICES " + std::to_string(n) + " " + std::to_string(2ull * n) + "\n";
  buf.insert(buf.end(), verts.begin(), verts.end());
  for (uint32_t k = 0; k < n; ++k) {
    put_be(buf, (int32_t)1);
    put_be(buf, (int32_t)k);
  }
  const std::string pd = "\nPOINT_DATA " + std::to_string(n) +
                         "\nSCALARS speed float 1\nLOOKUP_TABLE default\n";
  buf.insert(buf.end(), pd.begin(), pd.end());
  for (uint32_t k = 0; k < n; ++k) put_be(buf, pos4[4 * (size_t)k + 3]);
  const std::string vv = "\nVECTORS velocity float\n";
  buf.insert(buf.end(), vv.begin(), vv.end());
  for (uint32_t k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) put_be(buf, vel4[4 * (size_t)k + a]);
  buf.push_back('\n');
  std::ofstream f(path, std::ios::binary);
  if (!f) {
    pbf::set_error_message(std::string("could not open ") + path);
    return PBF_ERR_IO;
  }
  f.write(buf.data(), (std::streamsize)buf.size());
  return f ? PBF_OK : PBF_ERR_IO;
}

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
