// Headless particle renderer: the reference's point-sprite drawing restated
// as CUDA kernels writing an RGB8 image (no graphics stack).
//
// Reference: the particle pass of CVisual::visualizeParticles
// (src/visual/visual.cpp:270-330) with the camera of
// CVisual::resolveCamPosition / calcLookAtMatrix (:86-125) and the matrices
// set up at :217-227 (glm::perspective(45, w/h, 0.1, 1000), the box moved to
// be centred on the origin); the vertex shader
// (src/shaders/particlevertex.glsl: gl_PointSize = 200 / clip.w) and the
// fragment shader (src/shaders/particlefragment.glsl: a sphere normal from
// gl_PointCoord, discard outside the unit disc, colour (|v|, |v|, 1) times
// clamp(dot(n, (1,1,1)), 0, 1)); depth test GL_LESS with depth cleared to 1
// and colour cleared to 0.05 grey.
//
// The translation unit is compiled with -fmad=false (and its host code
// without floating-point contraction): every expression rounds operator by
// operator in IEEE binary32, with correctly rounded division and square
// root, so the image is reproducible bit for bit by a restatement that
// evaluates the same expressions in the same order.
//
// GL rasterises points in submission order; here each pixel keeps the
// fragment of least depth, ties to the lowest input index (the particle GL
// would have drawn first), through a 64-bit atomicMin on (depth bits, index),
// so the image does not depend on thread scheduling.  A second pass shades
// every pixel from its winning particle.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>

#include "pbf_host.hpp"

namespace pbf {
namespace {

struct RenderView {
  float m[16];        // clip = m * (p, 1), column-major like glm
  float width, height;
  float max_size;     // largest point size in pixels
  float half[3];      // box centre offset (model-to-world translation)
};

// Sprite of particle position p: window centre (x, y), window depth z and
// point size s.  False if GL would clip the point (centre outside the view
// volume).
__device__ __forceinline__ bool sprite(const RenderView &v, float px, float py, float pz,
                                       float &x, float &y, float &z, float &s) {
  const float wx = px + v.half[0], wy = py + v.half[1], wz = pz + v.half[2];
  const float cx = v.m[0] * wx + v.m[4] * wy + v.m[8] * wz + v.m[12];
  const float cy = v.m[1] * wx + v.m[5] * wy + v.m[9] * wz + v.m[13];
  const float cz = v.m[2] * wx + v.m[6] * wy + v.m[10] * wz + v.m[14];
  const float cw = v.m[3] * wx + v.m[7] * wy + v.m[11] * wz + v.m[15];
  if (!(cw > 0.0f) || fabsf(cx) > cw || fabsf(cy) > cw || fabsf(cz) > cw) return false;
  const float inv = 1.0f / cw;
  x = (cx * inv + 1.0f) * 0.5f * v.width;
  y = (cy * inv + 1.0f) * 0.5f * v.height;
  z = (cz * inv + 1.0f) * 0.5f;
  s = fminf(200.0f * inv, v.max_size);
  return true;
}

// gl_PointCoord mapped to [-1, 1]^2 for the pixel whose lower-left corner is
// (ix, iy) in window coordinates (origin lower left; point coordinates have
// their origin at the sprite's upper left).
__device__ __forceinline__ void point_coord(float x, float y, float s, int ix, int iy,
                                            float &mx, float &my) {
  const float u = ((float)ix + 0.5f - (x - 0.5f * s)) / s;
  const float w = ((y + 0.5f * s) - ((float)iy + 0.5f)) / s;
  mx = u * 2.0f - 1.0f;
  my = w * 2.0f - 1.0f;
}

__global__ void k_render_clear(unsigned long long *__restrict__ zbuf, uint32_t pixels) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < pixels) zbuf[i] = ~0ull;
}

__global__ void k_render_splat(const float4 *__restrict__ X, const uint32_t *__restrict__ ID,
                               uint32_t n, RenderView v, unsigned long long *__restrict__ zbuf) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float4 p = X[k];
  float x, y, z, s;
  if (!sprite(v, p.x, p.y, p.z, x, y, z, s)) return;
  const uint32_t idx = ID ? ID[k] : k;
  const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | idx;
  const int W = (int)v.width, H = (int)v.height;
  // pixels whose centres fall inside the sprite square
  const int x0 = max(0, (int)ceilf(x - 0.5f * s - 0.5f));
  const int x1 = min(W - 1, (int)floorf(x + 0.5f * s - 0.5f));
  const int y0 = max(0, (int)ceilf(y - 0.5f * s - 0.5f));
  const int y1 = min(H - 1, (int)floorf(y + 0.5f * s - 0.5f));
  for (int iy = y0; iy <= y1; ++iy)
    for (int ix = x0; ix <= x1; ++ix) {
      float mx, my;
      point_coord(x, y, s, ix, iy, mx, my);
      if (mx * mx + my * my > 1.0f) continue;
      atomicMin(&zbuf[(size_t)iy * W + ix], key);
    }
}

// Shades every pixel from its winning particle; rows are written top first.
__global__ void k_render_shade(const float4 *__restrict__ X, const uint32_t *__restrict__ ID,
                               const uint32_t *__restrict__ slot_of, uint32_t n, RenderView v,
                               const unsigned long long *__restrict__ zbuf,
                               uint8_t *__restrict__ rgb) {
  const int W = (int)v.width, H = (int)v.height;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)(W * H)) return;
  const int ix = (int)(i % (uint32_t)W), iy = (int)(i / (uint32_t)W);
  float r = 0.05f, g = 0.05f, b = 0.05f;
  const unsigned long long key = zbuf[i];
  if (key != ~0ull) {
    const uint32_t idx = (uint32_t)(key & 0xffffffffu);
    const uint32_t k = min(ID ? slot_of[idx] : idx, n - 1u);
    const float4 p = X[k];
    float x, y, z, s, mx, my;
    if (sprite(v, p.x, p.y, p.z, x, y, z, s)) {
      point_coord(x, y, s, ix, iy, mx, my);
      const float l2 = mx * mx + my * my;
      const float nz = sqrtf(fmaxf(0.0f, 1.0f - l2));
      const float inv = 1.0f / sqrtf(fmaxf(l2 + nz * nz, 1e-30f));
      const float cosang = fminf(fmaxf((mx + my + nz) * inv, 0.0f), 1.0f);
      r = p.w * cosang;
      g = p.w * cosang;
      b = cosang;
    }
  }
  const size_t o = ((size_t)(H - 1 - iy) * W + ix) * 3;
  rgb[o + 0] = (uint8_t)__float2int_rn(fminf(fmaxf(r, 0.0f), 1.0f) * 255.0f);
  rgb[o + 1] = (uint8_t)__float2int_rn(fminf(fmaxf(g, 0.0f), 1.0f) * 255.0f);
  rgb[o + 2] = (uint8_t)__float2int_rn(fminf(fmaxf(b, 0.0f), 1.0f) * 255.0f);
}

__global__ void k_render_invert(const uint32_t *__restrict__ ID, uint32_t n,
                                uint32_t *__restrict__ slot_of) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) slot_of[min(ID[k], n - 1u)] = k;
}

// glm-style column-major 4x4 helpers (host).
void mat_mul(const float a[16], const float b[16], float out[16]) {
  float r[16];
  for (int c = 0; c < 4; ++c)
    for (int row = 0; row < 4; ++row) {
      float acc = 0.f;
      for (int k = 0; k < 4; ++k) acc += a[k * 4 + row] * b[c * 4 + k];
      r[c * 4 + row] = acc;
    }
  std::memcpy(out, r, sizeof r);
}

}  // namespace

void render_view_matrix(const pbf_camera &cam, float aspect, float out[16]) {
  // camera position on the sphere around the target (visual.cpp:89-100)
  const double phi = M_PI / 180.0 * (cam.phi_deg - 90.0);
  const double theta = M_PI / 180.0 * (cam.theta_deg + 90.0);
  const float dir[3] = {(float)(std::sin(theta) * std::cos(phi)), (float)std::cos(theta),
                        (float)(std::sin(theta) * std::sin(phi))};
  float eye[3], look[3];
  for (int a = 0; a < 3; ++a) eye[a] = dir[a] * cam.distance + cam.target[a];
  for (int a = 0; a < 3; ++a) look[a] = cam.target[a] - eye[a];
  auto normalize = [](float v[3]) {
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int a = 0; a < 3; ++a) v[a] /= l;
  };
  normalize(look);
  float up[3] = {0.f, 1.f, 0.f};
  float right[3] = {look[1] * up[2] - look[2] * up[1], look[2] * up[0] - look[0] * up[2],
                    look[0] * up[1] - look[1] * up[0]};
  normalize(right);
  const float pup[3] = {right[1] * look[2] - right[2] * look[1],
                        right[2] * look[0] - right[0] * look[2],
                        right[0] * look[1] - right[1] * look[0]};
  // view = R * T (visual.cpp:104-125)
  float view[16] = {right[0], pup[0], -look[0], 0.f, right[1], pup[1], -look[1], 0.f,
                    right[2], pup[2], -look[2], 0.f, 0.f,      0.f,    0.f,      1.f};
  float trans[16] = {1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f,
                     0.f, 0.f, 1.f, 0.f, -eye[0], -eye[1], -eye[2], 1.f};
  mat_mul(view, trans, view);
  // perspective (glm::perspective with fovy in degrees)
  const float f = 1.0f / (float)std::tan(M_PI / 180.0 * cam.fovy_deg / 2.0);
  const float zn = cam.znear, zf = cam.zfar;
  float proj[16] = {0.f};
  proj[0] = f / aspect;
  proj[5] = f;
  proj[10] = -(zf + zn) / (zf - zn);
  proj[11] = -1.f;
  proj[14] = -(2.f * zf * zn) / (zf - zn);
  mat_mul(proj, view, out);
}

int render_particles(const float4 *X, const uint32_t *ID, uint32_t n, const pbf_params &prm,
                     const pbf_camera &cam, uint32_t width, uint32_t height, uint8_t *rgb,
                     cudaStream_t st) {
  if (width == 0 || height == 0 || width > 16384 || height > 16384) return PBF_ERR_INVALID;
  RenderView v;
  render_view_matrix(cam, (float)width / (float)height, v.m);
  v.width = (float)width;
  v.height = (float)height;
  v.max_size = cam.max_point_size > 0.f ? cam.max_point_size : 64.f;
  // model-to-world: the box moved by minus half its extent (visual.cpp:219-223)
  v.half[0] = -(prm.x_max - prm.x_min) / 2.0f;
  v.half[1] = -(prm.y_max - prm.y_min) / 2.0f;
  v.half[2] = -(prm.z_max - prm.z_min) / 2.0f;
  const uint32_t pixels = width * height;
  unsigned long long *zbuf = nullptr;
  uint8_t *img = nullptr;
  uint32_t *slot_of = nullptr;
  int rc = PBF_OK;
  auto cuda = [&](cudaError_t e, const char *where) {
    if (e != cudaSuccess && rc == PBF_OK) rc = cuda_status(e, where);
    return rc == PBF_OK;
  };
  if (cuda(cudaMallocAsync(&zbuf, (size_t)pixels * 8, st), "render alloc") &&
      cuda(cudaMallocAsync(&img, (size_t)pixels * 3, st), "render alloc") &&
      (!ID || cuda(cudaMallocAsync(&slot_of, (size_t)n * 4, st), "render alloc"))) {
    k_render_clear<<<(pixels + 255) / 256, 256, 0, st>>>(zbuf, pixels);
    if (ID && n) k_render_invert<<<(n + 255) / 256, 256, 0, st>>>(ID, n, slot_of);
    if (n) k_render_splat<<<(n + 127) / 128, 128, 0, st>>>(X, ID, n, v, zbuf);
    k_render_shade<<<(pixels + 255) / 256, 256, 0, st>>>(X, ID, slot_of, n ? n : 1u, v, zbuf,
                                                          img);
    if (cuda(cudaGetLastError(), "render launch"))
      cuda(cudaMemcpyAsync(rgb, img, (size_t)pixels * 3, cudaMemcpyDeviceToHost, st),
           "render copy");
    cuda(cudaStreamSynchronize(st), "render sync");
  }
  if (zbuf) cudaFreeAsync(zbuf, st);
  if (img) cudaFreeAsync(img, st);
  if (slot_of) cudaFreeAsync(slot_of, st);
  cudaStreamSynchronize(st);
  return rc;
}

}  // namespace pbf

extern "C" void pbf_camera_default(const pbf_params *p, pbf_camera *out) {
  if (!out) return;
  std::memset(out, 0, sizeof *out);
  // CVisual's initial camera sphere (visual.cpp:38-39) with the distance set
  // from the box depth (:225)
  out->phi_deg = 0.0f;
  out->theta_deg = 20.0f;
  out->distance = p ? -(p->z_max - p->z_min) * 2.0f : -1.0f;
  out->fovy_deg = 45.0f;
  out->znear = 0.1f;
  out->zfar = 1000.0f;
  out->max_point_size = 64.0f;
}
