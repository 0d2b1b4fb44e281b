/*
 * TEST INFRASTRUCTURE (oracle) -- never linked into the product library.
 *
 * A C++ rendering of the small subset of OpenCL C 1.1 that the reference's
 * live kernels (MrMagne/position-based-fluids, src/kernels/*.cl) use, so that
 * g++ can compile those kernel files *unchanged* as host code:
 *
 *   g++ -x c++ -include oracle/clshim.hpp -c src/kernels/compute_scaling.cl
 *
 * What is rendered here, and the semantics chosen where OpenCL leaves room:
 *   - address-space qualifiers (__kernel/__global/__local) vanish;
 *   - get_global_id(0) reads a thread-local work-item id that the launcher
 *     (oracle/ref_launch.cpp) sets before each call, one call per work-item;
 *   - float3 / float4 with component access (.x .y .z .w), the .xyz swizzle
 *     (read, write, +=), and the element-wise operators the kernels use;
 *   - length(v) = sqrt((x*x + y*y) + z*z), evaluated in that order;
 *   - atomic_xchg on int via the GCC builtin;
 *   - the -D constants that src/main.cpp:149-168 bakes into the program are
 *     routed to a global struct (clshim_k) that the launcher fills with the
 *     same 6-significant-digit values main.cpp prints.
 *
 * All arithmetic is IEEE-754 binary32 with FMA contraction disabled
 * (-ffp-contract=off): one legal execution of the reference's kernels, whose
 * build flags (-cl-fast-relaxed-math -cl-mad-enable) merely *permit* a
 * compiler to deviate from it.
 *
 * predict_positions.cl writes a vector literal `(float3)(a, b, c)`, which a
 * C++ compiler would read as a cast of a comma expression.  That file is
 * compiled with oracle/clshim_predict.hpp instead, which spells float3 as a
 * constructor function for that single translation unit.
 */
#ifndef PBF_ORACLE_CLSHIM_HPP
#define PBF_ORACLE_CLSHIM_HPP

#include <cmath>
#include <cstddef>

typedef unsigned int uint;

#define __kernel
#define __global
#define __local
#define __constant const

using std::sqrt;

/* ---- work-item id -------------------------------------------------------- */
extern thread_local size_t clshim_global_id;
static inline size_t get_global_id(uint) { return clshim_global_id; }

/* ---- constants baked by the reference host (src/main.cpp:149-168) -------- */
struct clshim_constants {
  float k_SYSTEM_MIN_X;
  float k_SYSTEM_MAX_X;
  float k_SYSTEM_MIN_Y;
  float k_SYSTEM_MAX_Y;
  float k_SYSTEM_MIN_Z;
  float k_SYSTEM_MAX_Z;
  float k_NUMBER_OF_CELLS_X;
  float k_NUMBER_OF_CELLS_Y;
  float k_NUMBER_OF_CELLS_Z;
  float k_CELL_LENGTH_X;
  float k_CELL_LENGTH_Y;
  float k_CELL_LENGTH_Z;
  float k_TIMESTEP;
  float k_REST_DENSITY;
  float k_PBF_H;
  float k_PBF_H_2;
  float k_POLY6_FACTOR;
  float k_GRAD_SPIKY_FACTOR;
};
extern clshim_constants clshim_k;

#define SYSTEM_MIN_X (clshim_k.k_SYSTEM_MIN_X)
#define SYSTEM_MAX_X (clshim_k.k_SYSTEM_MAX_X)
#define SYSTEM_MIN_Y (clshim_k.k_SYSTEM_MIN_Y)
#define SYSTEM_MAX_Y (clshim_k.k_SYSTEM_MAX_Y)
#define SYSTEM_MIN_Z (clshim_k.k_SYSTEM_MIN_Z)
#define SYSTEM_MAX_Z (clshim_k.k_SYSTEM_MAX_Z)
#define NUMBER_OF_CELLS_X (clshim_k.k_NUMBER_OF_CELLS_X)
#define NUMBER_OF_CELLS_Y (clshim_k.k_NUMBER_OF_CELLS_Y)
#define NUMBER_OF_CELLS_Z (clshim_k.k_NUMBER_OF_CELLS_Z)
#define CELL_LENGTH_X (clshim_k.k_CELL_LENGTH_X)
#define CELL_LENGTH_Y (clshim_k.k_CELL_LENGTH_Y)
#define CELL_LENGTH_Z (clshim_k.k_CELL_LENGTH_Z)
#define TIMESTEP (clshim_k.k_TIMESTEP)
#define REST_DENSITY (clshim_k.k_REST_DENSITY)
#define PBF_H (clshim_k.k_PBF_H)
#define PBF_H_2 (clshim_k.k_PBF_H_2)
#define POLY6_FACTOR (clshim_k.k_POLY6_FACTOR)
#define GRAD_SPIKY_FACTOR (clshim_k.k_GRAD_SPIKY_FACTOR)

/* The linked-cell build (src/CMakeLists.txt:9 and src/main.cpp:145-147). */
#ifndef USE_LINKEDCELL
#define USE_LINKEDCELL 1
#endif

/* ---- vector types --------------------------------------------------------- */
struct clshim_float3 {
  float x, y, z;
  clshim_float3() = default;
  explicit clshim_float3(float s) : x(s), y(s), z(s) {}
  clshim_float3(float a, float b, float c) : x(a), y(b), z(c) {}
};

static inline clshim_float3 operator+(clshim_float3 a, clshim_float3 b) {
  return clshim_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
static inline clshim_float3 operator-(clshim_float3 a, clshim_float3 b) {
  return clshim_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
static inline clshim_float3 operator*(float s, clshim_float3 a) {
  return clshim_float3(s * a.x, s * a.y, s * a.z);
}
static inline clshim_float3 operator*(clshim_float3 a, float s) {
  return clshim_float3(a.x * s, a.y * s, a.z * s);
}
static inline clshim_float3 operator/(clshim_float3 a, float s) {
  return clshim_float3(a.x / s, a.y / s, a.z / s);
}
static inline clshim_float3 &operator+=(clshim_float3 &a, clshim_float3 b) {
  a = a + b;
  return a;
}
static inline float length(clshim_float3 a) {
  return sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
}

/* .xyz of a float4: an lvalue view of the first three components. */
struct clshim_swz_xyz {
  float s[4];
  operator clshim_float3() const { return clshim_float3(s[0], s[1], s[2]); }
  clshim_swz_xyz &operator=(const clshim_float3 &v) {
    s[0] = v.x;
    s[1] = v.y;
    s[2] = v.z;
    return *this;
  }
  clshim_swz_xyz &operator=(const clshim_swz_xyz &o) {
    return *this = clshim_float3(o);
  }
  clshim_swz_xyz &operator+=(const clshim_float3 &v) {
    return *this = clshim_float3(*this) + v;
  }
};

union clshim_float4 {
  struct {
    float x, y, z, w;
  };
  clshim_swz_xyz xyz;
  clshim_float4() { x = y = z = w = 0.0f; }
  explicit clshim_float4(float v) { x = y = z = w = v; }
  clshim_float4(float a, float b, float c, float d) {
    x = a;
    y = b;
    z = c;
    w = d;
  }
  clshim_float4(const clshim_float4 &o) {
    x = o.x;
    y = o.y;
    z = o.z;
    w = o.w;
  }
  clshim_float4 &operator=(const clshim_float4 &o) {
    x = o.x;
    y = o.y;
    z = o.z;
    w = o.w;
    return *this;
  }
};

static inline clshim_float4 operator+(const clshim_float4 &a,
                                      const clshim_float4 &b) {
  return clshim_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
static inline clshim_float4 operator-(const clshim_float4 &a,
                                      const clshim_float4 &b) {
  return clshim_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
static inline clshim_float4 operator*(float s, const clshim_float4 &a) {
  return clshim_float4(s * a.x, s * a.y, s * a.z, s * a.w);
}
static inline clshim_float4 operator*(const clshim_float4 &a, float s) {
  return clshim_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}
static inline clshim_float4 operator/(const clshim_float4 &a, float s) {
  return clshim_float4(a.x / s, a.y / s, a.z / s, a.w / s);
}
static inline clshim_float4 &operator+=(clshim_float4 &a,
                                        const clshim_float4 &b) {
  a = a + b;
  return a;
}

typedef clshim_float4 float4;
#ifndef CLSHIM_FLOAT3_IS_CONSTRUCTOR
typedef clshim_float3 float3;
#endif

/* ---- atomics ------------------------------------------------------------- */
static inline int atomic_xchg(volatile int *p, int v) {
  return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST);
}

#endif /* PBF_ORACLE_CLSHIM_HPP */
