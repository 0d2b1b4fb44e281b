/*
 * TEST INFRASTRUCTURE (oracle) -- never linked into the product library.
 *
 * Force-included instead of clshim.hpp for the one reference kernel file
 * that writes an OpenCL vector literal, predict_positions.cl:8
 *   `(float3)(0.0f, -9.81f, 0.0f)`.
 * In C++ that text parses as a cast applied to a comma expression.  Here
 * `float3` is spelled as a function that builds the vector, so the same text
 * becomes a three-argument constructor call.  That file declares no variable
 * of type float3, so nothing else changes meaning.
 */
#ifndef PBF_ORACLE_CLSHIM_PREDICT_HPP
#define PBF_ORACLE_CLSHIM_PREDICT_HPP

#define CLSHIM_FLOAT3_IS_CONSTRUCTOR 1
#include "clshim.hpp"

static inline clshim_float3 clshim_make_float3(float a, float b, float c) {
  return clshim_float3(a, b, c);
}
#define float3 clshim_make_float3

#endif /* PBF_ORACLE_CLSHIM_PREDICT_HPP */
