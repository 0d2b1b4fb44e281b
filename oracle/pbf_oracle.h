/*
 * TEST INFRASTRUCTURE (oracle) -- never linked into the product library.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * the library built from these declarations, and only as the oracle results
 * are compared against.
 *
 * C-ABI of the CPU restatement in oracle/pbf_oracle.cpp:
 *   - REF_COMPAT step: the reference's live kernels restated line by line
 *     (src/kernels/*.cl, step order src/Simulation.cpp:455-576), in float
 *     and in double;
 *   - PBF_PAPER step in double: Macklin & Mueller 2013 "Position Based
 *     Fluids" with the relaxation, tensile (s_corr), XSPH and vorticity
 *     terms, neighbour sets fixed at the start of each step;
 *   - the neighbour-structure intent of the reference's sort path: the cell
 *     hash (src/kernels/update_cells.cl:10-15), a stable sort of (cell,
 *     particle index) (src/kernels/calc_hash.cl, radix_*.cl) and inclusive
 *     [first,last] cell ranges with -1 for empty cells
 *     (src/kernels/init_cells.cl, find_cells.cl).
 */
#ifndef PBF_ORACLE_H
#define PBF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Raw .par values the reference's simulation reads (src/Parameters.hpp). */
typedef struct {
  float x_min, x_max, y_min, y_max, z_min, z_max;
  float x_n, y_n, z_n;
  float timestep_length;
  float rest_density;
} oracle_config;

/* PBF_PAPER parameters (double precision). rest_density is a number density
 * (particles per unit volume), as in the reference. */
typedef struct {
  double box_min[3], box_max[3];
  int32_t n_cells[3];
  int32_t iterations;
  double dt, rest_density, h;
  double relax_eps;   /* epsilon in the lambda denominator            */
  double scorr_k;     /* tensile instability term k                   */
  double scorr_dq;    /* delta q as a fraction of h                   */
  double xsph_c;      /* XSPH viscosity c                             */
  double vort_eps;    /* vorticity confinement epsilon                */
  double gravity_y;   /* gravity along y                              */
  double wall_margin; /* particles are kept this far inside the box   */
  int32_t scorr_n;    /* tensile instability exponent n               */
  int32_t pad_;
} oracle_paper_params;

/* The 18 constants src/main.cpp:149-168 bakes, in this order:
 * SYSTEM_MIN/MAX_X, _Y, _Z, NUMBER_OF_CELLS_X/Y/Z, CELL_LENGTH_X/Y/Z,
 * TIMESTEP, REST_DENSITY, PBF_H, PBF_H_2, POLY6_FACTOR, GRAD_SPIKY_FACTOR. */
int oracle_ref_constants(const oracle_config *cfg, float *out18);

/* Cell hash of each predicted position (float4 per particle). */
int oracle_cell_hash(const oracle_config *cfg, const float *pred4, uint32_t n,
                     uint32_t *hash_out);

/* Stable ascending sort of hash, ties by particle index. */
int oracle_sort_cells(const uint32_t *hash, uint32_t n,
                      uint32_t *sorted_hash_out, uint32_t *perm_out);

/* Inclusive [first,last] per cell (int2), (-1,-1) if empty. */
int oracle_find_cells(const uint32_t *sorted_hash, uint32_t n,
                      uint32_t ncells, int32_t *first_last_out);

/* REF_COMPAT: `steps` reference steps in place on pos4/vel4 (dumpData
 * layout).  Cell lists are built in ascending index order, so each list runs
 * in descending index, as a sequential launch of updateCells produces.
 * Optional outputs from the last step (NULL to skip): predicted4, scaling. */
int oracle_refcompat_steps_f32(const oracle_config *cfg, uint32_t n,
                               float *pos4, float *vel4, uint32_t steps,
                               float wave, int threads, float *predicted4_out,
                               float *scaling_out);
int oracle_refcompat_steps_f64(const oracle_config *cfg, uint32_t n,
                               double *pos4, double *vel4, uint32_t steps,
                               double wave, int threads);

/* PBF_PAPER in double: `steps` steps in place on pos4/vel4.  Optional
 * outputs from the last step: density (N), lambda of the last iteration (N),
 * neighbour counts (N). */
int oracle_paper_steps_f64(const oracle_paper_params *p, uint32_t n,
                           double *pos4, double *vel4, uint32_t steps,
                           double wave, int threads, double *density_out,
                           double *lambda_out, uint32_t *nbr_count_out);
/* The same algorithm evaluated in float (IEEE, no contraction), for
 * measuring how far binary32 arithmetic alone moves the result. */
int oracle_paper_steps_f32(const oracle_paper_params *p, uint32_t n,
                           double *pos4, double *vel4, uint32_t steps,
                           double wave, int threads, double *density_out,
                           double *lambda_out, uint32_t *nbr_count_out);

#ifdef __cplusplus
}
#endif

#endif /* PBF_ORACLE_H */
