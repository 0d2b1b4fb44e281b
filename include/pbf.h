/*
 * pbf.h -- C-ABI of the GB300 position-based-fluids (PBF) step.
 *
 * This is the drop-in boundary for the simulation step of
 * MrMagne/position-based-fluids.  It replaces two reference interfaces:
 *
 *  1. the Simulation step interface (src/Simulation.hpp:41-108): construct,
 *     init(), initCells(), step(), dumpData(), the size getters and
 *     setWaveGenerator(); the reference's caller is Runner::run
 *     (src/Runner.cpp:43-46,83,102);
 *  2. the kernel operator interface for the neighbour structure, i.e. the
 *     `__kernel` entry points the reference looks up by name
 *     (src/ocl/clsetup.cpp:343-358) for the cell hash (update_cells.cl,
 *     calc_hash.cl), the radix sort of (cell, particle) keys
 *     (radix_histogram.cl, radix_scan.cl, radix_paste.cl, radix_reorder.cl)
 *     and the cell ranges (init_cells.cl, find_cells.cl).
 *
 * Conventions
 *  - Every function returns an int status (pbf_status); no exception crosses
 *    the boundary.  The reference throws cl::Error / std::runtime_error
 *    (src/hesp.hpp:33, src/io/ConfigReader.cpp, src/io/PartReader.cpp) and
 *    its main() exits on them
 *    (src/main.cpp:180-186).
 *  - Host arrays of particle state use the reference's dumpData layout
 *    (src/Simulation.cpp:578-591, 120-134): N float4 positions with
 *    .w = |v| after a step (0 before the first step), N float4 velocities
 *    with .w = particle mass.
 *  - A pbf_sim owns one CUDA stream.  Calls on one pbf_sim are not
 *    thread-safe; separate pbf_sim objects are independent.  pbf_step is
 *    asynchronous; pbf_sync, pbf_dump_data and the getters that read device
 *    state synchronise.
 *  - `void *stream` arguments are cudaStream_t values (0 = legacy default).
 *  - Device-pointer arguments (d_*) point to memory of the current CUDA
 *    device.
 */
#ifndef PBF_GB300_H
#define PBF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBF_ABI_VERSION 1

typedef enum {
  PBF_OK = 0,
  PBF_ERR_INVALID = 1,  /* bad argument or parameter combination          */
  PBF_ERR_OOM = 2,      /* device or pinned-host allocation failed         */
  PBF_ERR_CUDA = 3,     /* CUDA runtime error (see pbf_last_error_message) */
  PBF_ERR_DEVICE = 4,   /* a kernel's bounded wait gave up; results void   */
  PBF_ERR_IO = 5,       /* file could not be opened or parsed              */
  PBF_ERR_BUDGET = 6,   /* request does not fit the HBM budget             */
  PBF_ERR_STATE = 7,    /* call out of order (e.g. step before init)       */
  PBF_ERR_NOT_FOUND = 8 /* unknown scene / request id                      */
} pbf_status;

/* Equation set of the solver. */
typedef enum {
  /* The reference's kernels as shipped: relaxation 1e4, no s_corr, no
   * vorticity, density without the self term, XSPH c = 0.01 with 1/rho_j,
   * walls at h from the box, constants rounded to 6 significant digits as
   * src/main.cpp:149-168 prints them.  Results match the reference's
   * kernels run with each cell list in descending particle order. */
  PBF_MODE_REF_COMPAT = 0,
  /* Macklin & Mueller 2013 with the relaxation epsilon, s_corr, XSPH and
   * vorticity confinement taken from pbf_params; neighbour sets fixed at
   * the start of each step. */
  PBF_MODE_PAPER = 1
} pbf_mode;

/* ConfigParameters (src/Parameters.hpp:12-31) followed by the solver
 * settings the reference hard-codes in its kernels.  pbf_params_default
 * fills every field; pbf_read_config overwrites the fields a .par file
 * names (src/io/ConfigReader.cpp:45-84 keys, plus the extension keys listed
 * beside each field). */
typedef struct {
  char part_input_file[256];      /* part_input_file                      */
  float time_step_length;         /* timestep_length                      */
  float time_end;                 /* time_end                             */
  uint32_t part_out_freq;         /* part_out_freq                        */
  char part_out_name_base[256];   /* part_out_name_base                   */
  uint32_t vtk_out_freq;          /* vtk_out_freq                         */
  char vtk_out_name_base[256];    /* vtk_out_name_base                    */
  uint32_t cl_workgroup_1dsize;   /* cl_workgroup_1dsize (unused)         */
  float x_min, x_max, y_min, y_max, z_min, z_max; /* x_min ... z_max      */
  float x_n, y_n, z_n;            /* x_n y_n z_n: cells per axis          */
  float rest_density;             /* restdensity: particles per volume    */
  /* ---- extensions (keys in brackets) ---- */
  int32_t mode;                   /* [mode] ref_compat | paper            */
  uint32_t solver_iterations;     /* [solver_iterations] reference: 4     */
  float relax_eps;                /* [relax_eps] paper mode               */
  float scorr_k;                  /* [scorr_k]                            */
  float scorr_dq;                 /* [scorr_dq] fraction of h             */
  int32_t scorr_n;                /* [scorr_n]                            */
  float xsph_c;                   /* [xsph_c]                             */
  float vort_eps;                 /* [vort_eps]                           */
  float gravity_y;                /* [gravity_y] paper mode               */
  float wall_margin;              /* [wall_margin] paper mode, in metres  */
  uint32_t max_neighbours;        /* [max_neighbours] stored per particle */
  uint32_t grow_lists;            /* [grow_lists] 1: a simulation's list  */
                                  /* capacity grows with its scene (see   */
                                  /* pbf_list_capacity); 0: fixed         */
} pbf_params;

/* Particle (src/Particle.hpp:9-14): mass, position, velocity, acceleration
 * (the acceleration is never read, as in the reference). */
typedef struct {
  float m;
  float x[3];
  float v[3];
  float a[3];
} pbf_particle;

/* ------------------------------------------------------------------ misc */
int pbf_abi_version(void);
const char *pbf_status_string(int status);
/* Text of the last CUDA error seen by this thread (empty if none). */
const char *pbf_last_error_message(void);

/* Defaults: mode PAPER, 4 iterations, relax_eps 600, s_corr k 0.1 n 4
 * dq 0.2, XSPH c 0.01, vorticity eps 0.0005, gravity -9.81, wall margin
 * h/4 (resolved at create time when negative), max_neighbours 128,
 * grow_lists 1. */
void pbf_params_default(pbf_params *p);

/* ------------------------------------------------ scenario layer (L0) */
/* ConfigReader::read (src/io/ConfigReader.cpp:19-91).  Fields absent from
 * the file keep the values already in *out (call pbf_params_default
 * first); unknown keys are skipped with a warning on stderr, as in the
 * reference. */
int pbf_read_config(const char *path, pbf_params *out);
/* PartReader::read (src/io/PartReader.cpp:21-95): first line N, then one
 * "m x y z vx vy vz" line per particle.  *out is allocated by the library
 * (release with pbf_free); a malformed line ends the read with the
 * particles parsed so far and a warning, as in the reference. */
int pbf_read_particles(const char *path, pbf_particle **out, uint32_t *n);
void pbf_free(void *ptr);
/* Also reads the binary particle format (detected by its "PBFB" magic):
 * u32 version 1, u64 count, count pbf_particle records, little-endian. */
/* Writers: the .in text format above (values printed to round-trip float32
 * exactly), the binary format, a .par file with every key (reference keys
 * and the extension keys), and a legacy binary VTK POLYDATA file of the
 * dumpData arrays (points, |v| as "speed", velocity vectors).  No
 * reference counterpart (the reference reads scenarios only; its
 * part_out_* / vtk_out_* keys are parsed but unused). */
int pbf_write_particles(const char *path, const pbf_particle *p, uint32_t n);
int pbf_write_particles_bin(const char *path, const pbf_particle *p, uint32_t n);
int pbf_write_config(const char *path, const pbf_params *p);
int pbf_write_vtk(const char *path, const float *pos4, const float *vel4, uint32_t n);
/* DataLoader::getPathFor* (src/DataLoader.cpp:20-31) with an explicit root
 * instead of the executable's directory: root/data/<kind>s/<name> for kind
 * "scenario", "kernel", "shader" or "texture". */
int pbf_data_path(const char *root, const char *kind, const char *name,
                  char *out, size_t cap);
/* Lattice block generator (the semantics of tools/gen_grid.py, with seeded
 * jitter): nx*ny*nz particles at `spacing` from `origin`, each coordinate
 * jittered by U(-jitter, +jitter) from a splitmix64 stream seeded with
 * `seed`, zero velocity, mass `mass`.  `out` holds nx*ny*nz particles. */
int pbf_generate_block(const float origin[3], uint32_t nx, uint32_t ny,
                       uint32_t nz, float spacing, float jitter, float mass,
                       uint64_t seed, pbf_particle *out);

/* ---------------------------------------- Simulation step interface (L3) */
typedef struct pbf_sim pbf_sim;

/* Simulation::Simulation.  Copies the parameters and particles; no device
 * work yet.  Rejects: n == 0, a grid with fewer than one cell per axis or
 * more than 2^31 cells, a non-positive time step or rest density, and in
 * paper mode a cell shorter than h on any axis (the 27-cell search would
 * miss neighbours). */
int pbf_create(const pbf_params *params, const pbf_particle *particles,
               uint32_t n, pbf_sim **out);
/* Simulation::init: selects the current CUDA device, creates the stream,
 * allocates device state and uploads the particles. */
int pbf_init(pbf_sim *sim);
/* Simulation::initCells: validates that init ran.  The neighbour structure
 * is rebuilt inside every step, so there is no separate cell state. */
int pbf_init_cells(pbf_sim *sim);
/* Simulation::step, `nsteps` times, enqueued on the sim's stream. */
int pbf_step(pbf_sim *sim, uint32_t nsteps);
/* Waits for the sim's stream; returns PBF_ERR_DEVICE if a kernel reported
 * an error since the last check. */
int pbf_sync(pbf_sim *sim);
/* Simulation::dumpData into caller memory: pos4/vel4 hold N float4 each,
 * in the input particle order.  Blocking. */
int pbf_dump_data(pbf_sim *sim, float *pos4, float *vel4);
/* Replaces the state (same layout as pbf_dump_data).  Blocking. */
int pbf_set_state(pbf_sim *sim, const float *pos4, const float *vel4);
/* Stream-ordered variants for page-locked host buffers: they return after
 * enqueueing; the copies complete in stream order. */
int pbf_set_state_async(pbf_sim *sim, const float *pos4, const float *vel4);
int pbf_dump_data_async(pbf_sim *sim, float *pos4, float *vel4);
/* Page-locked host buffer helpers for the async variants. */
int pbf_host_alloc(size_t bytes, void **out);
int pbf_host_free(void *ptr);
/* Simulation::setWaveGenerator: offset of the moving x-min wall. */
int pbf_set_wave(pbf_sim *sim, float value);
int pbf_get_num_particles(const pbf_sim *sim, uint32_t *n);
/* getSizesMin / getSizesMax (.w = 0). */
int pbf_get_sizes(const pbf_sim *sim, float min4[4], float max4[4]);
/* The cudaStream_t of the sim (valid after pbf_init). */
int pbf_get_stream(const pbf_sim *sim, void **stream);
/* Per-stage device times of the last step run with timing enabled:
 * ms[0] neighbour search (predict, hash, sort, cell ranges, reorder),
 * ms[1] lambda passes, ms[2] delta-p passes, ms[3] velocity update.
 * Enabling timing turns off CUDA-graph replay for the timed steps. */
int pbf_set_stage_timing(pbf_sim *sim, int enable);
int pbf_stage_times(pbf_sim *sim, float ms[4]);
/* Per-kernel device times accumulated over every step run since timing was
 * last enabled: for entry q < min(cap, *count), names[32q..32q+31] is the
 * kernel (or kernel group) name, total_ms[q] its summed time and
 * launches[q] its number of kernel launches.  *count receives the number of
 * entries; any output pointer but count may be NULL. */
int pbf_kernel_times(pbf_sim *sim, uint32_t cap, char *names, float *total_ms,
                     uint32_t *launches, uint32_t *count);
/* Replays each step as one CUDA graph (default on). */
int pbf_set_graph(pbf_sim *sim, int enable);
/* Number of this library's kernel launches one step issues. */
int pbf_launches_per_step(const pbf_sim *sim, uint32_t *launches);

/* Launch shape of the paper-mode gather passes, per pass: index 0 the
 * neighbour-list build, 1 the list build fused with the first lambda, 2
 * lambda, 3 delta-p, 4 vorticity, 5 XSPH + commit.  threads = 64, 128 or
 * 256 per CTA; batch = 4 or 8 neighbour loads in flight per thread (ignored
 * for 0 and 1); fuse_first = 1 (the default) runs 1 instead of 0 + 2 for
 * the first solver iteration.  staged = 1 runs every gather pass on staged cell blocks
 * instead: persistent CTAs walk the step's occupied blocks of 4 x 4 x 4
 * cells, copy each block's neighbourhood into shared memory with bulk
 * asynchronous copies and read neighbours from there (threads, batch and
 * fuse_first then do not apply).  radix_sort = 1 sorts the step's cell keys
 * with the onesweep radix sort instead of the counting sort by cell (the
 * default); both give the stable permutation.  masked_build = 1 (the
 * default) has the list build (0 and 1) test each row of candidates into a
 * membership mask and store the members from the mask afterwards; 0 stores
 * each member as it is found.  No choice changes a result bit.  trial_ms is the tuner's best time per launch of each pass (0 when
 * untuned). */
typedef struct pbf_tuning {
  uint32_t threads[6];
  uint32_t batch[6];
  uint32_t fuse_first;
  float trial_ms[6];
  uint32_t staged;
  uint32_t radix_sort;
  uint32_t masked_build;
} pbf_tuning;
/* Times every shape over `trial_steps` steps (1..32) of this simulation
 * from its current state, keeps the fastest per pass and restores the state
 * (PAPER mode; a no-op returning the defaults in REF_COMPAT mode).  Later
 * steps are bitwise the ones an untuned simulation takes.  `out` may be
 * NULL.  No reference counterpart. */
int pbf_autotune(pbf_sim *sim, uint32_t trial_steps, pbf_tuning *out);
int pbf_get_tuning(const pbf_sim *sim, pbf_tuning *out);
/* PBF_ERR_INVALID for a shape outside the values above. */
int pbf_set_tuning(pbf_sim *sim, const pbf_tuning *tuning);
/* Density of every particle from the last lambda pass of the last step
 * (input order). */
int pbf_get_density(pbf_sim *sim, float *density);
/* Neighbour lists of the last step (PAPER mode): the largest neighbour
 * count and how many particles had more neighbours than the list capacity
 * (max_neighbours rounded down to a multiple of 8).  Those particles
 * re-derive their sets from the cells in every pass, several times as slow
 * as a listed set; a nonzero *overflow says the capacity is too small for
 * the scene.  PBF_ERR_STATE in REF_COMPAT mode or before the first step. */
int pbf_neighbour_stats(pbf_sim *sim, uint32_t *max_count, uint32_t *overflow);
/* Neighbour-list capacity (entries per particle) the simulation uses now,
 * and how many times it has grown.  It starts at max_neighbours rounded down
 * to a multiple of 8 and grows by itself: each step records its largest
 * neighbour count, and when that comes within 1/8 of the capacity the lists
 * are reallocated to 1.5x the count (at most 1024) before the next step is
 * launched, unless pbf_params.grow_lists is 0.  (Batches and servers keep
 * the capacity they were created with.)  (pbf_step therefore keeps at most two steps queued: before
 * launching a step it waits for the step two back -- the first step's
 * count right after that step -- while the step before still runs.)  No
 * reference counterpart; grows may be NULL. */
int pbf_list_capacity(const pbf_sim *sim, uint32_t *capacity, uint32_t *grows);
/* Staged cell blocks of the last step (PAPER mode with staged = 1 in the
 * tuning): how many occupied blocks of 4 x 4 x 4 cells staged their
 * neighbourhood in shared memory and how many gathered through L1 instead
 * (more than 3072 candidates in the block's neighbourhood).  Both 0 when
 * the last step ran the L1 passes.  PBF_ERR_STATE in REF_COMPAT mode or
 * before the first step.  No reference counterpart. */
int pbf_tile_stats(pbf_sim *sim, uint32_t *staged, uint32_t *unstaged);
/* The neighbour structure the last step built, in input particle order:
 * hash[i] = cell of particle i; perm[q] = input index of the particle at
 * sorted position q (ties by input index in REF_COMPAT mode, by previous
 * sorted position in PAPER mode); ranges = inclusive (first,last) int2 per
 * cell, (-1,-1) if empty.  Any pointer may be NULL. */
int pbf_get_cells(pbf_sim *sim, uint32_t *hash, uint32_t *perm,
                  int32_t *ranges);
int pbf_destroy(pbf_sim *sim);

/* ------------------------------------------------- headless rendering */
/* The reference's particle drawing (src/visual/visual.cpp:86-125,217-330,
 * src/shaders/particlevertex.glsl, particlefragment.glsl) as CUDA kernels
 * writing an image instead of a window: a spherical camera around `target`
 * (angles in degrees, negative distance as the reference uses), a
 * perspective projection, point sprites of 200 / clip.w pixels shaded as
 * spheres lit from (1,1,1), colour (|v|, |v|, 1), depth test "less" with
 * ties to the lower input index, background 0.05 grey. */
typedef struct pbf_camera {
  float phi_deg, theta_deg, distance;
  float target[3];
  float fovy_deg, znear, zfar;
  float max_point_size;           /* cap on a sprite's diameter, pixels   */
} pbf_camera;
/* The reference's initial camera for this box. */
void pbf_camera_default(const pbf_params *p, pbf_camera *out);
/* Renders the current state into rgb (width * height * 3 bytes, rows top
 * first).  Synchronous. */
int pbf_render(pbf_sim *sim, const pbf_camera *cam, uint32_t width,
               uint32_t height, uint8_t *rgb);

/* ------------------------------------------------------ batched scenes */
/* Many independent scenes advanced together (no counterpart in the
 * reference, which runs one scene): one sort over scene-major keys (scene s
 * owns the key range [cell_base_s, cell_base_s + cells_s), i.e. the scene in
 * the high-order part of the key), one launch per kernel for all scenes, and
 * each step replayed as one CUDA graph.  A scene's trajectory is the same,
 * bit for bit, alone (pbf_sim) and in any mix.
 *
 * Solver settings come from `solver` (mode must be PBF_MODE_PAPER; time
 * step, rest density, h = (x_max - x_min) / x_n, iterations, relaxation,
 * s_corr, XSPH, vorticity, gravity, max_neighbours).  Each scene brings its
 * own box, grid and wall margin.  Capacities fix the device allocation. */
typedef struct pbf_batch pbf_batch;
int pbf_batch_create(const pbf_params *solver, uint32_t max_scenes,
                     uint32_t max_particles, uint32_t max_cells,
                     pbf_batch **out);
/* Device bytes a batch with these capacities allocates. */
size_t pbf_batch_device_bytes(const pbf_params *solver, uint32_t max_scenes,
                              uint32_t max_particles, uint32_t max_cells);
/* Adds a scene; *scene_id identifies it until removal.  Takes effect at the
 * next step.  PBF_ERR_BUDGET if a capacity would be exceeded. */
int pbf_batch_add_scene(pbf_batch *b, const pbf_params *scene,
                        const pbf_particle *particles, uint32_t n,
                        uint32_t *scene_id);
int pbf_batch_remove_scene(pbf_batch *b, uint32_t scene_id);
/* Advances every scene `nsteps` steps, enqueued on the batch's stream. */
int pbf_batch_step(pbf_batch *b, uint32_t nsteps);
int pbf_batch_sync(pbf_batch *b);
/* State of one scene in its input particle order (dumpData layout). */
int pbf_batch_dump_scene(pbf_batch *b, uint32_t scene_id, float *pos4,
                         float *vel4);
int pbf_batch_set_wave(pbf_batch *b, uint32_t scene_id, float value);
int pbf_batch_info(const pbf_batch *b, uint32_t *scenes, uint32_t *particles,
                   uint32_t *cells);
int pbf_batch_get_stream(const pbf_batch *b, void **stream);
int pbf_batch_launches_per_step(const pbf_batch *b, uint32_t *launches);
/* pbf_neighbour_stats over every scene of the batch (the last step's
 * lists); PBF_ERR_STATE until a step has run since the last add or
 * remove. */
int pbf_batch_neighbour_stats(pbf_batch *b, uint32_t *max_count, uint32_t *overflow);
/* pbf_autotune for a batch, over the scenes it holds. */
int pbf_batch_autotune(pbf_batch *b, uint32_t trial_steps, pbf_tuning *out);
int pbf_batch_get_tuning(const pbf_batch *b, pbf_tuning *out);
int pbf_batch_set_tuning(pbf_batch *b, const pbf_tuning *tuning);
int pbf_batch_destroy(pbf_batch *b);
/* pbf_render for one scene of a batch (the scene's own box). */
int pbf_batch_render_scene(pbf_batch *b, uint32_t scene_id, const pbf_camera *cam,
                           uint32_t width, uint32_t height, uint8_t *rgb);

/* ------------------------------------------------------- served scenes */
/* A request loop over one batch (continuous batching).  Requests (a scene
 * and a step count) are queued by pbf_server_submit; pbf_server_poll
 * retires the requests whose steps are done (their final state is copied to
 * host memory held by the server), admits queued requests in arrival order
 * while they fit the batch (first fit: a request that does not fit yet does
 * not hold back smaller ones behind it), and enqueues the next chunk of
 * batched steps.  A chunk is at most `max_chunk` steps and never longer than
 * the fewest steps any active request still needs, so every request runs
 * exactly its own step count.  The batch's capacities are derived from an
 * HBM budget at creation and allocated once; admission never allocates.
 * A request's result is bitwise the same as the scene run alone.
 * No reference counterpart (the reference runs one scene per process). */
typedef struct pbf_server pbf_server;

typedef enum pbf_request_state {
  PBF_REQ_QUEUED = 0,
  PBF_REQ_ACTIVE = 1,
  PBF_REQ_DONE = 2
} pbf_request_state;

typedef struct pbf_server_stats {
  uint64_t submitted, admitted, completed;
  uint64_t batch_steps;          /* batched steps enqueued                */
  uint64_t particle_steps;       /* sum over steps of active particles    */
  uint32_t queued, active;       /* requests now waiting / on the device  */
  uint32_t active_particles, active_cells;
  uint32_t max_particles, max_cells, max_scenes; /* capacities            */
  uint32_t pad_;
  uint64_t device_bytes;         /* bytes the batch allocated             */
  uint64_t launches;             /* kernel launches enqueued              */
} pbf_server_stats;

/* Creates a server whose batch fits `hbm_budget_bytes` of device memory.
 * Cells are budgeted at `cells_per_particle` per particle slot (at least 1).
 * PBF_ERR_BUDGET if the budget holds no useful batch. */
int pbf_server_create(const pbf_params *solver, uint64_t hbm_budget_bytes,
                      uint32_t max_scenes, float cells_per_particle,
                      uint32_t max_chunk, pbf_server **out);
/* Queues a request (the particles are copied).  PBF_ERR_BUDGET if the
 * scene alone exceeds the server's capacities. */
int pbf_server_submit(pbf_server *s, const pbf_params *scene,
                      const pbf_particle *particles, uint32_t n,
                      uint32_t steps, uint64_t *request_id);
/* One turn of the loop.  With `wait` = 0 it returns at once while a chunk
 * is still running (*ncompleted = 0); with `wait` = 1 it first waits for the
 * running chunk.  Ids of requests completed in this turn are written to
 * completed[0 .. min(*ncompleted, cap)).  *busy is set to 1 while requests
 * remain queued or active. */
int pbf_server_poll(pbf_server *s, int wait, uint64_t *completed, uint32_t cap,
                    uint32_t *ncompleted, int *busy);
int pbf_server_request_info(const pbf_server *s, uint64_t request_id,
                            int *state, uint32_t *n, uint32_t *steps_done);
/* Copies a completed request's final state (dumpData layout) and releases
 * it.  PBF_ERR_STATE if it is not done, PBF_ERR_NOT_FOUND if unknown. */
int pbf_server_result(pbf_server *s, uint64_t request_id, float *pos4,
                      float *vel4);
int pbf_server_stats_get(const pbf_server *s, pbf_server_stats *out);
int pbf_server_destroy(pbf_server *s);

/* ------------------------------------ neighbour-structure operators (L4) */
/* Cell hash of N predicted positions (float4, .w ignored) on the grid of
 * `params` (update_cells.cl:10-15 / calc_hash.cl:15-20).  Each axis cell
 * is trunc((p - min) / cell_length) clamped to [0, n-1]; inside the grid
 * the clamp never fires. */
int pbf_op_cell_hash(const pbf_params *params, const float *d_pred4,
                     uint32_t n, uint32_t *d_hash, void *stream);
/* Bytes of device scratch pbf_op_sort_pairs needs. */
size_t pbf_op_sort_scratch_bytes(uint32_t n, uint32_t key_bits);
/* Stable LSD radix sort of (key, value) pairs by the low `key_bits` bits
 * of key (onesweep: one histogram pass, then one pass per 8-bit digit with
 * decoupled look-back).  d_vals_in may be NULL, meaning values 0..n-1,
 * which makes d_vals_out the stable permutation (ties by index).  Inputs
 * are not modified; outputs must not alias inputs.  Keys must be < 2^key_bits. */
int pbf_op_sort_pairs(const uint32_t *d_keys_in, const uint32_t *d_vals_in,
                      uint32_t n, uint32_t key_bits, uint32_t *d_keys_out,
                      uint32_t *d_vals_out, void *d_scratch,
                      size_t scratch_bytes, void *stream);
/* Synchronises `stream` and reports PBF_ERR_DEVICE if the last
 * pbf_op_sort_pairs with this scratch, n and key_bits had a look-back wait
 * give up (its output is then void). */
int pbf_op_sort_status(const void *d_scratch, uint32_t n, uint32_t key_bits,
                       void *stream);
/* pbf_op_sort_pairs without any device allocation, for callers that cannot
 * allocate (a host engine whose own pool owns all device memory, or a
 * per-frame callback where cudaMalloc/cudaFree would synchronise the device).
 * No counterpart in the reference.  Scratch is a file-scope device array
 * sized for at most 1048576 keys (about 9.4 MB on every GPU that loads the
 * library, held until exit); larger n returns PBF_ERR_INVALID.  The first
 * call in a device's context looks the array's address up
 * (cudaGetSymbolAddress), so make that first call before any stream
 * capture; a later context on the same device (after cudaDeviceReset) is
 * recognised by its id and looked up again on its first call.  All calls
 * share the array: calls whose work overlaps on the GPU race.  If d_status
 * is not NULL, look-back failures are OR-ed into *d_status (zeroed by the
 * caller); otherwise they are not reported, so pass it wherever the result
 * matters. */
int pbf_op_sort_pairs_noalloc(const uint32_t *d_keys_in,
                              const uint32_t *d_vals_in, uint32_t n,
                              uint32_t key_bits, uint32_t *d_keys_out,
                              uint32_t *d_vals_out, uint32_t *d_status,
                              void *stream);
/* Bytes of device scratch pbf_op_sort_cells needs. */
size_t pbf_op_sort_cells_scratch_bytes(uint32_t n, uint32_t ncells);
/* The stable sort of cell keys (every key < ncells) in one counting pass,
 * as the PAPER step sorts: d_offsets[c] = number of keys < c for c in
 * [0, ncells] (the CSR cell offsets), d_sorted_keys and d_perm the stable
 * order (ties by index: d_perm[q] = index of the q-th key), the same as
 * pbf_op_sort_pairs with values NULL followed by pbf_op_cell_offsets.
 * Keys are counted per cell with warp-aggregated atomics, the counts
 * scanned into the offsets (decoupled look-back), every key scattered to its
 * cell, and each cell put back in index order (by one thread up to 16 keys,
 * one warp up to 64, in shared memory up to 8192, through a bitmap of the
 * indices beyond).
 * Outputs must not alias the keys.  No reference counterpart beyond the
 * intent of init_cells.cl + find_cells.cl + the radix kernels. */
int pbf_op_sort_cells(const uint32_t *d_keys, uint32_t n, uint32_t ncells,
                      uint32_t *d_offsets, uint32_t *d_sorted_keys, uint32_t *d_perm,
                      void *d_scratch, size_t scratch_bytes, void *stream);
/* Synchronises `stream` and reports PBF_ERR_DEVICE if the last
 * pbf_op_sort_cells with this scratch, n and ncells had its look-back wait
 * give up (its output is then void). */
int pbf_op_sort_cells_status(const void *d_scratch, uint32_t n, uint32_t ncells, void *stream);
/* CSR cell offsets of sorted keys: d_offsets[c] = number of keys < c for
 * c in [0, ncells]; every key must be < ncells. */
int pbf_op_cell_offsets(const uint32_t *d_sorted_keys, uint32_t n,
                        uint32_t ncells, uint32_t *d_offsets, void *stream);
/* The reference's cell ranges (init_cells.cl + find_cells.cl intent):
 * inclusive (first,last) int2 per cell, (-1,-1) if empty. */
/* Failure-detection self-test: runs the radix sort's bounded look-back wait
 * against a predecessor tile that never publishes, with `spin_limit` polls
 * (1 .. 2^26).  The wait gives up, the kernel sets its error bit and
 * returns; the call reports PBF_ERR_DEVICE with the device flag word in
 * *device_flag, and the CUDA context stays usable.  PBF_OK would mean the
 * wait did not give up.  No reference counterpart. */
int pbf_selftest_bounded_wait(uint32_t spin_limit, uint32_t *device_flag);
int pbf_op_find_cells(const uint32_t *d_offsets, uint32_t ncells,
                      int32_t *d_first_last, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PBF_GB300_H */
