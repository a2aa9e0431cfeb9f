/* fsgpu -- GB300 (sm_103a) implementation of Fluid_Simulation's per-step
 * PIC/FLIP + MAC-grid + pressure-projection path, behind a C ABI.
 *
 * The reference's boundary for this path is a C++ class API:
 *   FluidDomain(int, int, MyFloat, MyFloat, MyFloat density, MyFloat pic_ratio)
 *       (include/FluidDomain.h:40-48, src/FluidDomain.cpp:54-68)
 *   FluidSolverMemoryPool(const FluidDomain&)  (include/FluidSolver.h:17-22)
 *   FluidSolver(FluidSolverMemoryPool)         (include/FluidSolver.h:48)
 *   FluidSolver::step{SemiLagrangian,PIC,FLIP,PICFLIP}(FluidDomain&, MyFloat dt)
 *       (include/FluidSolver.h:51-54, src/FluidSolver.cpp:99-251)
 * A handle here is one FluidDomain together with its FluidSolver: the grid,
 * the marker particles and the solver's scratch pool live in device memory
 * (HBM) for the handle's lifetime.  The C++ drop-in headers in
 * fluid_simulation_gb300/dropin keep the reference's class API and call these
 * functions.
 *
 * Conventions: every function returns an int status (FS_OK = 0).  Host
 * pointers are plain host memory; *_device variants take device pointers.
 * Work is queued on the handle's CUDA stream; functions that return data to
 * the host synchronise that stream.  A handle is not thread-safe (nor is the
 * reference's FluidSolver); distinct handles are independent.  Arrays are
 * row-major, index i + j * size_x (include/Grid.h:63-67); particles are
 * interleaved {pos_x, pos_y, vel_x, vel_y} floats, the layout of
 * MarkerParticle (include/MarkerParticleSet.h:43-50).
 */
#ifndef FSGPU_H
#define FSGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define FS_API __attribute__((visibility("default")))
#else
#define FS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define FS_OK 0
#define FS_ERR_INVALID_ARGUMENT 1
#define FS_ERR_VALIDATE 2       /* domain/pool mismatch: the reference throws std::runtime_error
                                   (src/FluidSolver.cpp:89-107, 215-221) */
#define FS_ERR_CUDA 3
#define FS_ERR_TIMEOUT 4        /* a bounded device-side wait gave up */
#define FS_ERR_TOO_LARGE 5
#define FS_ERR_INTERNAL 6
#define FS_ERR_OUT_OF_MEMORY 7

/* Warning bits of fs_step_stats.warnings. */
#define FS_WARN_PARTICLE_OUTSIDE 1u  /* a particle lay outside the grid when pressureSolve counted
                                        particles per cell; the reference indexes out of bounds there
                                        (src/FluidSolver.cpp:353-360), this build skips it */
#define FS_WARN_CG_NOT_CONVERGED 2u  /* the CG stopped at its iteration limit (the reference ignores
                                        this, src/FluidSolver.cpp:424-425) */

/* CellType (include/MacGrid.h:14-17). */
#define FS_LIQUID 0
#define FS_AIR 1
#define FS_SOLID 2

/* Grids of MacGrid (include/MacGrid.h:164-176). */
#define FS_U_FRONT 0
#define FS_V_FRONT 1
#define FS_U_BACK 2
#define FS_V_BACK 3
#define FS_U_PREV 4
#define FS_V_PREV 5
#define FS_U_DIFF 6
#define FS_V_DIFF 7

/* Step methods: FluidSolver::step* (include/FluidSolver.h:51-54). */
#define FS_STEP_SEMI_LAGRANGIAN 0
#define FS_STEP_PIC 1
#define FS_STEP_FLIP 2
#define FS_STEP_PICFLIP 3

/* Single phases, in the reference's function granularity. */
#define FS_PH_CLASSIFY 0       /* FluidDomain::classifyCells(MarkerParticleSet&), src/FluidDomain.cpp:150-180 */
#define FS_PH_P2G 1            /* FluidSolver::transferVelocityToGridSpread, src/FluidSolver.cpp:873-919 */
#define FS_PH_SAVE_PREV 2      /* MacGrid::updatePreviousVelocityBuffer, src/MacGrid.cpp:52-56 */
#define FS_PH_GRAVITY 3        /* FluidSolver::addExternalAcceleration, src/FluidSolver.cpp:276-295 */
#define FS_PH_DIRICHLET 4      /* FluidSolver::enforceDirichlet, src/FluidSolver.cpp:297-321 */
#define FS_PH_EXTEND 5         /* FluidSolver::extendVelocityIndividual, src/FluidSolver.cpp:485-622 */
#define FS_PH_PRESSURE 6       /* FluidSolver::pressureSolve, src/FluidSolver.cpp:323-483 */
#define FS_PH_SAVE_DIFF 7      /* MacGrid::updateVelocityDiffBuffer, src/MacGrid.cpp:58-70 */
#define FS_PH_G2P_PICFLIP 8    /* FluidSolver::transferVelocityToParticlesPICFLIP, src/FluidSolver.cpp:945-963 */
#define FS_PH_G2P_PIC 9        /* FluidSolver::transferVelocityToParticlesPIC, src/FluidSolver.cpp:921-931 */
#define FS_PH_G2P_FLIP 10      /* FluidSolver::transferVelocityToParticlesFLIP, src/FluidSolver.cpp:933-943 */
#define FS_PH_ADVECT_SAFE 11   /* MarkerParticleSet::advectAndEnsureOutsideObstacles, src/MarkerParticleSet.cpp:48-62 */
#define FS_PH_ADVECT 12        /* MarkerParticleSet::advect, src/MarkerParticleSet.cpp:40-46 */
#define FS_PH_SL_VELOCITY 13   /* FluidSolver::advectVelocitySemiLagrangian, src/FluidSolver.cpp:709-772 */
#define FS_PH_SL_PARTICLES 14  /* FluidSolver::advectParticlesWithGrid, src/FluidSolver.cpp:774-791 */
#define FS_PH_SWAP 15          /* MacGrid::swapVelocityBuffers, src/MacGrid.cpp:89-93 */

/* Precision of the CG dot products.  FS_CG_FLOAT sums float products in
 * float, the precision of the reference's Eigen::ConjugateGradient over
 * VectorXf; FS_CG_DOUBLE sums exact float*float products in double.  Both use
 * one fixed summation order, so results are reproducible run to run. */
#define FS_CG_FLOAT 0
#define FS_CG_DOUBLE 1
/* Double-single: each float*float product exact as a pair of floats (product
 * and its fmaf error), the 32 products of each warp summed in such pairs
 * (TwoSum of the high parts, the low parts added to its error), every level
 * above in double;
 * no counterpart in the reference.  Steps and fs_poisson_solve's inner CG;
 * not batches. */
#define FS_CG_DS 2

/* Timed phases reported in fs_step_stats.ms_phase when timing is enabled. */
#define FS_T_CLASSIFY 0   /* labels */
#define FS_T_P2G 1        /* particle-to-grid transfer (+ previous-velocity copy) */
#define FS_T_FORCES 2     /* gravity, Dirichlet, velocity extension, semi-Lagrangian advection */
#define FS_T_ASSEMBLY 3   /* particle counts, fluid indexing, divergence and matrix rows */
#define FS_T_CG 4         /* the conjugate-gradient kernel */
#define FS_T_PROJECT 5    /* pressure-gradient update, second Dirichlet, velocity difference */
#define FS_T_G2P 6        /* grid-to-particle transfer and particle advection */
#define FS_NUM_TIMED 7

typedef struct fs_config
{
    int size_x, size_y;           /* cells */
    float length_x, length_y;     /* world size; delta = length / size */
    float density;                /* FluidDomain density (the projection scales by dt / density) */
    float pic_ratio;              /* FluidDomain pic_ratio in [0, 1] */
    float gravity_x, gravity_y;   /* reference: (0, -9.82), src/FluidSolver.cpp:232 */
    int cg_max_iterations;        /* reference: 100, src/FluidSolver.cpp:81 */
    double cg_tolerance;          /* reference: FLT_EPSILON (Eigen's default) */
    int extension_iterations;     /* reference: 2, src/FluidSolver.cpp:234 */
    int device;                   /* CUDA device ordinal */
    int cg_precision;             /* FS_CG_FLOAT (default) or FS_CG_DOUBLE */
    int reserved[7];
} fs_config;

typedef struct fs_step_stats
{
    int cg_iterations;      /* CG updates performed in the last pressure solve */
    int n_fluid;            /* fluid (LIQUID) cells in the last pressure solve */
    double cg_residual;     /* ||r|| / ||b|| at exit */
    unsigned int warnings;  /* FS_WARN_* bits accumulated since the last query */
    float ms_total;         /* device time of the last fs_step (timing enabled) */
    float ms_phase[FS_NUM_TIMED];
} fs_step_stats;

typedef struct fs_handle fs_handle;

/* Fills *cfg with the reference's defaults for a size_x x size_y grid of
 * unit cells: density 1, pic_ratio 0, gravity (0, -9.82), CG maxit 100,
 * tolerance FLT_EPSILON, 2 extension sweeps, device 0. */
FS_API void fs_config_init(fs_config* cfg, int size_x, int size_y);

/* Creates a domain + solver pair on cfg->device (FluidDomain ctor,
 * FluidSolverMemoryPool(const FluidDomain&), FluidSolver(pool)). */
FS_API int fs_create(const fs_config* cfg, fs_handle** out);
FS_API int fs_destroy(fs_handle* h);

/* Message of the last failure on h, or of the last fs_create failure on this
 * thread when h is NULL. */
FS_API const char* fs_last_error(const fs_handle* h);

/* Settings that the reference hard-codes or keeps on FluidDomain. */
FS_API int fs_set_pic_ratio(fs_handle* h, float pic_ratio); /* FluidDomain::setPicRatio: clamps to [0, 1] */
FS_API int fs_set_gravity(fs_handle* h, float gx, float gy);
FS_API int fs_set_cg(fs_handle* h, double tolerance, int max_iterations);
FS_API int fs_set_cg_precision(fs_handle* h, int precision);
FS_API int fs_set_extension_iterations(fs_handle* h, int n);
/* Pressure solver of the step.  FS_SOLVER_JACOBI_PCG (default): the
 * reference's Jacobi-preconditioned CG, bit-exact.  FS_SOLVER_MGPCG: CG
 * preconditioned by a geometric multigrid V-cycle on the same system, to the
 * same relative residual -- far fewer iterations, a different converged
 * pressure (not the reference's result); steps with it are direct launches. */
#define FS_SOLVER_JACOBI_PCG 0
#define FS_SOLVER_MGPCG 1
FS_API int fs_set_pressure_solver(fs_handle* h, int solver);
/* Persistent solid cells re-applied after every classification (extension;
 * the reference re-labels only the border).  mask: size_x*size_y bytes,
 * non-zero = solid; NULL clears. */
FS_API int fs_set_solid_mask(fs_handle* h, const uint8_t* mask);

/* Marker particles (MarkerParticleSet, include/MarkerParticleSet.h:53-78). */
FS_API int fs_set_particles(fs_handle* h, const float* xyuv, int64_t n);
FS_API int fs_set_particles_device(fs_handle* h, const float* d_xyuv, int64_t n);
FS_API int fs_add_particles(fs_handle* h, const float* xyuv, int64_t n);
FS_API int fs_num_particles(fs_handle* h, int64_t* n);
FS_API int fs_get_particles(fs_handle* h, float* xyuv, int64_t n);
FS_API int fs_get_particles_device(fs_handle* h, float* d_xyuv, int64_t n);

/* Grid state (host copies). */
FS_API int fs_get_grid(fs_handle* h, int which, float* out);
FS_API int fs_set_grid(fs_handle* h, int which, const float* in);
FS_API int fs_get_labels(fs_handle* h, uint8_t* out);
FS_API int fs_set_labels(fs_handle* h, const uint8_t* in);
FS_API int fs_get_fluid_indices(fs_handle* h, int32_t* out);
FS_API int fs_get_particle_counts(fs_handle* h, uint8_t* out);
/* Pressure of the last solve scattered to the grid by fluid index (0 elsewhere). */
FS_API int fs_get_pressure(fs_handle* h, float* out);

/* One step of the given method (FS_STEP_*), queued on the handle's stream. */
FS_API int fs_step(fs_handle* h, int method, float dt);
/* One phase (FS_PH_*), queued on the handle's stream. */
FS_API int fs_phase(fs_handle* h, int phase, float dt);
/* Waits for queued work; reports device-side failures (FS_ERR_TIMEOUT ...). */
FS_API int fs_synchronize(fs_handle* h);
/* Synchronises and returns the statistics of the last step / pressure solve. */
FS_API int fs_get_stats(fs_handle* h, fs_step_stats* out);

/* Per-phase CUDA-event timing of fs_step (off by default). */
FS_API int fs_set_timing(fs_handle* h, int enable);
/* Replays fs_step through a cached CUDA graph of the whole step (default
 * on); 0 launches kernel by kernel. */
FS_API int fs_set_graphs(fs_handle* h, int enable);
/* The handle's CUDA stream (cudaStream_t) and a way to replace it. */
FS_API void* fs_get_stream(fs_handle* h);
FS_API int fs_set_stream(fs_handle* h, void* stream);
/* Test hook of the failure path: the next solves' grid barriers wait for
 * missing_arrivals CTAs that do not exist, each wait bounded by
 * wait_limit_seconds (0 < limit <= 10; normally 2).  Every CTA then gives up,
 * the solve ends early, and fs_synchronize / fs_get_stats return
 * FS_ERR_TIMEOUT; the handle stays usable.  (0, 2.0) is normal operation.
 * Solves of at most 16 chunks of 1024 fluid cells run in one CTA and have no
 * grid barrier. */
FS_API int fs_debug_set_cg_barrier_fault(fs_handle* h, int missing_arrivals, double wait_limit_seconds);

/* Number of this library's kernel launches queued so far on h. */
FS_API int64_t fs_kernel_launches(fs_handle* h);

/* Fluid sources on the device: FluidDomain::addFluidSource / update /
 * clearFluidSources / resetParticleSet (src/FluidDomain.cpp:3-52,75-97).  A
 * source spawns, every time_step of accumulated dt and at most max_spawns
 * times (-1: unlimited), a lattice of spacing delta / 2.5 over
 * [x_min, x_max) x [y_min, y_max) with velocity (x_velocity, y_velocity),
 * appended in the reference's loop order (y outer, x inner, float-accumulated
 * coordinates).  The lattice is written by a kernel into device memory: no
 * particle crosses the host.  A lattice whose increment cannot advance its
 * coordinate (the reference would loop forever) is FS_ERR_INVALID_ARGUMENT. */
FS_API int fs_add_fluid_source(fs_handle* h, float x_min, float x_max, float y_min, float y_max, float delta_x,
                               float delta_y, float x_velocity, float y_velocity, float time_step, int max_spawns);
FS_API int fs_update(fs_handle* h, float dt);
FS_API int fs_clear_fluid_sources(fs_handle* h);
FS_API int fs_num_fluid_sources(fs_handle* h, int* n);
/* The timing state of source `index` (in order of addition), for a FluidSource
 * copy that was already updated: its time since the last spawn and spawns so far. */
FS_API int fs_set_fluid_source_state(fs_handle* h, int index, float time_since_last, int n_spawns);
FS_API int fs_reset_particles(fs_handle* h);

/* The level-set path the reference keeps beside the particle labelling
 * (FluidDomain::levelSet / advectLevelSet / classifyCells(LevelSet&),
 * src/FluidDomain.cpp:104-148, src/LevelSet.cpp): the level set is
 * size_x * size_y floats, zero at creation.  The advection follows the
 * reference as written (loops over j < size_x, i < size_y; velocities through
 * the linear index); where the reference reads past the end of its arrays
 * (the last row) the read is 0 here.  Classification leaves a SOLID border,
 * LIQUID where the level set is negative, AIR elsewhere, then applies the
 * persistent solid mask. */
FS_API int fs_get_level_set(fs_handle* h, float* out);
FS_API int fs_set_level_set(fs_handle* h, const float* in);
FS_API int fs_advect_level_set(fs_handle* h, float dt);
FS_API int fs_classify_level_set(fs_handle* h);

/* Snapshots: a device copy of a handle's simulation state -- the eight
 * velocity grids, labels, extension masks, fluid indices, particle counts,
 * pressure, particles, the last CG result and warnings, buffer parities and
 * the fluid sources' timing state (settings are not part of it).  fs_restore
 * puts it back into the same handle; it fails if sources were added or
 * cleared in between.  A snapshot holds device memory until destroyed. */
typedef struct fs_saved_state fs_saved_state;
FS_API int fs_snapshot(fs_handle* h, fs_saved_state** out);
FS_API int fs_restore(fs_handle* h, const fs_saved_state* snap);
FS_API int fs_snapshot_destroy(fs_saved_state* snap);

/* Headless renderer: Renderer (src/Renderer.cpp) drawing a handle's state
 * onto a Canvas (src/Canvas.cpp) of width * height RGB floats in device
 * memory, bit-identical to the reference's CPU drawing.  A new canvas is
 * white with a black line colour and a white fill colour, as Canvas(w, h).
 * area = {x_min, x_max, y_min, y_max}, the world rectangle of Renderer(area).
 * Passes: FS_RENDER_CLEAR (clearCanvas), FS_RENDER_CELLS
 * (renderGridCellsToCanvas), FS_RENDER_VELOCITIES (renderGridVelocitiesToCanvas),
 * FS_RENDER_PARTICLES (renderParticlesToCanvas), FS_RENDER_METABALLS
 * (renderMetaBallsToCanvas); each draws over what the canvas holds and leaves
 * the line / fill colours the reference leaves.  fs_render returns after the
 * pass; pixels are rows of {r, g, b} floats. */
#define FS_RENDER_CLEAR 0
#define FS_RENDER_CELLS 1
#define FS_RENDER_VELOCITIES 2
#define FS_RENDER_PARTICLES 3
#define FS_RENDER_METABALLS 4
#define FS_RENDER_LEVEL_SET 5 /* renderLevelSetFunctionValuesToCanvas */

typedef struct fs_canvas fs_canvas;
FS_API int fs_canvas_create(int width, int height, int device, fs_canvas** out);
FS_API int fs_canvas_destroy(fs_canvas* c);
/* NULL c: the message of the last failed fs_canvas_create on this thread. */
FS_API const char* fs_canvas_last_error(const fs_canvas* c);
FS_API int fs_canvas_set_pixels(fs_canvas* c, const float* rgb);
FS_API int fs_canvas_get_pixels(fs_canvas* c, float* rgb);
FS_API int fs_canvas_set_colors(fs_canvas* c, const float* line_rgb, const float* fill_rgb);
FS_API int fs_canvas_get_colors(fs_canvas* c, float* line_rgb, float* fill_rgb);
/* Renderer::writeCanvasToPpm's bytes: CLAMP(c, 0, 1) * 255 truncated, 3 per pixel. */
FS_API int fs_canvas_get_bytes(fs_canvas* c, uint8_t* rgb8);
/* Renderer::writeCanvasToPpm: a binary PPM (P6) of those bytes. */
FS_API int fs_canvas_write_ppm(fs_canvas* c, const char* path);
FS_API int64_t fs_canvas_kernel_launches(const fs_canvas* c);
FS_API int fs_render(fs_handle* h, fs_canvas* c, int what, const float* area);

/* Pressure projection alone (no particles): the
 * Poisson system of FluidSolver::pressureSolve (src/FluidSolver.cpp:363-425)
 * built from a label grid (FS_LIQUID = unknown, FS_AIR = pressure 0,
 * FS_SOLID = wall), with a double right-hand side per cell, solved by
 *   FS_POISSON_FP32   the step's CG: float vectors, dots per inner_precision;
 *   FS_POISSON_FP64   CG with double vectors, SpMV and dots;
 *   FS_POISSON_MIXED  FP64 iterative refinement (x and b - A x in double)
 *                     around float-vector CG corrections solved to
 *                     inner_tolerance.
 * tolerance is the relative residual ||b - A x|| / ||b|| (for MIXED and FP64
 * measured in double; for FP32 in the CG's own precision).  A fluid
 * component with no AIR neighbour is singular: its right-hand side must sum
 * to zero. */
#define FS_POISSON_FP32 0
#define FS_POISSON_FP64 1
#define FS_POISSON_MIXED 2
/* Not the reference's method: CG preconditioned by a geometric multigrid
 * V-cycle on the cell grid (float vectors, double dot products); far fewer
 * iterations than the Jacobi-preconditioned CG, a different converged x. */
#define FS_POISSON_MGPCG 3
/* FS_POISSON_MIXED with multigrid-preconditioned float corrections. */
#define FS_POISSON_MIXED_MG 4

typedef struct fs_poisson fs_poisson;
typedef struct fs_poisson_stats
{
    int outer_iterations;  /* refinement steps (1 for FP32 / FP64) */
    int inner_iterations;  /* CG updates in total */
    double residual;       /* final ||b - A x|| / ||b||, evaluated in double */
    float ms;              /* device time of the solve */
} fs_poisson_stats;

FS_API int fs_poisson_create(int size_x, int size_y, float length_x, float length_y, int device, fs_poisson** out);
FS_API int fs_poisson_destroy(fs_poisson* p);
/* labels and rhs: host arrays of size_x * size_y (row-major); rhs is read on LIQUID cells. */
FS_API int fs_poisson_set_problem(fs_poisson* p, const uint8_t* labels, const double* rhs);
FS_API int fs_poisson_solve(fs_poisson* p, int method, double tolerance, int max_iterations, double inner_tolerance,
                            int inner_precision, fs_poisson_stats* stats);
/* The solution on every cell (0 outside fluid), host array of doubles. */
FS_API int fs_poisson_get_solution(fs_poisson* p, double* out);
FS_API int64_t fs_poisson_kernel_launches(const fs_poisson* p);

/* A batch of independent simulations stepped together (no counterpart in the
 * reference, whose caller would loop over FluidSolver/FluidDomain pairs,
 * src/FluidSolver.cpp:211-251, include/FluidDomain.h:40-64).  Simulation s is
 * configured by cfgs[s] exactly like fs_create; sizes may differ.  Batch-wide
 * settings come from cfgs[0]: device, extension_iterations, cg_precision.
 * Each simulation's results are bit-identical to stepping it alone through a
 * handle.  Limits: at most 65536 interior cells ((size_x-2) * (size_y-2)) per
 * simulation and 16 Mi cells in total (FS_ERR_TOO_LARGE).
 *
 * Particles set with fs_batch_set_particles are laid out on the device at the
 * next step or particle read.  fs_batch_step runs every simulation's
 * FluidSolver::step* once, as one CUDA graph (captured on first use per
 * method, dt and particle layout).  The pressure solves run one thread-block
 * cluster per simulation; fs_batch_tune times whole steps for each cluster
 * plan (1, 2, 4 or 8 chunks of 1024 fluid cells per CTA), keeps the fastest
 * and leaves the state as it found it (ms_out: 4 floats or NULL). */
typedef struct fs_batch fs_batch;

FS_API int fs_batch_create(int n, const fs_config* cfgs, fs_batch** out);
FS_API int fs_batch_destroy(fs_batch* b);
/* NULL b: the message of the last failed fs_batch_create on this thread. */
FS_API const char* fs_batch_last_error(const fs_batch* b);
FS_API int fs_batch_size(const fs_batch* b);
/* AoS {x, y, vx, vy} float quadruples, as fs_set_particles. */
FS_API int fs_batch_set_particles(fs_batch* b, int sim, const float* xyuv, int64_t n);
FS_API int fs_batch_num_particles(fs_batch* b, int sim, int64_t* n);
FS_API int fs_batch_get_particles(fs_batch* b, int sim, float* xyuv, int64_t n);
/* size_x * size_y uint8 of simulation sim (non-zero = solid), or NULL to clear. */
FS_API int fs_batch_set_solid_mask(fs_batch* b, int sim, const uint8_t* mask);
FS_API int fs_batch_get_grid(fs_batch* b, int sim, int which, float* out);
FS_API int fs_batch_get_labels(fs_batch* b, int sim, uint8_t* out);
FS_API int fs_batch_get_pressure(fs_batch* b, int sim, float* out);
FS_API int fs_batch_step(fs_batch* b, int method, float dt);
FS_API int fs_batch_synchronize(fs_batch* b);
/* CG iterations, residual, fluid cells and warnings of simulation sim's last
 * pressure solve (ms fields are 0). */
FS_API int fs_batch_get_stats(fs_batch* b, int sim, fs_step_stats* out);
FS_API int fs_batch_tune(fs_batch* b, int method, float dt, int steps, float* ms_out);
/* Plans clusters of chunks_per_cta (1, 2, 4 or 8) chunks per CTA without
 * timing: after a step, for the fluid cells that step counted (plus the
 * tuner's 25% margin), before any step for each simulation's interior. */
FS_API int fs_batch_set_tuning(fs_batch* b, int chunks_per_cta);
FS_API int fs_batch_get_tuning(const fs_batch* b);
FS_API int fs_batch_set_graphs(fs_batch* b, int enable);
FS_API void* fs_batch_get_stream(fs_batch* b);
FS_API int64_t fs_batch_kernel_launches(fs_batch* b);

/* Differentiable smoke (no counterpart in the reference, whose
 * semi-Lagrangian step scatters, src/FluidSolver.cpp:709-772): a passive
 * density and the velocity advected by gathering semi-Lagrangian steps
 * (bilinear sampling as Grid::valueInterpolated, include/Grid.h:117-144;
 * back-trace by explicit Euler, the midpoint rule or RK3 as
 * include/OdeSolver.h:102-113), faces touching a solid cell closed, then the
 * pressure projection (FluidSolver::pressureSolve's matrix, solved by
 * projection_method to cg_tolerance).  The grid has a solid border.
 * fs_smoke_forward runs `steps` steps from the state of fs_smoke_set_state
 * and returns L = ||density - target||_2; fs_smoke_backward returns dL/d(the
 * initial u, v, density) from a hand-written adjoint, recomputing the states
 * between checkpoints stored every checkpoint_every steps.  Fields are float
 * or double on the device (precision); adjoints are double, each node adding
 * its contributions in a fixed order, so gradients repeat to the bit.  Host
 * arrays are size_x * size_y doubles, row-major: u(i, j) on the face at
 * (i h, (j + 1/2) h), v(i, j) at ((i + 1/2) h, j h), density at cell centres. */
#define FS_INTEGRATOR_EULER 0
#define FS_INTEGRATOR_RK2 1
#define FS_INTEGRATOR_RK3 2
#define FS_SMOKE_FP32 0
#define FS_SMOKE_FP64 1
/* float fields whose back-traces (positions, footprints, samples) run in double */
#define FS_SMOKE_FP32_TRACE64 2

typedef struct fs_smoke fs_smoke;
typedef struct fs_smoke_config
{
    int size_x, size_y;
    float length_x, length_y;  /* square cells: length_x / size_x == length_y / size_y */
    float dt;
    int integrator;            /* FS_INTEGRATOR_* */
    int precision;             /* FS_SMOKE_FP32 / FS_SMOKE_FP64 / FS_SMOKE_FP32_TRACE64 */
    int projection_method;     /* FS_POISSON_* (FS_POISSON_MIXED_MG: multigrid-preconditioned corrections) */
    double cg_tolerance;       /* relative residual of each projection */
    int cg_max_iterations;
    double inner_tolerance;    /* FS_POISSON_MIXED(_MG): tolerance of each float correction */
    int checkpoint_every;      /* steps between stored states */
    int device;
    int reserved[8];
} fs_smoke_config;

/* Defaults: unit cells, dt 0.01, RK2, FP32 fields, mixed-precision projection
 * to 1e-10, checkpoints every 8 steps. */
FS_API void fs_smoke_config_init(fs_smoke_config* c, int size_x, int size_y);
FS_API int fs_smoke_create(const fs_smoke_config* cfg, fs_smoke** out);
FS_API int fs_smoke_destroy(fs_smoke* s);
/* NULL s: the message of the last failed fs_smoke_create on this thread. */
FS_API const char* fs_smoke_last_error(const fs_smoke* s);
/* size_x * size_y uint8 (non-zero = solid) added to the solid border, or NULL. */
FS_API int fs_smoke_set_solid_mask(fs_smoke* s, const uint8_t* mask);
FS_API int fs_smoke_set_state(fs_smoke* s, const double* u, const double* v, const double* density);
FS_API int fs_smoke_set_target(fs_smoke* s, const double* target);
FS_API int fs_smoke_forward(fs_smoke* s, int steps, double* loss);
/* The state after the last fs_smoke_forward. */
FS_API int fs_smoke_get_state(fs_smoke* s, double* u, double* v, double* density);
FS_API int fs_smoke_backward(fs_smoke* s, double* grad_u, double* grad_v, double* grad_density);
FS_API int64_t fs_smoke_kernel_launches(const fs_smoke* s);

/* Allocation-free pressure solve.  No counterpart in the reference: this is
 * FluidSolver::pressureSolve's fluid indexing, assembly and conjugate gradient
 * for callers that cannot allocate device memory -- an application that owns
 * all device memory and forbids cudaMalloc/cudaFree once running (a real-time
 * frame loop, where an allocation can stall the device), or a plugin living
 * in a host application's fixed memory budget.  Such callers cannot use
 * fs_create, which allocates every grid of a handle.
 *
 * Inputs are device pointers to size_x * size_y cells: labels (FS_LIQUID /
 * FS_AIR / FS_SOLID with a SOLID border, as classification leaves them) and
 * the front velocities u, v; the output is the pressure of every cell
 * (0 outside fluid), as fs_get_pressure reports after FS_PH_PRESSURE.  The
 * velocity update is left to the caller.  Work is queued on `stream`
 * (cudaStream_t, NULL = default stream) and the call synchronises that
 * stream before it returns, so that its return code reports a failure on
 * the device (FS_ERR_TIMEOUT, FS_ERR_TOO_LARGE) as well as on the host;
 * cg_iterations and cg_residual may be NULL.
 *
 * Limit: size_x * size_y <= 16384 cells (e.g. 128 x 128); larger grids
 * return FS_ERR_TOO_LARGE.  All scratch lives in one static device array of
 * about 0.75 MB that every GPU loading this library holds until exit.  The
 * first call on a device looks up that array's address (cudaGetSymbolAddress)
 * and must come before any stream capture; the address is kept for the life
 * of the process, so a device reset (cudaDeviceReset) ends the use of this
 * entry point on that device.  Calls share the array: calls whose work
 * overlaps on the GPU race.  Messages go to fs_last_error(NULL). */
FS_API int fs_pressure_solve_noalloc(int size_x, int size_y, float length_x, float length_y,
                                     const uint8_t* labels, const float* u, const float* v,
                                     double cg_tolerance, int cg_max_iterations, int cg_precision,
                                     float* pressure, int* cg_iterations, double* cg_residual,
                                     void* stream);

#ifdef __cplusplus
}
#endif

#endif
