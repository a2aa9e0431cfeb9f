/* Oracle API: one C interface with two implementations, used only by the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
 *
 *   oracle/fs_oracle.c     -> oracle/_build/libfsoracle.so
 *       A plain-C restatement of the reference's per-step algorithm
 *       (kbladin/Fluid_Simulation src/FluidSolver.cpp, src/FluidDomain.cpp,
 *       src/MacGrid.cpp, src/MarkerParticleSet.cpp, include/Grid.h,
 *       include/MacGrid.h, include/OdeSolver.h), function by function.
 *   oracle/ref_harness.cpp -> oracle/_ref/libfsref.so
 *       The reference's own sources compiled unmodified against the
 *       project's Eigen-subset stand-in (oracle/eigen_shim), driven through
 *       their public and private methods.
 *
 * Both are test infrastructure: the GPU library never links or calls them.
 * Grids are row-major, index i + j * nx (Grid.h:63-67); particles are
 * interleaved {pos_x, pos_y, vel_x, vel_y} floats (MarkerParticleSet.h:43-50).
 */
#ifndef FS_ORACLE_H
#define FS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fso_sim fso_sim;

/* CellType values, MacGrid.h:14-17. */
enum { FSO_LIQUID = 0, FSO_AIR = 1, FSO_SOLID = 2 };

/* Velocity grids of MacGrid (MacGrid.h:164-176). */
enum {
    FSO_U_FRONT = 0,
    FSO_V_FRONT = 1,
    FSO_U_BACK = 2,
    FSO_V_BACK = 3,
    FSO_U_PREV = 4,
    FSO_V_PREV = 5,
    FSO_U_DIFF = 6,
    FSO_V_DIFF = 7
};

/* FluidSolver::step* (FluidSolver.h:51-54). */
enum {
    FSO_STEP_SEMI_LAGRANGIAN = 0,
    FSO_STEP_PIC = 1,
    FSO_STEP_FLIP = 2,
    FSO_STEP_PICFLIP = 3
};

/* Single phases of a step, in the reference's own function granularity. */
enum {
    FSO_PH_CLASSIFY = 0,        /* FluidDomain::classifyCells(MarkerParticleSet&) + solid mask */
    FSO_PH_P2G = 1,             /* FluidSolver::transferVelocityToGridSpread */
    FSO_PH_SAVE_PREV = 2,       /* MacGrid::updatePreviousVelocityBuffer */
    FSO_PH_GRAVITY = 3,         /* FluidSolver::addExternalAcceleration(gx, gy, dt) */
    FSO_PH_DIRICHLET = 4,       /* FluidSolver::enforceDirichlet */
    FSO_PH_EXTEND = 5,          /* FluidSolver::extendVelocityIndividual(n) */
    FSO_PH_PRESSURE = 6,        /* FluidSolver::pressureSolve */
    FSO_PH_SAVE_DIFF = 7,       /* MacGrid::updateVelocityDiffBuffer */
    FSO_PH_G2P_PICFLIP = 8,     /* FluidSolver::transferVelocityToParticlesPICFLIP */
    FSO_PH_G2P_PIC = 9,         /* FluidSolver::transferVelocityToParticlesPIC */
    FSO_PH_G2P_FLIP = 10,       /* FluidSolver::transferVelocityToParticlesFLIP */
    FSO_PH_ADVECT_SAFE = 11,    /* MarkerParticleSet::advectAndEnsureOutsideObstacles */
    FSO_PH_ADVECT = 12,         /* MarkerParticleSet::advect */
    FSO_PH_SL_VELOCITY = 13,    /* FluidSolver::advectVelocitySemiLagrangian */
    FSO_PH_SL_PARTICLES = 14,   /* FluidSolver::advectParticlesWithGrid */
    FSO_PH_SWAP = 15            /* MacGrid::swapVelocityBuffers */
};

fso_sim* fso_create(int size_x, int size_y, float length_x, float length_y, float density,
                    float pic_ratio);
void fso_destroy(fso_sim* s);

/* Pressure-solve settings; the reference fixes maxit = 100 (FluidSolver.cpp:81)
 * and leaves the tolerance at machine epsilon. */
void fso_set_cg(fso_sim* s, double tolerance, int max_iterations);
/* Precision of the CG dot products: 0 = float (the reference's, default),
 * 1 = double (exact products summed in double).  Same fixed summation tree
 * either way.  In the reference build the setting is process-wide. */
void fso_set_cg_precision(fso_sim* s, int precision);
/* Gravity; the reference hard-codes (0, -9.82) (FluidSolver.cpp:232). */
void fso_set_gravity(fso_sim* s, float gx, float gy);
/* Extension sweeps; the reference hard-codes 2 (FluidSolver.cpp:234). */
void fso_set_extension_iterations(fso_sim* s, int n);
/* Persistent solid cells, re-marked after every classification (an
 * extension: the reference re-labels only the border, FluidDomain.cpp:169-179).
 * NULL clears the mask. */
void fso_set_solid_mask(fso_sim* s, const uint8_t* mask);
/* 1 (default): run the reference's own step functions when no extension is
 * in use; 0: always run the phase sequence with the extensions applied. */
void fso_set_use_stock(fso_sim* s, int use_stock);
void fso_set_pic_ratio(fso_sim* s, float pic_ratio); /* FluidDomain::setPicRatio */

void fso_set_particles(fso_sim* s, const float* xyuv, int64_t n);
int64_t fso_num_particles(const fso_sim* s);
void fso_get_particles(const fso_sim* s, float* xyuv);

void fso_get_grid(const fso_sim* s, int which, float* out);
void fso_set_grid(fso_sim* s, int which, const float* in);
void fso_get_labels(const fso_sim* s, uint8_t* out);
void fso_set_labels(fso_sim* s, const uint8_t* in);
void fso_get_fluid_indices(const fso_sim* s, int32_t* out);
void fso_get_particle_counts(const fso_sim* s, uint8_t* out);
/* Last pressure solution, scattered to the grid by fluid index (0 elsewhere). */
void fso_get_pressure(const fso_sim* s, float* out);
void fso_get_cg_stats(const fso_sim* s, int* iterations, double* error, int* n_fluid);

/* Returns 0, or -1 when the reference would throw (FluidSolver.cpp:215-221). */
int fso_step(fso_sim* s, int method, float dt);
int fso_phase(fso_sim* s, int phase, float dt);

/* FluidSource / FluidDomain::update (FluidDomain.cpp:3-52, 80-87). */
void fso_add_source(fso_sim* s, float x_min, float x_max, float y_min, float y_max, float delta_x,
                    float delta_y, float x_velocity, float y_velocity, float time_step,
                    int max_spawns);
void fso_update(fso_sim* s, float dt);
/* FluidDomain::clearFluidSources (FluidDomain.cpp:89-92). */
void fso_clear_sources(fso_sim* s);

/* Pressure projection alone (the GPU's fs_poisson_*), restatement only:
 * method 0 float CG (dots per inner_precision), 1 double CG, 2 double
 * iterative refinement around float CG corrections solved to inner_tol.
 * x_out: size_x * size_y doubles (0 outside fluid).  Returns the fluid count. */
int fso_poisson_solve(int size_x, int size_y, float length_x, float length_y, const uint8_t* labels,
                      const double* rhs, int method, double tol, int max_iterations, double inner_tol,
                      int inner_precision, double* x_out, int* outer_iterations, int* inner_iterations,
                      double* residual);

/* Name of the implementation ("restatement" or "reference"). */
const char* fso_kind(void);

/* Renderer (Renderer.cpp) onto a canvas given as w * h RGB floats (row-major,
 * in/out) and its line / fill colours (colors[0..2], colors[3..5], in/out);
 * area = {x_min, x_max, y_min, y_max} in world units. */
enum { FSO_RENDER_CLEAR = 0, FSO_RENDER_CELLS = 1, FSO_RENDER_VELOCITIES = 2, FSO_RENDER_PARTICLES = 3,
       FSO_RENDER_METABALLS = 4, FSO_RENDER_LEVEL_SET = 5 };
void fso_render(fso_sim* s, int what, const float* area, int w, int h, float* rgb, float* colors);
/* The level set (FluidDomain::levelSet, LevelSet.h), size_x * size_y floats. */
void fso_get_level_set(const fso_sim* s, float* out);
void fso_set_level_set(fso_sim* s, const float* in);
/* FluidDomain::advectLevelSet (FluidDomain.cpp:104-125). */
void fso_advect_level_set(fso_sim* s, float dt);
/* FluidDomain::classifyCells(LevelSet&) (FluidDomain.cpp:127-148). */
void fso_classify_level_set(fso_sim* s);
/* Renderer::writeCanvasToPpm's byte conversion of n RGB pixels. */
void fso_canvas_bytes(const float* rgb, int64_t n, uint8_t* out);
/* renderMetaBallsToCanvas's weight of pixel offset (i, j), i, j in [-5, 5). */
float fso_metaball_weight(int i, int j);

#ifdef __cplusplus
}
#endif

#endif
