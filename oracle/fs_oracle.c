/* CPU restatement of the reference's per-step algorithm (test infrastructure).
 *
 * This file restates, function by function, the hot path of
 * kbladin/Fluid_Simulation in plain C with the reference's exact float
 * evaluation order, so that the GPU library can be checked against it bit for
 * bit on machines where the reference itself cannot be built.  It is pinned
 * against the reference's own code (oracle/ref_harness.cpp, the same C API)
 * by tests/test_oracle_vs_reference.py and by the committed fixtures in
 * tests/golden/.  Only the tests, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it; the GPU library never links or calls it.
 *
 * Floating point: compile with -ffp-contract=off (no FMA contraction) and
 * without -ffast-math.  Expressions that the reference writes with double
 * literals on float operands (e.g. `y - _DELTA_Y * 0.5`, MacGrid.h:69) are
 * written the same way here.
 *
 * The pressure solve's conjugate gradient lives in Eigen in the reference
 * (absent here, unpinned version); it is restated as the published
 * Jacobi-preconditioned CG with the floating-point discipline documented in
 * oracle/eigen_shim/Eigen/fs_shim_core.h, which this file mirrors exactly.
 */
#include "fs_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct
{
    float x_min, x_max, y_min, y_max;
    float vx, vy, dx, dy, time_step, time_since_last;
    int max_spawns, n_spawns;
} fso_source;

struct fso_sim
{
    int nx, ny;
    float dx, dy;         /* GridInterface deltas: length / size (FluidDomain.cpp:62) */
    float lx, ly;         /* GridInterface::lengthX(): size * delta (Grid.h:90-91) */
    float pool_dy;        /* the solver's pool keeps dx for dy (FluidSolver.cpp:56-62) */
    float density, pic;
    float gx, gy;
    int n_ext;
    double cg_tol;
    int cg_maxit;
    int cg_double;        /* dot-product precision: 0 float, 1 double, 2 double-single */
    int use_stock;

    float* u[2];
    float* v[2];
    int front;            /* index of the front buffer in u[] / v[] */
    float *u_prev, *v_prev, *u_diff, *v_diff;
    uint8_t* labels;
    uint8_t* solid;       /* NULL when no persistent mask */
    int32_t* fidx;
    uint8_t* counts;
    uint8_t* vmask_x[2];
    uint8_t* vmask_y[2];
    int vfront;           /* index of the front valid-mask buffers */
    float *sum_u, *sum_v, *w_u, *w_v;

    float* level_set;     /* FluidDomain::_level_set (LevelSet.cpp:3-13: zero) */

    float* part;          /* {x, y, vx, vy} per particle */
    int64_t n_part, cap_part;

    float* pressure;      /* by fluid index */
    int cg_iters;
    double cg_error;
    int n_fluid;

    fso_source* src;
    int n_src, cap_src;

    /* CG scratch */
    float *cg_b, *cg_x, *cg_r, *cg_p, *cg_q, *cg_z, *cg_diag, *cg_inv;
    int32_t *cg_down, *cg_up, *cg_left, *cg_right;
    uint8_t* cg_nns;      /* non-solid neighbours of each fluid cell */
    double* cg_acc;
    float* cg_accf;
};

#define IDX(s, i, j) ((size_t)(i) + (size_t)(j) * (size_t)(s)->nx)
#define UF(s) ((s)->u[(s)->front])
#define VF(s) ((s)->v[(s)->front])
#define UB(s) ((s)->u[1 - (s)->front])
#define VB(s) ((s)->v[1 - (s)->front])

const char* fso_kind(void) { return "restatement"; }

/* MathDefinitions.h:16-19: CLAMP takes and returns MyFloat (float). */
static inline float clampf_ref(float d, float lo, float hi)
{
    const float t = d < lo ? lo : d;
    return t > hi ? hi : t;
}
static inline int clampi_ref(int d, int lo, int hi) { return (int)clampf_ref((float)d, (float)lo, (float)hi); }

/* MacGrid::cellType (MacGrid.h:92-97): clamped lookup. */
static inline uint8_t cell_type(const fso_sim* s, int i, int j)
{
    i = clampi_ref(i, 0, s->nx - 1);
    j = clampi_ref(j, 0, s->ny - 1);
    return s->labels[IDX(s, i, j)];
}

/* Grid::valueInterpolated (Grid.h:117-144).  Note the +1 neighbour is formed
 * after clamping here (unlike addToValueInterpolated). */
static float value_interp(const fso_sim* s, const float* g, float gdx, float gdy, float x, float y)
{
    int i = (int)(x / gdx);
    int j = (int)(y / gdy);
    float i_frac = x / gdx - (float)i;
    float j_frac = y / gdy - (float)j;
    i = clampi_ref(i, 0, s->nx - 1);
    j = clampi_ref(j, 0, s->ny - 1);
    int i1 = clampi_ref(i + 1, 0, s->nx - 1);
    int j1 = clampi_ref(j + 1, 0, s->ny - 1);
    float v00 = g[IDX(s, i, j)];
    float v10 = g[IDX(s, i1, j)];
    float v01 = g[IDX(s, i, j1)];
    float v11 = g[IDX(s, i1, j1)];
    float a = (1 - i_frac) * v00;
    float b = i_frac * v10;
    float value_0 = a + b;
    a = (1 - i_frac) * v01;
    b = i_frac * v11;
    float value_1 = a + b;
    a = (1 - j_frac) * value_0;
    b = j_frac * value_1;
    return a + b;
}

/* Grid::addToValueInterpolated (Grid.h:152-184).  The +1 neighbour is formed
 * before clamping. */
static void add_interp(const fso_sim* s, float* g, float gdx, float gdy, float x, float y, float value)
{
    int i = (int)(x / gdx);
    int j = (int)(y / gdy);
    int i1 = i + 1;
    int j1 = j + 1;
    float i_frac = x / gdx - (float)i;
    float j_frac = y / gdy - (float)j;
    i = clampi_ref(i, 0, s->nx - 1);
    j = clampi_ref(j, 0, s->ny - 1);
    i1 = clampi_ref(i1, 0, s->nx - 1);
    j1 = clampi_ref(j1, 0, s->ny - 1);
    float value_0 = (1 - j_frac) * value;
    float value_1 = j_frac * value;
    float value_00 = (1 - i_frac) * value_0;
    float value_10 = i_frac * value_0;
    float value_01 = (1 - i_frac) * value_1;
    float value_11 = i_frac * value_1;
    g[IDX(s, i, j)] += value_00;
    g[IDX(s, i1, j)] += value_10;
    g[IDX(s, i, j1)] += value_01;
    g[IDX(s, i1, j1)] += value_11;
}

/* MacGrid::velXInterpolated / velYInterpolated (MacGrid.h:66-79). */
static inline float vel_x_interp(const fso_sim* s, const float* u, float x, float y)
{
    return value_interp(s, u, s->dx, s->dy, x, (float)(y - s->dy * 0.5));
}
static inline float vel_y_interp(const fso_sim* s, const float* v, float x, float y)
{
    return value_interp(s, v, s->dx, s->dy, (float)(x - s->dx * 0.5), y);
}

static void* xcalloc(size_t n, size_t sz)
{
    void* p = calloc(n ? n : 1, sz);
    return p;
}

fso_sim* fso_create(int nx, int ny, float lx, float ly, float density, float pic)
{
    fso_sim* s = (fso_sim*)xcalloc(1, sizeof(fso_sim));
    size_t n = (size_t)nx * (size_t)ny;
    s->nx = nx;
    s->ny = ny;
    s->dx = lx / nx;
    s->dy = ly / ny;
    s->lx = nx * s->dx;
    s->ly = ny * s->dy;
    s->pool_dy = s->dx;
    s->density = density;
    s->pic = pic;
    s->gx = 0.0f;
    s->gy = (float)-9.82;
    s->n_ext = 2;
    s->cg_tol = (double)FLT_EPSILON;
    s->cg_maxit = 100;
    s->use_stock = 1;
    for (int b = 0; b < 2; ++b) {
        s->u[b] = (float*)xcalloc(n, sizeof(float));
        s->v[b] = (float*)xcalloc(n, sizeof(float));
        s->vmask_x[b] = (uint8_t*)xcalloc(n, 1);
        s->vmask_y[b] = (uint8_t*)xcalloc(n, 1);
    }
    s->u_prev = (float*)xcalloc(n, sizeof(float));
    s->v_prev = (float*)xcalloc(n, sizeof(float));
    s->u_diff = (float*)xcalloc(n, sizeof(float));
    s->v_diff = (float*)xcalloc(n, sizeof(float));
    s->labels = (uint8_t*)xcalloc(n, 1);
    s->level_set = (float*)xcalloc(n, sizeof(float));
    s->fidx = (int32_t*)xcalloc(n, sizeof(int32_t));
    s->counts = (uint8_t*)xcalloc(n, 1);
    s->sum_u = (float*)xcalloc(n, sizeof(float));
    s->sum_v = (float*)xcalloc(n, sizeof(float));
    s->w_u = (float*)xcalloc(n, sizeof(float));
    s->w_v = (float*)xcalloc(n, sizeof(float));
    s->pressure = (float*)xcalloc(n, sizeof(float));
    s->cg_b = (float*)xcalloc(n, sizeof(float));
    s->cg_x = (float*)xcalloc(n, sizeof(float));
    s->cg_r = (float*)xcalloc(n, sizeof(float));
    s->cg_p = (float*)xcalloc(n, sizeof(float));
    s->cg_q = (float*)xcalloc(n, sizeof(float));
    s->cg_z = (float*)xcalloc(n, sizeof(float));
    s->cg_diag = (float*)xcalloc(n, sizeof(float));
    s->cg_inv = (float*)xcalloc(n, sizeof(float));
    s->cg_down = (int32_t*)xcalloc(n, sizeof(int32_t));
    s->cg_up = (int32_t*)xcalloc(n, sizeof(int32_t));
    s->cg_left = (int32_t*)xcalloc(n, sizeof(int32_t));
    s->cg_right = (int32_t*)xcalloc(n, sizeof(int32_t));
    s->cg_nns = (uint8_t*)xcalloc(n, 1);
    s->cg_acc = (double*)xcalloc(n, sizeof(double));
    s->cg_accf = (float*)xcalloc(n, sizeof(float));
    /* MacGrid ctor clears the cell types (MacGrid.cpp:24 -> :32-50). */
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
            s->labels[IDX(s, i, j)] = (i > 0 && j > 0 && i < nx - 1 && j < ny - 1) ? FSO_AIR : FSO_SOLID;
    return s;
}

void fso_destroy(fso_sim* s)
{
    if (!s) return;
    for (int b = 0; b < 2; ++b) {
        free(s->u[b]);
        free(s->v[b]);
        free(s->vmask_x[b]);
        free(s->vmask_y[b]);
    }
    free(s->u_prev); free(s->v_prev); free(s->u_diff); free(s->v_diff);
    free(s->labels); free(s->solid); free(s->fidx); free(s->counts);
    free(s->sum_u); free(s->sum_v); free(s->w_u); free(s->w_v);
    free(s->part); free(s->pressure); free(s->src); free(s->level_set);
    free(s->cg_b); free(s->cg_x); free(s->cg_r); free(s->cg_p); free(s->cg_q); free(s->cg_z);
    free(s->cg_diag); free(s->cg_inv); free(s->cg_down); free(s->cg_up); free(s->cg_left);
    free(s->cg_right); free(s->cg_acc); free(s->cg_accf); free(s->cg_nns);
    free(s);
}

void fso_set_cg(fso_sim* s, double tol, int maxit)
{
    s->cg_tol = tol;
    s->cg_maxit = maxit;
}
void fso_set_cg_precision(fso_sim* s, int precision) { s->cg_double = precision; }
void fso_set_gravity(fso_sim* s, float gx, float gy)
{
    s->gx = gx;
    s->gy = gy;
}
void fso_set_extension_iterations(fso_sim* s, int n) { s->n_ext = n; }
void fso_set_use_stock(fso_sim* s, int use_stock) { s->use_stock = use_stock; }
/* FluidDomain::setPicRatio (FluidDomain.cpp:99-102). */
void fso_set_pic_ratio(fso_sim* s, float pic) { s->pic = clampf_ref(pic, 0, 1); }

void fso_set_solid_mask(fso_sim* s, const uint8_t* mask)
{
    size_t n = (size_t)s->nx * (size_t)s->ny;
    free(s->solid);
    s->solid = NULL;
    if (mask) {
        s->solid = (uint8_t*)xcalloc(n, 1);
        memcpy(s->solid, mask, n);
    }
}

static void reserve_particles(fso_sim* s, int64_t n)
{
    if (n <= s->cap_part) return;
    int64_t cap = s->cap_part ? s->cap_part : 1024;
    while (cap < n) cap *= 2;
    s->part = (float*)realloc(s->part, (size_t)cap * 4 * sizeof(float));
    s->cap_part = cap;
}

void fso_set_particles(fso_sim* s, const float* xyuv, int64_t n)
{
    reserve_particles(s, n);
    if (n) memcpy(s->part, xyuv, (size_t)n * 4 * sizeof(float));
    s->n_part = n;
}
int64_t fso_num_particles(const fso_sim* s) { return s->n_part; }
void fso_get_particles(const fso_sim* s, float* xyuv)
{
    if (s->n_part) memcpy(xyuv, s->part, (size_t)s->n_part * 4 * sizeof(float));
}

static float* grid_ptr(const fso_sim* s, int which)
{
    switch (which) {
        case FSO_U_FRONT: return s->u[s->front];
        case FSO_V_FRONT: return s->v[s->front];
        case FSO_U_BACK: return s->u[1 - s->front];
        case FSO_V_BACK: return s->v[1 - s->front];
        case FSO_U_PREV: return s->u_prev;
        case FSO_V_PREV: return s->v_prev;
        case FSO_U_DIFF: return s->u_diff;
        case FSO_V_DIFF: return s->v_diff;
        default: return NULL;
    }
}

void fso_get_grid(const fso_sim* s, int which, float* out)
{
    float* g = grid_ptr(s, which);
    if (g) memcpy(out, g, (size_t)s->nx * s->ny * sizeof(float));
}
void fso_set_grid(fso_sim* s, int which, const float* in)
{
    float* g = grid_ptr(s, which);
    if (g) memcpy(g, in, (size_t)s->nx * s->ny * sizeof(float));
}
void fso_get_labels(const fso_sim* s, uint8_t* out) { memcpy(out, s->labels, (size_t)s->nx * s->ny); }
void fso_set_labels(fso_sim* s, const uint8_t* in) { memcpy(s->labels, in, (size_t)s->nx * s->ny); }
void fso_get_fluid_indices(const fso_sim* s, int32_t* out)
{
    memcpy(out, s->fidx, (size_t)s->nx * s->ny * sizeof(int32_t));
}
void fso_get_particle_counts(const fso_sim* s, uint8_t* out) { memcpy(out, s->counts, (size_t)s->nx * s->ny); }
void fso_get_pressure(const fso_sim* s, float* out)
{
    size_t n = (size_t)s->nx * s->ny;
    for (size_t c = 0; c < n; ++c) {
        int32_t k = s->fidx[c];
        out[c] = (k >= 0 && k < s->n_fluid) ? s->pressure[k] : 0.0f;
    }
}
void fso_get_cg_stats(const fso_sim* s, int* iters, double* err, int* n_fluid)
{
    if (iters) *iters = s->cg_iters;
    if (err) *err = s->cg_error;
    if (n_fluid) *n_fluid = s->n_fluid;
}

/* ---- phases ------------------------------------------------------------- */

/* MacGrid::clearCellTypeBuffer (MacGrid.cpp:32-50) + FluidDomain::classifyCells
 * (FluidDomain.cpp:150-180; it labels from the domain's own particle set),
 * then the persistent solid mask (extension). */
static void ph_classify(fso_sim* s)
{
    const int nx = s->nx, ny = s->ny;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) s->labels[IDX(s, i, j)] = FSO_SOLID;
    for (int j = 1; j < ny - 1; ++j)
        for (int i = 1; i < nx - 1; ++i) s->labels[IDX(s, i, j)] = FSO_AIR;
    for (int64_t k = 0; k < s->n_part; ++k) {
        const float px = s->part[4 * k], py = s->part[4 * k + 1];
        int x = (int)((px / s->lx) * nx);
        int y = (int)((py / s->ly) * ny);
        x = clampi_ref(x, 0, nx - 1);
        y = clampi_ref(y, 0, ny - 1);
        s->labels[IDX(s, x, y)] = FSO_LIQUID;
    }
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
            if (i == 0 || j == 0 || i == nx - 1 || j == ny - 1) s->labels[IDX(s, i, j)] = FSO_SOLID;
    if (s->solid) {
        for (size_t c = 0; c < (size_t)nx * ny; ++c)
            if (s->solid[c]) s->labels[c] = FSO_SOLID;
    }
}

/* FluidSolver::transferVelocityToGridSpread (FluidSolver.cpp:873-919).  The
 * accumulator grids live in the solver's pool, whose y spacing is dx. */
static void ph_p2g(fso_sim* s)
{
    const size_t n = (size_t)s->nx * s->ny;
    const float pdx = s->dx, pdy = s->pool_dy;
    memset(s->sum_u, 0, n * sizeof(float));
    memset(s->sum_v, 0, n * sizeof(float));
    memset(s->w_u, 0, n * sizeof(float));
    memset(s->w_v, 0, n * sizeof(float));
    for (int64_t k = 0; k < s->n_part; ++k) {
        const float px = s->part[4 * k], py = s->part[4 * k + 1];
        const float vx = s->part[4 * k + 2], vy = s->part[4 * k + 3];
        add_interp(s, s->sum_u, pdx, pdy, px, (float)(py - 0.5 * s->dy), vx);
        add_interp(s, s->sum_v, pdx, pdy, (float)(px - 0.5 * s->dx), py, vy);
        add_interp(s, s->w_u, pdx, pdy, px, (float)(py - 0.5 * s->dy), (float)1.0);
        add_interp(s, s->w_v, pdx, pdy, (float)(px - 0.5 * s->dx), py, (float)1.0);
    }
    float* ub = UB(s);
    float* vb = VB(s);
    for (size_t c = 0; c < n; ++c) {
        if (s->w_u[c] > 0.000001) ub[c] = s->sum_u[c] / s->w_u[c];
        if (s->w_v[c] > 0.000001) vb[c] = s->sum_v[c] / s->w_v[c];
    }
    s->front = 1 - s->front; /* MacGrid::swapVelocityBuffers (MacGrid.cpp:89-93) */
}

/* MacGrid::updatePreviousVelocityBuffer (MacGrid.cpp:52-56). */
static void ph_save_prev(fso_sim* s)
{
    const size_t n = (size_t)s->nx * s->ny;
    memcpy(s->u_prev, UF(s), n * sizeof(float));
    memcpy(s->v_prev, VF(s), n * sizeof(float));
}

/* MacGrid::updateVelocityDiffBuffer (MacGrid.cpp:58-70). */
static void ph_save_diff(fso_sim* s)
{
    const size_t n = (size_t)s->nx * s->ny;
    const float* uf = UF(s);
    const float* vf = VF(s);
    for (size_t c = 0; c < n; ++c) {
        s->u_diff[c] = uf[c] - s->u_prev[c];
        s->v_diff[c] = vf[c] - s->v_prev[c];
    }
}

/* FluidSolver::addExternalAcceleration (FluidSolver.cpp:276-295). */
static void ph_gravity(fso_sim* s, float dt)
{
    float* uf = UF(s);
    float* vf = VF(s);
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i)
            if (cell_type(s, i, j) == FSO_LIQUID) {
                const size_t c = IDX(s, i, j);
                float t = s->gx * dt;
                uf[c] = uf[c] + t;
                t = s->gy * dt;
                vf[c] = vf[c] + t;
            }
}

/* FluidSolver::enforceDirichlet (FluidSolver.cpp:297-321). */
static void ph_dirichlet(fso_sim* s)
{
    float* uf = UF(s);
    float* vf = VF(s);
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
            const int im1 = clampi_ref(i - 1, 0, s->nx - 1);
            const int jm1 = clampi_ref(j - 1, 0, s->ny - 1);
            const size_t c = IDX(s, i, j);
            if ((cell_type(s, im1, j) == FSO_SOLID && uf[c] < 0) || (cell_type(s, i, j) == FSO_SOLID && uf[c] > 0))
                uf[c] = 0;
            if ((cell_type(s, i, jm1) == FSO_SOLID && vf[c] < 0) || (cell_type(s, i, j) == FSO_SOLID && vf[c] > 0))
                vf[c] = 0;
        }
}

/* FluidSolver::extendVelocityIndividual (FluidSolver.cpp:485-622) with
 * FluidSolverMemoryPool::swapValidMaskBuffer (:72-76).  The else-branch of
 * the y validity test zeroes the front *x* velocity (:527); that is kept. */
static void ph_extend(fso_sim* s, int n_iterations)
{
    const int nx = s->nx, ny = s->ny;
    float* uf = UF(s);
    float* vf = VF(s);
    float* ub = UB(s);
    float* vb = VB(s);
    uint8_t* mxf = s->vmask_x[s->vfront];
    uint8_t* mxb = s->vmask_x[1 - s->vfront];
    uint8_t* myf = s->vmask_y[s->vfront];
    uint8_t* myb = s->vmask_y[1 - s->vfront];
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t c = IDX(s, i, j);
            if (cell_type(s, i, j) == FSO_LIQUID || cell_type(s, i - 1, j) == FSO_LIQUID) {
                mxf[c] = 1;
                mxb[c] = 1;
                ub[c] = uf[c];
            } else {
                mxf[c] = 0;
                mxb[c] = 0;
                ub[c] = 0;
                uf[c] = 0;
            }
            if (cell_type(s, i, j) == FSO_LIQUID || cell_type(s, i, j - 1) == FSO_LIQUID) {
                myf[c] = 1;
                myb[c] = 1;
                vb[c] = vf[c];
            } else {
                myf[c] = 0;
                myb[c] = 0;
                vb[c] = 0;
                uf[c] = 0;
            }
        }
    for (int iter = 0; iter < n_iterations; ++iter) {
        mxf = s->vmask_x[s->vfront];
        mxb = s->vmask_x[1 - s->vfront];
        myf = s->vmask_y[s->vfront];
        myb = s->vmask_y[1 - s->vfront];
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t c = IDX(s, i, j);
                if (mxf[c] == 0 && cell_type(s, i, j) != FSO_SOLID && cell_type(s, i - 1, j) != FSO_SOLID) {
                    float nv = 0;
                    int nn = 0;
                    if (mxf[IDX(s, i - 1, j)] == 1) { nv += ub[IDX(s, i - 1, j)]; nn++; }
                    if (mxf[IDX(s, i, j - 1)] == 1) { nv += ub[IDX(s, i, j - 1)]; nn++; }
                    if (mxf[IDX(s, i, j + 1)] == 1) { nv += ub[IDX(s, i, j + 1)]; nn++; }
                    if (mxf[IDX(s, i + 1, j)] == 1) { nv += ub[IDX(s, i + 1, j)]; nn++; }
                    if (nn > 0) {
                        nv /= nn;
                        ub[c] = nv;
                        mxb[c] = 1;
                    }
                }
                if (myf[c] == 0 && cell_type(s, i, j) != FSO_SOLID && cell_type(s, i, j - 1) != FSO_SOLID) {
                    float nv = 0;
                    int nn = 0;
                    if (myf[IDX(s, i - 1, j)] == 1) { nv += vb[IDX(s, i - 1, j)]; nn++; }
                    if (myf[IDX(s, i, j - 1)] == 1) { nv += vb[IDX(s, i, j - 1)]; nn++; }
                    if (myf[IDX(s, i, j + 1)] == 1) { nv += vb[IDX(s, i, j + 1)]; nn++; }
                    if (myf[IDX(s, i + 1, j)] == 1) { nv += vb[IDX(s, i + 1, j)]; nn++; }
                    if (nn > 0) {
                        nv /= nn;
                        vb[c] = nv;
                        myb[c] = 1;
                    }
                }
            }
        s->vfront = 1 - s->vfront;
    }
    s->front = 1 - s->front;
}

/* The sum of n doubles by the fixed 32-ary stride-halving tree used by every
 * CG dot product (same order as fs_rsum32 in the Eigen stand-in and as the
 * GPU's warp-shuffle reduction).  Destroys a[]. */
static double rsum32(double* a, int64_t n)
{
    if (n <= 0) return 0.0;
    while (n > 1) {
        const int64_t groups = (n + 31) / 32;
        for (int64_t g = 0; g < groups; ++g) {
            double t[32];
            for (int l = 0; l < 32; ++l) {
                const int64_t k = g * 32 + l;
                t[l] = k < n ? a[k] : 0.0;
            }
            for (int st = 16; st >= 1; st >>= 1)
                for (int l = 0; l < st; ++l) t[l] = t[l] + t[l + st];
            a[g] = t[0];
        }
        n = groups;
    }
    return a[0];
}

/* The same tree in float. */
static float rsum32f(float* a, int64_t n)
{
    if (n <= 0) return 0.0f;
    while (n > 1) {
        const int64_t groups = (n + 31) / 32;
        for (int64_t g = 0; g < groups; ++g) {
            float t[32];
            for (int l = 0; l < 32; ++l) {
                const int64_t k = g * 32 + l;
                t[l] = k < n ? a[k] : 0.0f;
            }
            for (int st = 16; st >= 1; st >>= 1)
                for (int l = 0; l < st; ++l) t[l] = t[l] + t[l + st];
            a[g] = t[0];
        }
        n = groups;
    }
    return a[0];
}

/* Exact float*float products summed in double. */
static double dot_d(fso_sim* s, const float* a, const float* b, int n)
{
    for (int k = 0; k < n; ++k) s->cg_acc[k] = (double)a[k] * (double)b[k];
    return rsum32(s->cg_acc, n);
}

/* Double-single dot product (the GPU's FS_CG_DS; no counterpart in the
 * reference): each float*float product exactly as a float pair (the product
 * and its fmaf error), each group of 32 consecutive elements summed in such
 * pairs along the 32-ary stride-halving tree -- TwoSum of the high parts, the
 * error and both low parts added to it in float, no renormalisation -- each
 * group's pair converted to double (high + low, exact), and the groups summed
 * by rsum32. */
typedef struct {
    float hi, lo;
} fso_ds;

static fso_ds ds_prod(float a, float b)
{
    fso_ds r;
    r.hi = a * b;
    r.lo = fmaf(a, b, -r.hi);
    return r;
}

static fso_ds ds_add(fso_ds a, fso_ds b)
{
    const float s = a.hi + b.hi;
    const float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);
    e = e + a.lo;
    e = e + b.lo;
    fso_ds r;
    r.hi = s;
    r.lo = e;
    return r;
}

static double dot_ds(fso_sim* s, const float* a, const float* b, int n)
{
    const int groups = (n + 31) / 32;
    for (int g = 0; g < groups; ++g) {
        fso_ds t[32];
        for (int l = 0; l < 32; ++l) {
            const int k = g * 32 + l;
            if (k < n) {
                t[l] = ds_prod(a[k], b[k]);
            } else {
                t[l].hi = 0.0f;
                t[l].lo = 0.0f;
            }
        }
        for (int st = 16; st >= 1; st >>= 1)
            for (int l = 0; l < st; ++l) t[l] = ds_add(t[l], t[l + st]);
        s->cg_acc[g] = (double)t[0].hi + (double)t[0].lo;
    }
    return rsum32(s->cg_acc, groups);
}

/* Float products summed in float (the precision of Eigen's VectorXf::dot). */
static float dot_f(fso_sim* s, const float* a, const float* b, int n)
{
    for (int k = 0; k < n; ++k) s->cg_accf[k] = a[k] * b[k];
    return rsum32f(s->cg_accf, n);
}

/* q = A p, each row summed in ascending column order from +0:
 * down (fluid row below), left, diagonal, right, up. */
static void spmv(fso_sim* s, const float* p, float* q, int n, float off)
{
    for (int k = 0; k < n; ++k) {
        float acc = 0.0f, t;
        if (s->cg_down[k] >= 0) { t = off * p[s->cg_down[k]]; acc = acc + t; }
        if (s->cg_left[k] >= 0) { t = off * p[s->cg_left[k]]; acc = acc + t; }
        t = s->cg_diag[k] * p[k];
        acc = acc + t;
        if (s->cg_right[k] >= 0) { t = off * p[s->cg_right[k]]; acc = acc + t; }
        if (s->cg_up[k] >= 0) { t = off * p[s->cg_up[k]]; acc = acc + t; }
        q[k] = acc;
    }
}

/* Jacobi-preconditioned CG, zero initial guess (the published algorithm that
 * Eigen::ConjugateGradient implements; FluidSolver.cpp:423-425).  R is the
 * accumulation type of the dot products and of alpha / beta / the stopping
 * threshold (float: the reference's precision; double: the FP64 variant). */
#define FSO_CG_BODY(R, DOT, RMIN)                                              \
    do {                                                                       \
        const R bb = DOT(s, r, r, n);                                          \
        if (bb == (R)0) return;                                                \
        const R tolr = (R)s->cg_tol;                                           \
        R thr = tolr * tolr;                                                   \
        thr = thr * bb;                                                        \
        if (thr < RMIN) thr = RMIN;                                            \
        R rr = bb;                                                             \
        if (rr < thr) {                                                        \
            s->cg_error = sqrt((double)rr / (double)bb);                       \
            return;                                                            \
        }                                                                      \
        for (int k = 0; k < n; ++k) p[k] = s->cg_inv[k] * r[k];                \
        R rz = DOT(s, r, p, n);                                                \
        for (int it = 1; it <= s->cg_maxit; ++it) {                            \
            spmv(s, p, q, n, off);                                             \
            const R pq = DOT(s, p, q, n);                                      \
            const float alpha = (float)(rz / pq);                              \
            for (int k = 0; k < n; ++k) {                                      \
                float t = alpha * p[k];                                        \
                x[k] = x[k] + t;                                               \
                t = alpha * q[k];                                              \
                r[k] = r[k] - t;                                               \
            }                                                                  \
            rr = DOT(s, r, r, n);                                              \
            s->cg_iters = it;                                                  \
            if (rr < thr) break;                                               \
            for (int k = 0; k < n; ++k) z[k] = s->cg_inv[k] * r[k];            \
            const R rz_new = DOT(s, r, z, n);                                  \
            const float beta = (float)(rz_new / rz);                           \
            rz = rz_new;                                                       \
            for (int k = 0; k < n; ++k) {                                      \
                const float t = beta * p[k];                                   \
                p[k] = z[k] + t;                                               \
            }                                                                  \
        }                                                                      \
        s->cg_error = sqrt((double)rr / (double)bb);                           \
    } while (0)

static void cg_solve(fso_sim* s, int n, float off)
{
    float *b = s->cg_b, *x = s->cg_x, *r = s->cg_r, *p = s->cg_p, *q = s->cg_q, *z = s->cg_z;
    for (int k = 0; k < n; ++k) {
        const float d = s->cg_diag[k];
        s->cg_inv[k] = d != 0.0f ? 1.0f / d : 1.0f;
        x[k] = 0.0f;
        r[k] = b[k];
    }
    s->cg_iters = 0;
    s->cg_error = 0.0;
    if (s->cg_double == 2) FSO_CG_BODY(double, dot_ds, DBL_MIN);
    else if (s->cg_double) FSO_CG_BODY(double, dot_d, DBL_MIN);
    else FSO_CG_BODY(float, dot_f, FLT_MIN);
}

/* Fluid indexing (FluidSolver.cpp:329-346; the particle counts are reset) and
 * the matrix rows of :363-416 (off-diagonal and diagonal in float through
 * double pow(), as the reference).  Returns the number of fluid cells. */
static int index_and_assemble(fso_sim* s)
{
    const int nx = s->nx, ny = s->ny;
    int nf = 0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t c = IDX(s, i, j);
            if (cell_type(s, i, j) == FSO_LIQUID) s->fidx[c] = nf++;
            else s->fidx[c] = -1;
            s->counts[c] = 0;
        }
    s->n_fluid = nf;
    const float* uf = UF(s);
    const float* vf = VF(s);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t c = IDX(s, i, j);
            const int k = s->fidx[c];
            if (k == -1) continue;
            int nns = 0;
            s->cg_left[k] = s->cg_right[k] = s->cg_down[k] = s->cg_up[k] = -1;
            if (cell_type(s, i - 1, j) != FSO_SOLID) {
                if (cell_type(s, i - 1, j) == FSO_LIQUID) s->cg_left[k] = s->fidx[IDX(s, i - 1, j)];
                nns++;
            }
            if (cell_type(s, i + 1, j) != FSO_SOLID) {
                if (cell_type(s, i + 1, j) == FSO_LIQUID) s->cg_right[k] = s->fidx[IDX(s, i + 1, j)];
                nns++;
            }
            if (cell_type(s, i, j - 1) != FSO_SOLID) {
                if (cell_type(s, i, j - 1) == FSO_LIQUID) s->cg_down[k] = s->fidx[IDX(s, i, j - 1)];
                nns++;
            }
            if (cell_type(s, i, j + 1) != FSO_SOLID) {
                if (cell_type(s, i, j + 1) == FSO_LIQUID) s->cg_up[k] = s->fidx[IDX(s, i, j + 1)];
                nns++;
            }
            s->cg_diag[k] = (float)(-nns / pow(s->dx, 2));
            s->cg_nns[k] = (uint8_t)nns;
            /* MacGrid::divVelX + divVelY (MacGrid.h:98-111). */
            float ddx = uf[IDX(s, i + 1, j)] - uf[c];
            ddx = ddx / s->dx;
            float ddy = vf[IDX(s, i, j + 1)] - vf[c];
            ddy = ddy / s->dy;
            s->cg_b[k] = ddx + ddy;
        }
    return nf;
}

/* FluidSolver::pressureSolve (FluidSolver.cpp:323-483). */
static void ph_pressure(fso_sim* s, float dt)
{
    const int nx = s->nx, ny = s->ny;
    const int nf = index_and_assemble(s);
    if (nf == 0) {
        s->cg_iters = 0;
        s->cg_error = 0.0;
        return;
    }
    /* :353-360 -- unclamped; out-of-range indices are undefined behaviour in
     * the reference and are skipped here. */
    for (int64_t k = 0; k < s->n_part; ++k) {
        const float px = s->part[4 * k], py = s->part[4 * k + 1];
        const int x = (int)((px / s->lx) * nx);
        const int y = (int)((py / s->ly) * ny);
        if (x >= 0 && x < nx && y >= 0 && y < ny) s->counts[IDX(s, x, y)]++;
    }
    const float off = (float)(1 / pow(s->dx, 2));
    const float* uf = UF(s);
    const float* vf = VF(s);
    cg_solve(s, nf, off);
    memcpy(s->pressure, s->cg_x, (size_t)nf * sizeof(float));

    /* :428-482 (volume-loss term with k = 0). */
    float* ub = UB(s);
    float* vb = VB(s);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int im1 = clampi_ref(i - 1, 0, nx - 1);
            const int jm1 = clampi_ref(j - 1, 0, ny - 1);
            const int idx = s->fidx[IDX(s, i, j)];
            const int idx_im1 = s->fidx[IDX(s, im1, j)];
            const int idx_jm1 = s->fidx[IDX(s, i, jm1)];
            if (idx >= 0 || idx_im1 >= 0 || idx_jm1 >= 0) {
                /* The reference reads n_particles(i-1, j) and (i, j-1) unclamped;
                 * the term is multiplied by k = 0, so an out-of-grid read only
                 * ever contributes +0 there and is replaced by 0 here. */
                const float kk = 0.0;
                const int c_ij = s->counts[IDX(s, i, j)];
                const int c_im1 = i > 0 ? s->counts[IDX(s, i - 1, j)] : 0;
                const int c_jm1 = j > 0 ? s->counts[IDX(s, i, j - 1)] : 0;
                const float pp_ij = kk * (c_ij > 9 ? c_ij - 8 : 0);
                const float pp_im1 = kk * (c_im1 > 9 ? c_im1 - 8 : 0);
                const float pp_jm1 = kk * (c_jm1 > 9 ? c_jm1 - 8 : 0);
                const float p = idx >= 0 ? s->cg_x[idx] + pp_ij : 0;
                const float p_im1 = idx_im1 >= 0 ? s->cg_x[idx_im1] + pp_im1 : 0;
                const float p_jm1 = idx_jm1 >= 0 ? s->cg_x[idx_jm1] + pp_jm1 : 0;
                const float dpx = p - p_im1;
                const float dpy = p - p_jm1;
                const size_t c = IDX(s, i, j);
                const float vel_x = uf[c];
                const float vel_y = vf[c];
                float t = dt / s->density;
                t = t * dpx;
                t = t / s->dx;
                ub[c] = vel_x - t;
                t = dt / s->density;
                t = t * dpy;
                t = t / s->dy;
                vb[c] = vel_y - t;
            }
        }
    s->front = 1 - s->front;
}

/* FluidSolver::transferVelocityToParticlesPICFLIP (FluidSolver.cpp:945-963). */
static void ph_g2p_picflip(fso_sim* s)
{
    const float r = s->pic;
    const float* uf = UF(s);
    const float* vf = VF(s);
    for (int64_t k = 0; k < s->n_part; ++k) {
        float* pp = s->part + 4 * k;
        const float px = pp[0], py = pp[1];
        const float pic_x = vel_x_interp(s, uf, px, py);
        const float pic_y = vel_y_interp(s, vf, px, py);
        const float flip_x = pp[2] + vel_x_interp(s, s->u_diff, px, py);
        const float flip_y = pp[3] + vel_y_interp(s, s->v_diff, px, py);
        float a = pic_x * r;
        float b = flip_x * (1 - r);
        pp[2] = a + b;
        a = pic_y * r;
        b = flip_y * (1 - r);
        pp[3] = a + b;
    }
}

/* FluidSolver::transferVelocityToParticlesPIC (FluidSolver.cpp:921-931). */
static void ph_g2p_pic(fso_sim* s)
{
    const float* uf = UF(s);
    const float* vf = VF(s);
    for (int64_t k = 0; k < s->n_part; ++k) {
        float* pp = s->part + 4 * k;
        const float vx = vel_x_interp(s, uf, pp[0], pp[1]);
        const float vy = vel_y_interp(s, vf, pp[0], pp[1]);
        pp[2] = vx;
        pp[3] = vy;
    }
}

/* FluidSolver::transferVelocityToParticlesFLIP (FluidSolver.cpp:933-943). */
static void ph_g2p_flip(fso_sim* s)
{
    for (int64_t k = 0; k < s->n_part; ++k) {
        float* pp = s->part + 4 * k;
        const float vx = pp[2] + vel_x_interp(s, s->u_diff, pp[0], pp[1]);
        const float vy = pp[3] + vel_y_interp(s, s->v_diff, pp[0], pp[1]);
        pp[2] = vx;
        pp[3] = vy;
    }
}

/* MarkerParticleSet::advectAndEnsureOutsideObstacles (MarkerParticleSet.cpp:48-62)
 * with MarkerParticle::advect (MarkerParticleSet.h:37-41). */
static void ph_advect_safe(fso_sim* s, float dt)
{
    for (int64_t k = 0; k < s->n_part; ++k) {
        float* pp = s->part + 4 * k;
        float t = pp[2] * dt;
        pp[0] = pp[0] + t;
        t = pp[3] * dt;
        pp[1] = pp[1] + t;
        const int x = (int)(pp[0] / s->dx);
        const int y = (int)(pp[1] / s->dy);
        if (cell_type(s, x, y) == FSO_SOLID) {
            const float mdt = -dt;
            t = pp[2] * mdt;
            pp[0] = pp[0] + t;
            t = pp[3] * mdt;
            pp[1] = pp[1] + t;
        }
    }
}

/* MarkerParticleSet::advect (MarkerParticleSet.cpp:40-46). */
static void ph_advect(fso_sim* s, float dt)
{
    for (int64_t k = 0; k < s->n_part; ++k) {
        float* pp = s->part + 4 * k;
        float t = pp[2] * dt;
        pp[0] = pp[0] + t;
        t = pp[3] * dt;
        pp[1] = pp[1] + t;
    }
}

/* FluidSolver::getAdvectedPosition (FluidSolver.cpp:793-814) with
 * RK3::step (OdeSolver.h:102-113) on the Vec2 of FluidSolver.h:120-141:
 *   k1 = f(x); k2 = f(x + ((k1*h)*1)/2); k3 = f(x + ((k2*h)*3)/4);
 *   dy = ((((k1*2 + k2*3) + k3*4) * h) * 1) / 9. */
static void advected_position(const fso_sim* s, float x, float y, float h, float* ox, float* oy)
{
    const float* uf = UF(s);
    const float* vf = VF(s);
    float k1x = vel_x_interp(s, uf, x, y);
    float k1y = vel_y_interp(s, vf, x, y);
    float tx = k1x * h, ty = k1y * h;
    tx = tx * (float)1.0;
    ty = ty * (float)1.0;
    tx = tx / (float)2;
    ty = ty / (float)2;
    float ax = x + tx, ay = y + ty;
    float k2x = vel_x_interp(s, uf, ax, ay);
    float k2y = vel_y_interp(s, vf, ax, ay);
    tx = k2x * h;
    ty = k2y * h;
    tx = tx * (float)3.0;
    ty = ty * (float)3.0;
    tx = tx / (float)4;
    ty = ty / (float)4;
    ax = x + tx;
    ay = y + ty;
    float k3x = vel_x_interp(s, uf, ax, ay);
    float k3y = vel_y_interp(s, vf, ax, ay);
    float sx = k1x * (float)2, sy = k1y * (float)2;
    float t2x = k2x * (float)3, t2y = k2y * (float)3;
    sx = sx + t2x;
    sy = sy + t2y;
    float t3x = k3x * (float)4, t3y = k3y * (float)4;
    sx = sx + t3x;
    sy = sy + t3y;
    sx = sx * h;
    sy = sy * h;
    sx = sx * (float)1.0;
    sy = sy * (float)1.0;
    sx = sx / (float)9;
    sy = sy / (float)9;
    *ox = x + sx;
    *oy = y + sy;
}

/* FluidSolver::advectVelocitySemiLagrangian (FluidSolver.cpp:709-772): clears
 * the back buffers, then splats the front velocity sampled at each face with
 * a liquid neighbour onto its RK3 back-traced position.  No swap. */
static void ph_sl_velocity(fso_sim* s, float dt)
{
    const int nx = s->nx, ny = s->ny;
    float* ub = UB(s);
    float* vb = VB(s);
    const float* uf = UF(s);
    const float* vf = VF(s);
    memset(ub, 0, (size_t)nx * ny * sizeof(float));
    memset(vb, 0, (size_t)nx * ny * sizeof(float));
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            if (cell_type(s, i, j) == FSO_LIQUID || cell_type(s, i - 1, j) == FSO_LIQUID) {
                const float x = i * s->dx;
                const float y = (float)((j + 0.5) * s->dy);
                float xp, yp;
                advected_position(s, x, y, -dt, &xp, &yp);
                const float vx = vel_x_interp(s, uf, x, y);
                add_interp(s, ub, s->dx, s->dy, xp, (float)(yp - 0.5 * s->dy), vx);
            }
            if (cell_type(s, i, j) == FSO_LIQUID || cell_type(s, i, j - 1) == FSO_LIQUID) {
                const float x = (float)((i + 0.5) * s->dx);
                const float y = j * s->dy;
                float xp, yp;
                advected_position(s, x, y, -dt, &xp, &yp);
                const float vy = vel_y_interp(s, vf, x, y);
                add_interp(s, vb, s->dx, s->dy, (float)(xp - 0.5 * s->dx), yp, vy);
            }
        }
}

/* FluidSolver::advectParticlesWithGrid (FluidSolver.cpp:774-791). */
static void ph_sl_particles(fso_sim* s, float dt)
{
    for (int64_t k = 0; k < s->n_part; ++k) {
        float* pp = s->part + 4 * k;
        float nx_, ny_;
        advected_position(s, pp[0], pp[1], dt, &nx_, &ny_);
        pp[0] = nx_;
        pp[1] = ny_;
    }
}

int fso_phase(fso_sim* s, int ph, float dt)
{
    switch (ph) {
        case FSO_PH_CLASSIFY: ph_classify(s); break;
        case FSO_PH_P2G: ph_p2g(s); break;
        case FSO_PH_SAVE_PREV: ph_save_prev(s); break;
        case FSO_PH_GRAVITY: ph_gravity(s, dt); break;
        case FSO_PH_DIRICHLET: ph_dirichlet(s); break;
        case FSO_PH_EXTEND: ph_extend(s, s->n_ext); break;
        case FSO_PH_PRESSURE: ph_pressure(s, dt); break;
        case FSO_PH_SAVE_DIFF: ph_save_diff(s); break;
        case FSO_PH_G2P_PICFLIP: ph_g2p_picflip(s); break;
        case FSO_PH_G2P_PIC: ph_g2p_pic(s); break;
        case FSO_PH_G2P_FLIP: ph_g2p_flip(s); break;
        case FSO_PH_ADVECT_SAFE: ph_advect_safe(s, dt); break;
        case FSO_PH_ADVECT: ph_advect(s, dt); break;
        case FSO_PH_SL_VELOCITY: ph_sl_velocity(s, dt); break;
        case FSO_PH_SL_PARTICLES: ph_sl_particles(s, dt); break;
        case FSO_PH_SWAP: s->front = 1 - s->front; break;
        default: return -2;
    }
    return 0;
}

/* FluidSolver::validate (FluidSolver.cpp:89-97) against the pool copy whose
 * delta_y equals delta_x. */
static int validate(const fso_sim* s)
{
    return fabsf(s->dx - s->dx) < 0.0000001 && fabsf(s->dy - s->pool_dy) < 0.0000001;
}

/* FluidSolver::step* (FluidSolver.cpp:99-251): phase order per method. */
int fso_step(fso_sim* s, int method, float dt)
{
    static const int seq_sl[] = {FSO_PH_CLASSIFY, FSO_PH_SL_VELOCITY, FSO_PH_GRAVITY, FSO_PH_DIRICHLET,
                                 FSO_PH_PRESSURE, FSO_PH_DIRICHLET, FSO_PH_SL_PARTICLES, -1};
    static const int seq_pic[] = {FSO_PH_CLASSIFY, FSO_PH_P2G, FSO_PH_GRAVITY, FSO_PH_DIRICHLET, FSO_PH_EXTEND,
                                  FSO_PH_PRESSURE, FSO_PH_DIRICHLET, FSO_PH_G2P_PIC, FSO_PH_ADVECT, -1};
    static const int seq_flip[] = {FSO_PH_CLASSIFY, FSO_PH_P2G, FSO_PH_SAVE_PREV, FSO_PH_GRAVITY,
                                   FSO_PH_DIRICHLET, FSO_PH_EXTEND, FSO_PH_PRESSURE, FSO_PH_DIRICHLET,
                                   FSO_PH_SAVE_DIFF, FSO_PH_G2P_FLIP, FSO_PH_ADVECT, -1};
    static const int seq_picflip[] = {FSO_PH_CLASSIFY, FSO_PH_P2G, FSO_PH_SAVE_PREV, FSO_PH_GRAVITY,
                                      FSO_PH_DIRICHLET, FSO_PH_EXTEND, FSO_PH_PRESSURE, FSO_PH_DIRICHLET,
                                      FSO_PH_SAVE_DIFF, FSO_PH_G2P_PICFLIP, FSO_PH_ADVECT_SAFE, -1};
    const int* seq;
    switch (method) {
        case FSO_STEP_SEMI_LAGRANGIAN: seq = seq_sl; break;
        case FSO_STEP_PIC: seq = seq_pic; break;
        case FSO_STEP_FLIP: seq = seq_flip; break;
        case FSO_STEP_PICFLIP: seq = seq_picflip; break;
        default: return -2;
    }
    if (!validate(s)) return -1;
    for (int k = 0; seq[k] >= 0; ++k) fso_phase(s, seq[k], dt);
    return 0;
}

/* FluidSource (FluidDomain.cpp:3-52) and FluidDomain::update (:80-87). */
void fso_add_source(fso_sim* s, float x_min, float x_max, float y_min, float y_max, float dx, float dy,
                    float vx, float vy, float time_step, int max_spawns)
{
    if (s->n_src == s->cap_src) {
        s->cap_src = s->cap_src ? 2 * s->cap_src : 4;
        s->src = (fso_source*)realloc(s->src, (size_t)s->cap_src * sizeof(fso_source));
    }
    fso_source* f = &s->src[s->n_src++];
    f->x_min = x_min;
    f->x_max = x_max;
    f->y_min = y_min;
    f->y_max = y_max;
    f->dx = dx;
    f->dy = dy;
    f->vx = vx;
    f->vy = vy;
    f->time_step = time_step;
    f->time_since_last = 0.0f;
    f->max_spawns = max_spawns;
    f->n_spawns = 0;
}

static void add_particle(fso_sim* s, float x, float y, float vx, float vy)
{
    reserve_particles(s, s->n_part + 1);
    float* pp = s->part + 4 * s->n_part;
    pp[0] = x;
    pp[1] = y;
    pp[2] = vx;
    pp[3] = vy;
    s->n_part++;
}

void fso_update(fso_sim* s, float dt)
{
    for (int k = 0; k < s->n_src; ++k) {
        fso_source* f = &s->src[k];
        if (f->max_spawns != -1 && f->n_spawns >= f->max_spawns) continue;
        if (f->time_since_last >= f->time_step) {
            const float x_incr = (float)(f->dx / 2.5);
            const float y_incr = (float)(f->dy / 2.5);
            for (float y = f->y_min; y < f->y_max; y += y_incr)
                for (float x = f->x_min; x < f->x_max; x += x_incr) add_particle(s, x, y, f->vx, f->vy);
            f->time_since_last = 0;
            f->n_spawns++;
        }
        f->time_since_last += dt;
    }
}

/* FluidDomain::clearFluidSources (FluidDomain.cpp:89-92). */
void fso_clear_sources(fso_sim* s) { s->n_src = 0; }


/* ---- pressure projection alone (the GPU's fs_poisson_*) ------------------- */

/* Row of A in double: ascending column order from +0 (as spmv()). */
static double row64(const fso_sim* s, const double* v, int k, double off, const double* dtab)
{
    double acc = 0.0, t;
    if (s->cg_down[k] >= 0) { t = off * v[s->cg_down[k]]; acc = acc + t; }
    if (s->cg_left[k] >= 0) { t = off * v[s->cg_left[k]]; acc = acc + t; }
    t = dtab[s->cg_nns[k]] * v[k];
    acc = acc + t;
    if (s->cg_right[k] >= 0) { t = off * v[s->cg_right[k]]; acc = acc + t; }
    if (s->cg_up[k] >= 0) { t = off * v[s->cg_up[k]]; acc = acc + t; }
    return acc;
}

static double dot64v(double* acc, const double* a, const double* b, int n)
{
    for (int k = 0; k < n; ++k) acc[k] = a[k] * b[k];
    return rsum32(acc, n);
}

/* CG with double vectors, SpMV and dots (the GPU's k_cg64). */
static void cg64(fso_sim* s, int n, const double* b, double* x, double tol, int maxit, double off,
                 const double* dtab, const double* itab, int* iters_out)
{
    double* r = (double*)xcalloc((size_t)n, sizeof(double));
    double* z = (double*)xcalloc((size_t)n, sizeof(double));
    double* p = (double*)xcalloc((size_t)n, sizeof(double));
    double* q = (double*)xcalloc((size_t)n, sizeof(double));
    double* acc = (double*)xcalloc((size_t)n, sizeof(double));
    for (int k = 0; k < n; ++k) {
        x[k] = 0.0;
        r[k] = b[k];
        z[k] = itab[s->cg_nns[k]] * r[k];
    }
    int iters = 0;
    const double bb = dot64v(acc, r, r, n);
    double rz = dot64v(acc, r, z, n), rr = bb;
    double thr = tol * tol;
    thr = thr * bb;
    if (thr < DBL_MIN) thr = DBL_MIN;
    if (bb != 0.0 && !(rr < thr)) {
        for (int k = 0; k < n; ++k) p[k] = z[k];
        for (int it = 1; it <= maxit; ++it) {
            for (int k = 0; k < n; ++k) q[k] = row64(s, p, k, off, dtab);
            const double alpha = rz / dot64v(acc, p, q, n);
            for (int k = 0; k < n; ++k) {
                double t = alpha * p[k];
                x[k] = x[k] + t;
                t = alpha * q[k];
                r[k] = r[k] - t;
                z[k] = itab[s->cg_nns[k]] * r[k];
            }
            rr = dot64v(acc, r, r, n);
            const double rz_new = dot64v(acc, r, z, n);
            iters = it;
            if (rr < thr) break;
            const double beta = rz_new / rz;
            rz = rz_new;
            for (int k = 0; k < n; ++k) {
                const double t = beta * p[k];
                p[k] = z[k] + t;
            }
        }
    }
    *iters_out = iters;
    free(r); free(z); free(p); free(q); free(acc);
}

int fso_poisson_solve(int nx, int ny, float lx, float ly, const uint8_t* labels, const double* rhs, int method,
                      double tol, int maxit, double inner_tol, int inner_precision, double* x_out,
                      int* outer_out, int* inner_out, double* residual_out)
{
    fso_sim* s = fso_create(nx, ny, lx, ly, 1.0f, 0.0f);
    memcpy(s->labels, labels, (size_t)nx * ny);
    const int nf = index_and_assemble(s);
    const double dx2 = pow(s->dx, 2);
    const float off32 = (float)(1 / dx2);
    const double off64 = 1.0 / dx2;
    double dtab[5], itab[5];
    for (int k = 0; k < 5; ++k) {
        dtab[k] = -k / dx2;
        itab[k] = k ? 1.0 / dtab[k] : 1.0;
    }
    double* b = (double*)xcalloc((size_t)nf, sizeof(double));
    double* x = (double*)xcalloc((size_t)nf, sizeof(double));
    double* r = (double*)xcalloc((size_t)nf, sizeof(double));
    double* acc = (double*)xcalloc((size_t)nf, sizeof(double));
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int k = s->fidx[IDX(s, i, j)];
            if (k >= 0) b[k] = rhs[IDX(s, i, j)];
        }
    int outer = 0, inner = 0;
    s->cg_double = inner_precision;
    if (method == 0) { /* float CG */
        for (int k = 0; k < nf; ++k) s->cg_b[k] = (float)b[k];
        s->cg_tol = tol;
        s->cg_maxit = maxit;
        cg_solve(s, nf, off32);
        for (int k = 0; k < nf; ++k) x[k] = (double)s->cg_x[k];
        outer = 1;
        inner = s->cg_iters;
    } else if (method == 1) { /* FP64 CG */
        cg64(s, nf, b, x, tol, maxit, off64, dtab, itab, &inner);
        outer = 1;
    } else { /* FP64 refinement around float CG corrections */
        for (int k = 0; k < nf; ++k) r[k] = b[k];
        const double bb = dot64v(acc, b, b, nf);
        const double thr = tol * tol * bb;
        double rr = bb;
        s->cg_tol = inner_tol;
        s->cg_maxit = maxit;
        for (int it = 0; it < 64; ++it) {
            if (!(rr >= thr) || bb == 0.0) break;
            for (int k = 0; k < nf; ++k) s->cg_b[k] = (float)r[k];
            cg_solve(s, nf, off32);
            for (int k = 0; k < nf; ++k) x[k] = x[k] + (double)s->cg_x[k];
            for (int k = 0; k < nf; ++k) r[k] = b[k] - row64(s, x, k, off64, dtab);
            const double rr_new = dot64v(acc, r, r, nf);
            inner += s->cg_iters;
            outer = it + 1;
            if (s->cg_iters == 0) break;
            rr = rr_new;
        }
    }
    /* final residual in double */
    for (int k = 0; k < nf; ++k) r[k] = b[k] - row64(s, x, k, off64, dtab);
    const double rr = dot64v(acc, r, r, nf), bb = dot64v(acc, b, b, nf);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int k = s->fidx[IDX(s, i, j)];
            x_out[IDX(s, i, j)] = k >= 0 ? x[k] : 0.0;
        }
    if (outer_out) *outer_out = outer;
    if (inner_out) *inner_out = inner;
    if (residual_out) *residual_out = bb > 0 ? sqrt(rr / bb) : 0.0;
    free(b); free(x); free(r); free(acc);
    fso_destroy(s);
    return nf;
}


/* ---- Canvas and Renderer (Canvas.cpp, Renderer.cpp): rendering to an RGB float canvas ---- */

typedef struct
{
    int w, h;
    float* px;       /* 3 floats per pixel, row-major */
    float line[3];
    float fill[3];
} fso_canvas;

static void cv_set(fso_canvas* c, int i, int j, const float* col)
{
    float* p = c->px + 3 * ((size_t)i + (size_t)j * (size_t)c->w);
    p[0] = col[0];
    p[1] = col[1];
    p[2] = col[2];
}

/* Canvas::fillRectangle (Canvas.cpp:76-97): bounds clamped through MyFloat,
 * border pixels in the line colour, inside in the fill colour. */
static void cv_fill_rect(fso_canvas* c, int x0, int x1, int y0, int y1)
{
    x0 = clampi_ref(x0, 0, c->w - 1);
    x1 = clampi_ref(x1, 0, c->w - 1);
    y0 = clampi_ref(y0, 0, c->h - 1);
    y1 = clampi_ref(y1, 0, c->h - 1);
    for (int j = y0; j <= y1; ++j)
        for (int i = x0; i <= x1; ++i)
            cv_set(c, i, j, (i == x0 || i == x1 || j == y0 || j == y1) ? c->line : c->fill);
}

/* Canvas::drawLine (Canvas.cpp:39-62): one pixel per unit of length, stopping
 * at the first pixel outside the canvas. */
static void cv_draw_line(fso_canvas* c, int fx, int fy, int tx, int ty)
{
    const float diff_x = (float)(tx - fx);
    const float diff_y = (float)(ty - fy);
    const float distance = sqrtf(diff_x * diff_x + diff_y * diff_y);
    for (int i = 0; (float)i < distance; ++i) {
        const int x = (int)((float)fx + (diff_x / distance) * (float)i);
        const int y = (int)((float)fy + (diff_y / distance) * (float)i);
        if (x < 0 || x >= c->w || y < 0 || y >= c->h) break;
        cv_set(c, x, y, c->line);
    }
}

/* The pixel mapping shared by the Renderer functions (Renderer.cpp:23-27). */
typedef struct
{
    float scale_x, scale_y, translate_x, translate_y;
} fso_view;

static fso_view view_of(const float* area, int w, int h)
{
    fso_view v;
    v.scale_x = (float)w / (area[1] - area[0]);
    v.scale_y = (float)h / (area[3] - area[2]);
    v.translate_x = (float)(0.5 * (double)(area[0] * (float)w));
    v.translate_y = (float)(0.5 * (double)(area[2] * (float)h));
    return v;
}

#ifndef M_PI /* strict C11 leaves it out; the value glibc's math.h gives */
#define M_PI 3.14159265358979323846
#endif

/* gaussian (MathDefinitions.h:29-34) with MyFloat arguments. */
static float gaussian_ref(float x, float sigma, float mu)
{
    const float a = (float)(1 / ((double)sigma * sqrt(2 * M_PI)));
    const float xm = x - mu;
    return a * expf(-(xm * xm) / (2 * sigma * sigma));
}

/* Renderer::renderMetaBallsToCanvas's kernel weight of offset (i, j), radius 5
 * (Renderer.cpp:186-187). */
float fso_metaball_weight(int i, int j)
{
    const float t = clampf_ref((float)(sqrt((double)(i * i + j * j)) / 5), 0, 1);
    return gaussian_ref(t, 0.4f, 0.0f);
}

static void render(fso_sim* s, int what, const float* area, fso_canvas* c)
{
    const fso_view v = view_of(area, c->w, c->h);
    if (what == FSO_RENDER_CLEAR) { /* Renderer::clearCanvas (Renderer.cpp:13-16) */
        const float white[3] = {1, 1, 1};
        for (int j = 0; j < c->h; ++j)
            for (int i = 0; i < c->w; ++i) cv_set(c, i, j, white);
    } else if (what == FSO_RENDER_CELLS) { /* renderGridCellsToCanvas (Renderer.cpp:18-56) */
        const float csx = s->dx * v.scale_x, csy = s->dy * v.scale_y;
        c->line[0] = c->line[1] = c->line[2] = 1;
        for (int j = 0; j < s->ny; ++j)
            for (int i = 0; i < s->nx; ++i) {
                const uint8_t t = s->labels[IDX(s, i, j)];
                if (t == FSO_LIQUID) { c->fill[0] = 0.7f; c->fill[1] = 0.7f; c->fill[2] = 1; }
                else if (t == FSO_AIR) { c->fill[0] = 1; c->fill[1] = 1; c->fill[2] = 1; }
                else { c->fill[0] = 0.5f; c->fill[1] = 0.5f; c->fill[2] = 0.5f; }
                cv_fill_rect(c, (int)(-v.translate_x + (float)i * csx), (int)(-v.translate_x + (float)(i + 1) * csx),
                             (int)(-v.translate_y + (float)j * csy), (int)(-v.translate_y + (float)(j + 1) * csy));
            }
    } else if (what == FSO_RENDER_VELOCITIES) { /* renderGridVelocitiesToCanvas (Renderer.cpp:93-139) */
        const float csx = s->dx * v.scale_x, csy = s->dy * v.scale_y;
        const float line_scale = 5;
        for (int j = 0; j < s->ny - 1; ++j)
            for (int i = 0; i < s->nx - 1; ++i) {
                /* MacGrid::velX / velY (MacGrid.h:30-39): the cell's two faces averaged */
                const float vel_x = (UF(s)[IDX(s, i, j)] + UF(s)[IDX(s, i + 1, j)]) / 2;
                const float vel_y = (VF(s)[IDX(s, i, j)] + VF(s)[IDX(s, i, j + 1)]) / 2;
                const int from_x = (int)((double)(-v.translate_x) + (0.5 + i) * (double)csx);
                const int from_y = (int)((double)(-v.translate_y) + (0.5 + j) * (double)csy);
                const int to_x = (int)((float)from_x + vel_x * line_scale);
                const int to_y = (int)((float)from_y + vel_y * line_scale);
                const float len = (float)sqrt((double)((from_x - to_x) * (from_x - to_x) +
                                                       (from_y - to_y) * (from_y - to_y)));
                const float ls = len / (float)(c->w / 40);
                const float blue = clampf_ref(1 - ls, 0, 1);
                const float green = clampf_ref(ls, 0, 1) - clampf_ref(ls - 1, 0, 1);
                const float red = clampf_ref(ls - 1, 0, 1);
                c->line[0] = red;
                c->line[1] = green;
                c->line[2] = blue;
                cv_draw_line(c, from_x, from_y, to_x, to_y);
            }
    } else if (what == FSO_RENDER_PARTICLES) { /* renderParticlesToCanvas (Renderer.cpp:141-161) */
        c->line[0] = c->fill[0] = 0.3f;
        c->line[1] = c->fill[1] = 0.6f;
        c->line[2] = c->fill[2] = 0.9f;
        for (int64_t k = 0; k < s->n_part; ++k) {
            const int x = (int)(-v.translate_x + v.scale_x * s->part[4 * k]);
            const int y = (int)(-v.translate_y + v.scale_y * s->part[4 * k + 1]);
            cv_fill_rect(c, x - 3 / 2, x + 3 / 2, y - 3 / 2, y + 3 / 2); /* Canvas::drawPoint (Canvas.cpp:64-74) */
        }
    } else if (what == FSO_RENDER_LEVEL_SET) { /* renderLevelSetFunctionValuesToCanvas (Renderer.cpp:58-91) */
        const float csx = s->dx * v.scale_x, csy = s->dy * v.scale_y;
        c->line[0] = c->line[1] = c->line[2] = 1;
        for (int j = 0; j < s->ny; ++j)
            for (int i = 0; i < s->nx; ++i) {
                const float val = s->level_set[IDX(s, i, j)];
                c->fill[0] = c->fill[1] = c->fill[2] = val;
                cv_fill_rect(c, (int)(-v.translate_x + (float)i * csx), (int)(-v.translate_x + (float)(i + 1) * csx),
                             (int)(-v.translate_y + (float)j * csy), (int)(-v.translate_y + (float)(j + 1) * csy));
            }
    } else if (what == FSO_RENDER_METABALLS) { /* renderMetaBallsToCanvas (Renderer.cpp:163-215) */
        const int w = c->w, h = c->h;
        float* df = (float*)xcalloc((size_t)w * h, sizeof(float));
        c->line[0] = 0.5f; c->line[1] = 0.9f; c->line[2] = 1.0f;
        c->fill[0] = 0.0f; c->fill[1] = 0.5f; c->fill[2] = 0.7f;
        for (int64_t k = 0; k < s->n_part; ++k) {
            const int x = (int)(-v.translate_x + v.scale_x * s->part[4 * k]);
            const int y = (int)(-v.translate_y + v.scale_y * s->part[4 * k + 1]);
            for (int j = -5; j < 5; ++j)
                for (int i = -5; i < 5; ++i) {
                    const float t = fso_metaball_weight(i, j);
                    const int xi = x + i, yj = y + j;
                    if (xi >= 0 && xi < w && yj >= 0 && yj < h) df[(size_t)xi + (size_t)yj * w] += t;
                }
        }
        for (int j = 0; j < h; ++j)
            for (int i = 0; i < w; ++i) {
                const double d = df[(size_t)i + (size_t)j * w];
                if (d > 0.6) cv_set(c, i, j, c->fill);
                else if (d > 0.2) cv_set(c, i, j, c->line);
            }
        free(df);
    }
}

void fso_render(fso_sim* s, int what, const float* area, int w, int h, float* rgb, float* colors)
{
    fso_canvas c;
    c.w = w;
    c.h = h;
    c.px = rgb;
    memcpy(c.line, colors, 3 * sizeof(float));
    memcpy(c.fill, colors + 3, 3 * sizeof(float));
    render(s, what, area, &c);
    memcpy(colors, c.line, 3 * sizeof(float));
    memcpy(colors + 3, c.fill, 3 * sizeof(float));
}

/* Renderer::writeCanvasToPpm's conversion (Renderer.cpp:217-240): CLAMP to
 * [0, 1], times 255, truncated to a byte. */
void fso_canvas_bytes(const float* rgb, int64_t n, uint8_t* out)
{
    for (int64_t k = 0; k < 3 * n; ++k) out[k] = (uint8_t)(clampf_ref(rgb[k], 0, 1) * 255);
}


/* ---- level set (FluidDomain.cpp:104-148, LevelSet.cpp:27-59) ------------ */

void fso_get_level_set(const fso_sim* s, float* out) { memcpy(out, s->level_set, (size_t)s->nx * s->ny * sizeof(float)); }
void fso_set_level_set(fso_sim* s, const float* in) { memcpy(s->level_set, in, (size_t)s->nx * s->ny * sizeof(float)); }

/* An element of a grid by its linear index; 0 past the end, where the
 * reference's std::vector read is undefined. */
static float at_lin(const float* a, size_t idx, size_t n) { return idx < n ? a[idx] : 0.0f; }

/* LevelSet::computeUpwindGradientX / Y (LevelSet.cpp:27-59). */
static float upwind_x(const fso_sim* s, int i, int j, float vel)
{
    int ip = i + 1, im = i - 1;
    i = clampi_ref(i, 0, s->nx - 1);
    j = clampi_ref(j, 0, s->ny - 1);
    ip = clampi_ref(ip, 0, s->nx - 1);
    im = clampi_ref(im, 0, s->nx - 1);
    const float* L = s->level_set;
    return vel < 0 ? L[IDX(s, ip, j)] - L[IDX(s, i, j)] : L[IDX(s, i, j)] - L[IDX(s, im, j)];
}

static float upwind_y(const fso_sim* s, int i, int j, float vel)
{
    int jp = j + 1, jm = j - 1;
    i = clampi_ref(i, 0, s->nx - 1);
    j = clampi_ref(j, 0, s->ny - 1);
    jp = clampi_ref(jp, 0, s->ny - 1);
    jm = clampi_ref(jm, 0, s->ny - 1);
    const float* L = s->level_set;
    return vel < 0 ? L[IDX(s, i, jp)] - L[IDX(s, i, j)] : L[IDX(s, i, j)] - L[IDX(s, i, jm)];
}

/* FluidDomain::advectLevelSet (FluidDomain.cpp:104-125) as written: the loops
 * run j < sizeX, i < sizeY; MacGrid::velX / velY (MacGrid.h:30-39) average the
 * cell's face with the next one through the linear index (Grid.h:27-31); an
 * access past the end of an array reads 0 and a write past it is dropped. */
void fso_advect_level_set(fso_sim* s, float dt)
{
    const size_t n = (size_t)s->nx * s->ny, nx = (size_t)s->nx;
    float* nl = (float*)xcalloc(n, sizeof(float));
    for (int j = 0; j < s->nx; ++j)
        for (int i = 0; i < s->ny; ++i) {
            const size_t lin = (size_t)i + (size_t)j * nx;
            const float vel_x = (at_lin(UF(s), lin, n) + at_lin(UF(s), lin + 1, n)) / 2;
            const float vel_y = (at_lin(VF(s), lin, n) + at_lin(VF(s), lin + nx, n)) / 2;
            const float gx = upwind_x(s, i, j, vel_x);
            const float gy = upwind_y(s, i, j, vel_y);
            const float change = -(vel_x * gx + vel_y * gy);
            const float v = at_lin(s->level_set, lin, n) + change * dt * 5;
            if (lin < n) nl[lin] = v;
        }
    memcpy(s->level_set, nl, n * sizeof(float));
    free(nl);
}

/* FluidDomain::classifyCells(LevelSet&) (FluidDomain.cpp:127-148): border
 * SOLID, negative level set LIQUID, else AIR; then the persistent solid mask,
 * as after the particle classification. */
void fso_classify_level_set(fso_sim* s)
{
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
            uint8_t t = (i > 0 && j > 0 && i < s->nx - 1 && j < s->ny - 1) ? FSO_AIR : FSO_SOLID;
            if (s->level_set[IDX(s, i, j)] < 0) t = FSO_LIQUID;
            if (i == 0 || j == 0 || i == s->nx - 1 || j == s->ny - 1) t = FSO_SOLID;
            s->labels[IDX(s, i, j)] = t;
        }
    if (s->solid)
        for (size_t c = 0; c < (size_t)s->nx * s->ny; ++c)
            if (s->solid[c]) s->labels[c] = FSO_SOLID;
}
