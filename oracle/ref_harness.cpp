// Oracle harness over the reference's own code (test infrastructure only).
//
// Compiled by oracle/build_oracle.py together with the unmodified reference
// sources src/{FluidSolver,FluidDomain,MacGrid,MarkerParticleSet,LevelSet}.cpp
// and the project's Eigen-subset stand-in, into oracle/_ref/libfsref.so.  It
// implements the C API of oracle/fs_oracle.h by calling the reference's
// classes; private members are reached by widening access in this one
// translation unit (class layout is unaffected).
//
// Step functions: with no extension in use (no solid mask, gravity (0,-9.82),
// 2 extension sweeps) fso_step calls the reference's own
// FluidSolver::step{SemiLagrangian,PIC,FLIP,PICFLIP} (FluidSolver.cpp:99-251).
// Otherwise it calls the same private phase functions in the same order
// (the order of FluidSolver.cpp:109-133, 146-169, 183-208, 223-250), adding
// the solid mask after classification and the configured gravity.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <vector>

#include <Eigen/IterativeLinearSolvers>
#include <Eigen/SparseCore>

#define private public
#define protected public
#include <FluidDomain.h>
#include <FluidSolver.h>
#include <MacGrid.h>
#include <MarkerParticleSet.h>
#include <Canvas.h>
#include <Renderer.h>
#undef private
#undef protected

#include "fs_oracle.h"

struct fso_sim
{
    FluidDomain domain;
    FluidSolverMemoryPool pool;
    FluidSolver solver;
    float gx = 0.0f, gy = -9.82f;
    int n_ext = 2;
    bool use_stock = true;
    std::vector<uint8_t> solid;
    std::vector<float> pressure;  // by fluid index, from the last pressure solve
    int cg_iters = 0;
    double cg_error = 0.0;
    int n_fluid = 0;

    fso_sim(int nx, int ny, float lx, float ly, float density, float pic)
        : domain(nx, ny, lx, ly, density, pic), pool(domain), solver(pool)
    {
    }
};

namespace {

Grid<MyFloat>* grid_of(fso_sim* s, int which)
{
    MacGrid& g = s->domain.macGrid();
    switch (which) {
        case FSO_U_FRONT: return g._vel_x_front_buffer.get();
        case FSO_V_FRONT: return g._vel_y_front_buffer.get();
        case FSO_U_BACK: return g._vel_x_back_buffer.get();
        case FSO_V_BACK: return g._vel_y_back_buffer.get();
        case FSO_U_PREV: return &g._vel_x_previous;
        case FSO_V_PREV: return &g._vel_y_previous;
        case FSO_U_DIFF: return &g._vel_x_diff;
        case FSO_V_DIFF: return &g._vel_y_diff;
        default: return nullptr;
    }
}

bool stock_ok(const fso_sim* s)
{
    return s->use_stock && s->solid.empty() && s->gx == 0.0f && s->gy == -9.82f && s->n_ext == 2;
}

// The persistent solid mask (an extension), applied after a classification.
void apply_solid_mask(fso_sim* s)
{
    if (s->solid.empty()) return;
    MacGrid& g = s->domain.macGrid();
    for (int j = 0; j < g.sizeY(); ++j)
        for (int i = 0; i < g.sizeX(); ++i)
            if (s->solid[static_cast<size_t>(i + j * g.sizeX())]) g.setCellType(i, j, SOLID);
}

void classify(fso_sim* s)
{
    s->domain.classifyCells(s->domain.markerParticleSet());
    apply_solid_mask(s);
}

void pressure(fso_sim* s, float dt)
{
    Eigen::fs_cg_record() = Eigen::FsCgRecord();
    Eigen::fs_cg_record().iterations = -1;
    s->solver.pressureSolve(s->domain.macGrid(), s->domain.markerParticleSet(), s->domain.density(), dt);
    Eigen::FsCgRecord& rec = Eigen::fs_cg_record();
    if (rec.iterations < 0) {  // no fluid: pressureSolve returned before solving
        s->pressure.clear();
        s->cg_iters = 0;
        s->cg_error = 0.0;
        s->n_fluid = 0;
    } else {
        s->pressure.assign(rec.solution.begin(), rec.solution.end());
        s->cg_iters = static_cast<int>(rec.iterations);
        s->cg_error = rec.error;
        s->n_fluid = static_cast<int>(rec.solution.size());
    }
}

int phase(fso_sim* s, int ph, float dt)
{
    FluidDomain& d = s->domain;
    MacGrid& g = d.macGrid();
    MarkerParticleSet& ps = d.markerParticleSet();
    FluidSolver& f = s->solver;
    switch (ph) {
        case FSO_PH_CLASSIFY: classify(s); break;
        case FSO_PH_P2G: f.transferVelocityToGridSpread(ps, g); break;
        case FSO_PH_SAVE_PREV: g.updatePreviousVelocityBuffer(); break;
        case FSO_PH_GRAVITY: f.addExternalAcceleration(g, s->gx, s->gy, dt); break;
        case FSO_PH_DIRICHLET: f.enforceDirichlet(g); break;
        case FSO_PH_EXTEND: f.extendVelocityIndividual(g, s->n_ext); break;
        case FSO_PH_PRESSURE: pressure(s, dt); break;
        case FSO_PH_SAVE_DIFF: g.updateVelocityDiffBuffer(); break;
        case FSO_PH_G2P_PICFLIP: f.transferVelocityToParticlesPICFLIP(g, ps, d.picRatio()); break;
        case FSO_PH_G2P_PIC: f.transferVelocityToParticlesPIC(g, ps); break;
        case FSO_PH_G2P_FLIP: f.transferVelocityToParticlesFLIP(g, ps); break;
        case FSO_PH_ADVECT_SAFE: ps.advectAndEnsureOutsideObstacles(dt, g); break;
        case FSO_PH_ADVECT: ps.advect(dt); break;
        case FSO_PH_SL_VELOCITY: f.advectVelocitySemiLagrangian(g, dt); break;
        case FSO_PH_SL_PARTICLES: f.advectParticlesWithGrid(ps, g, dt); break;
        case FSO_PH_SWAP: g.swapVelocityBuffers(); break;
        default: return -2;
    }
    return 0;
}

}  // namespace

extern "C" {

const char* fso_kind(void) { return "reference"; }

fso_sim* fso_create(int nx, int ny, float lx, float ly, float density, float pic)
{
    return new fso_sim(nx, ny, lx, ly, density, pic);
}

void fso_destroy(fso_sim* s) { delete s; }

void fso_set_cg(fso_sim* s, double tol, int maxit)
{
    s->solver._cg_solver.setTolerance(tol);
    s->solver._cg_solver.setMaxIterations(maxit);
}

void fso_set_cg_precision(fso_sim*, int precision)
{
    Eigen::fs_cg_precision() = precision ? Eigen::FS_CG_DOUBLE : Eigen::FS_CG_FLOAT;
}

void fso_set_gravity(fso_sim* s, float gx, float gy)
{
    s->gx = gx;
    s->gy = gy;
}

void fso_set_extension_iterations(fso_sim* s, int n) { s->n_ext = n; }

void fso_set_solid_mask(fso_sim* s, const uint8_t* mask)
{
    if (!mask) {
        s->solid.clear();
        return;
    }
    size_t n = static_cast<size_t>(s->domain.sizeX()) * static_cast<size_t>(s->domain.sizeY());
    s->solid.assign(mask, mask + n);
}

void fso_set_use_stock(fso_sim* s, int use_stock) { s->use_stock = use_stock != 0; }

void fso_set_pic_ratio(fso_sim* s, float pic) { s->domain.setPicRatio(pic); }

void fso_set_particles(fso_sim* s, const float* xyuv, int64_t n)
{
    MarkerParticleSet& ps = s->domain.markerParticleSet();
    ps.clear();
    ps.reserve(static_cast<int>(n));
    for (int64_t k = 0; k < n; ++k)
        ps.addParticle(MarkerParticle(xyuv[4 * k], xyuv[4 * k + 1], xyuv[4 * k + 2], xyuv[4 * k + 3]));
}

int64_t fso_num_particles(const fso_sim* s) { return s->domain.markerParticleSet().size(); }

void fso_get_particles(const fso_sim* s, float* xyuv)
{
    int64_t k = 0;
    for (auto it = s->domain.markerParticleSet().begin(); it != s->domain.markerParticleSet().end(); ++it, ++k) {
        xyuv[4 * k] = it->posX();
        xyuv[4 * k + 1] = it->posY();
        xyuv[4 * k + 2] = it->velX();
        xyuv[4 * k + 3] = it->velY();
    }
}

void fso_get_grid(const fso_sim* s, int which, float* out)
{
    Grid<MyFloat>* g = grid_of(const_cast<fso_sim*>(s), which);
    if (!g) return;
    for (int j = 0; j < g->sizeY(); ++j)
        for (int i = 0; i < g->sizeX(); ++i) out[i + j * g->sizeX()] = g->value(i, j);
}

void fso_set_grid(fso_sim* s, int which, const float* in)
{
    Grid<MyFloat>* g = grid_of(s, which);
    if (!g) return;
    for (int j = 0; j < g->sizeY(); ++j)
        for (int i = 0; i < g->sizeX(); ++i) (*g)(i, j) = in[i + j * g->sizeX()];
}

void fso_get_labels(const fso_sim* s, uint8_t* out)
{
    const MacGrid& g = s->domain.macGrid();
    for (int j = 0; j < g.sizeY(); ++j)
        for (int i = 0; i < g.sizeX(); ++i)
            out[i + j * g.sizeX()] = static_cast<uint8_t>(g._cell_type_buffer.value(i, j));
}

void fso_set_labels(fso_sim* s, const uint8_t* in)
{
    MacGrid& g = s->domain.macGrid();
    for (int j = 0; j < g.sizeY(); ++j)
        for (int i = 0; i < g.sizeX(); ++i) g.setCellType(i, j, static_cast<CellType>(in[i + j * g.sizeX()]));
}

void fso_get_fluid_indices(const fso_sim* s, int32_t* out)
{
    const FluidSolverMemoryPool& p = s->solver._mem_pool;
    for (int j = 0; j < p.sizeY(); ++j)
        for (int i = 0; i < p.sizeX(); ++i) out[i + j * p.sizeX()] = p.fluid_indices.value(i, j);
}

void fso_get_particle_counts(const fso_sim* s, uint8_t* out)
{
    const FluidSolverMemoryPool& p = s->solver._mem_pool;
    for (int j = 0; j < p.sizeY(); ++j)
        for (int i = 0; i < p.sizeX(); ++i) out[i + j * p.sizeX()] = p.n_particles.value(i, j);
}

void fso_get_pressure(const fso_sim* s, float* out)
{
    const FluidSolverMemoryPool& p = s->solver._mem_pool;
    const int nx = p.sizeX(), ny = p.sizeY();
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            int k = p.fluid_indices.value(i, j);
            out[i + j * nx] = (k >= 0 && static_cast<size_t>(k) < s->pressure.size()) ? s->pressure[static_cast<size_t>(k)] : 0.0f;
        }
}

void fso_get_cg_stats(const fso_sim* s, int* iters, double* err, int* n_fluid)
{
    if (iters) *iters = s->cg_iters;
    if (err) *err = s->cg_error;
    if (n_fluid) *n_fluid = s->n_fluid;
}

int fso_phase(fso_sim* s, int ph, float dt) { return phase(s, ph, dt); }

int fso_step(fso_sim* s, int method, float dt)
{
    FluidDomain& d = s->domain;
    try {
        if (stock_ok(s)) {
            // The reference's own step functions.  The pressure solve inside
            // them is observed through the shim's record of the last solve.
            Eigen::fs_cg_record() = Eigen::FsCgRecord();
            Eigen::fs_cg_record().iterations = -1;
            switch (method) {
                case FSO_STEP_SEMI_LAGRANGIAN: s->solver.stepSemiLagrangian(d, dt); break;
                case FSO_STEP_PIC: s->solver.stepPIC(d, dt); break;
                case FSO_STEP_FLIP: s->solver.stepFLIP(d, dt); break;
                case FSO_STEP_PICFLIP: s->solver.stepPICFLIP(d, dt); break;
                default: return -2;
            }
            Eigen::FsCgRecord& rec = Eigen::fs_cg_record();
            if (rec.iterations < 0) {
                s->pressure.clear();
                s->cg_iters = 0;
                s->cg_error = 0.0;
                s->n_fluid = 0;
            } else {
                s->pressure.assign(rec.solution.begin(), rec.solution.end());
                s->cg_iters = static_cast<int>(rec.iterations);
                s->cg_error = rec.error;
                s->n_fluid = static_cast<int>(rec.solution.size());
            }
            return 0;
        }
        if (!s->solver.validate(d)) return -1;
        switch (method) {
            case FSO_STEP_SEMI_LAGRANGIAN:  // FluidSolver.cpp:109-133
                phase(s, FSO_PH_CLASSIFY, dt);
                phase(s, FSO_PH_SL_VELOCITY, dt);
                phase(s, FSO_PH_GRAVITY, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_PRESSURE, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_SL_PARTICLES, dt);
                break;
            case FSO_STEP_PIC:  // FluidSolver.cpp:146-169
                phase(s, FSO_PH_CLASSIFY, dt);
                phase(s, FSO_PH_P2G, dt);
                phase(s, FSO_PH_GRAVITY, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_EXTEND, dt);
                phase(s, FSO_PH_PRESSURE, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_G2P_PIC, dt);
                phase(s, FSO_PH_ADVECT, dt);
                break;
            case FSO_STEP_FLIP:  // FluidSolver.cpp:183-208
                phase(s, FSO_PH_CLASSIFY, dt);
                phase(s, FSO_PH_P2G, dt);
                phase(s, FSO_PH_SAVE_PREV, dt);
                phase(s, FSO_PH_GRAVITY, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_EXTEND, dt);
                phase(s, FSO_PH_PRESSURE, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_SAVE_DIFF, dt);
                phase(s, FSO_PH_G2P_FLIP, dt);
                phase(s, FSO_PH_ADVECT, dt);
                break;
            case FSO_STEP_PICFLIP:  // FluidSolver.cpp:223-250
                phase(s, FSO_PH_CLASSIFY, dt);
                phase(s, FSO_PH_P2G, dt);
                phase(s, FSO_PH_SAVE_PREV, dt);
                phase(s, FSO_PH_GRAVITY, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_EXTEND, dt);
                phase(s, FSO_PH_PRESSURE, dt);
                phase(s, FSO_PH_DIRICHLET, dt);
                phase(s, FSO_PH_SAVE_DIFF, dt);
                phase(s, FSO_PH_G2P_PICFLIP, dt);
                phase(s, FSO_PH_ADVECT_SAFE, dt);
                break;
            default: return -2;
        }
    } catch (const std::runtime_error&) {
        return -1;
    }
    return 0;
}

void fso_add_source(fso_sim* s, float x_min, float x_max, float y_min, float y_max, float dx, float dy,
                    float vx, float vy, float time_step, int max_spawns)
{
    BBox<MyFloat> box{x_min, x_max, y_min, y_max};
    s->domain.addFluidSource(FluidSource(box, dx, dy, vx, vy, time_step, max_spawns));
}

void fso_update(fso_sim* s, float dt) { s->domain.update(dt); }

void fso_clear_sources(fso_sim* s) { s->domain.clearFluidSources(); }

// The reference's Renderer on its Canvas, the canvas loaded from and stored
// back to rgb / colors.
void fso_render(fso_sim* s, int what, const float* area, int w, int h, float* rgb, float* colors)
{
    Canvas canvas(w, h);
    for (int j = 0; j < h; ++j)
        for (int i = 0; i < w; ++i) {
            const float* p = rgb + 3 * ((size_t)i + (size_t)j * w);
            canvas.setPixel(i, j, Color(p[0], p[1], p[2]));
        }
    canvas.setLineColor(Color(colors[0], colors[1], colors[2]));
    canvas.setFillColor(Color(colors[3], colors[4], colors[5]));
    Renderer r({area[0], area[1], area[2], area[3]});
    switch (what) {
        case FSO_RENDER_CLEAR: r.clearCanvas(canvas); break;
        case FSO_RENDER_CELLS: r.renderGridCellsToCanvas(s->domain.macGrid(), canvas); break;
        case FSO_RENDER_VELOCITIES: r.renderGridVelocitiesToCanvas(s->domain.macGrid(), canvas); break;
        case FSO_RENDER_PARTICLES: r.renderParticlesToCanvas(s->domain.markerParticleSet(), canvas); break;
        case FSO_RENDER_METABALLS: r.renderMetaBallsToCanvas(s->domain.markerParticleSet(), canvas); break;
        case FSO_RENDER_LEVEL_SET: r.renderLevelSetFunctionValuesToCanvas(s->domain.levelSet(), canvas); break;
        default: break;
    }
    for (int j = 0; j < h; ++j)
        for (int i = 0; i < w; ++i) {
            const Color c = canvas.pixel(i, j);
            float* p = rgb + 3 * ((size_t)i + (size_t)j * w);
            p[0] = c.r;
            p[1] = c.g;
            p[2] = c.b;
        }
    const Color lc = canvas.lineColor(), fc = canvas.fillColor();
    colors[0] = lc.r;
    colors[1] = lc.g;
    colors[2] = lc.b;
    colors[3] = fc.r;
    colors[4] = fc.g;
    colors[5] = fc.b;
}

// The byte conversion of Renderer::writeCanvasToPpm (Renderer.cpp:217-240),
// written out here because the reference writes it straight to a file.
void fso_canvas_bytes(const float* rgb, int64_t n, uint8_t* out)
{
    for (int64_t k = 0; k < 3 * n; ++k) out[k] = static_cast<unsigned char>(CLAMP(rgb[k], 0, 1) * 255);
}

void fso_get_level_set(const fso_sim* s, float* out)
{
    const LevelSet& L = s->domain.levelSet();
    for (int j = 0; j < L.sizeY(); ++j)
        for (int i = 0; i < L.sizeX(); ++i) out[i + (size_t)j * L.sizeX()] = L.value(i, j);
}

void fso_set_level_set(fso_sim* s, const float* in)
{
    LevelSet& L = s->domain.levelSet();
    for (int j = 0; j < L.sizeY(); ++j)
        for (int i = 0; i < L.sizeX(); ++i) L(i, j) = in[i + (size_t)j * L.sizeX()];
}

void fso_advect_level_set(fso_sim* s, float dt) { s->domain.advectLevelSet(dt); }

void fso_classify_level_set(fso_sim* s)
{
    s->domain.classifyCells(s->domain.levelSet());
    apply_solid_mask(s);
}

float fso_metaball_weight(int i, int j)
{
    const int radius = 5;
    MyFloat t = CLAMP(sqrt((i * i + j * j)) / radius, 0, 1);
    return gaussian(t, 0.4, 0);
}

}  // extern "C"
