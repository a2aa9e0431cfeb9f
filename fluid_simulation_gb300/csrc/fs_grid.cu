// Per-cell (per-face) kernels of the step: labelling, transfer finishing,
// forces, Dirichlet conditions, velocity extension, pressure assembly and
// projection.  One thread per cell (or particle) of every simulation of the launch domain,
// row-major local cell index c = i + j * nx.
#include "fs_domain.cuh"

namespace fs {
namespace {

// MacGrid::clearCellTypeBuffer (src/MacGrid.cpp:32-50): border SOLID, interior AIR.
struct LabelsClear
{
    uint8_t* lab;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        lab[s.co + c] = (i > 0 && j > 0 && i < s.g.nx - 1 && j < s.g.ny - 1) ? AIR : SOLID;
    }
};

// FluidDomain::classifyCells (src/FluidDomain.cpp:157-167): the cell of each
// particle, x = (int)((px / lengthX) * sizeX), clamped, becomes LIQUID.
struct LabelsFromParticles
{
    const float* px;
    const float* py;
    uint8_t* lab;
    __device__ void operator()(const Seg& s, int64_t k) const
    {
        const Geom& g = s.g;
        int x = trunc_i(fmul(fdiv(px[s.po + k], g.lx), (float)g.nx));
        int y = trunc_i(fmul(fdiv(py[s.po + k], g.ly), (float)g.ny));
        x = clampi(x, 0, g.nx - 1);
        y = clampi(y, 0, g.ny - 1);
        lab[s.co + x + (int64_t)y * g.nx] = LIQUID;
    }
};

// The two per-particle passes of a step over the same positions, fused:
// LabelsFromParticles (classifyCells) and CountParticles (pressureSolve's
// count).  A step moves no particle between the two, so the counts are the
// ones pressureSolve would take.
struct LabelsAndCounts
{
    const float* px;
    const float* py;
    uint8_t* lab;
    int32_t* counts;
    unsigned* warn;
    __device__ void operator()(const Seg& s, int64_t k) const
    {
        const Geom& g = s.g;
        const int x = trunc_i(fmul(fdiv(px[s.po + k], g.lx), (float)g.nx));
        const int y = trunc_i(fmul(fdiv(py[s.po + k], g.ly), (float)g.ny));
        lab[s.co + clampi(x, 0, g.nx - 1) + (int64_t)clampi(y, 0, g.ny - 1) * g.nx] = LIQUID;
        if (x >= 0 && x < g.nx && y >= 0 && y < g.ny)
            atomicAdd(&counts[s.co + x + (int64_t)y * g.nx], 1);
        else
            atomicOr(warn, FS_WARN_PARTICLE_OUTSIDE);
    }
};

// Border reset (src/FluidDomain.cpp:169-179) and the persistent solid mask.
struct LabelsFinalize
{
    uint8_t* lab;
    const uint8_t* solid;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        if (i == 0 || j == 0 || i == s.g.nx - 1 || j == s.g.ny - 1 || (solid && solid[s.co + c]))
            lab[s.co + c] = SOLID;
    }
};

// pressureSolve's particle count (src/FluidSolver.cpp:353-360), unclamped.
struct CountParticles
{
    const float* px;
    const float* py;
    int32_t* counts;
    unsigned* warn;
    __device__ void operator()(const Seg& s, int64_t k) const
    {
        const Geom& g = s.g;
        const int x = trunc_i(fmul(fdiv(px[s.po + k], g.lx), (float)g.nx));
        const int y = trunc_i(fmul(fdiv(py[s.po + k], g.ly), (float)g.ny));
        if (x >= 0 && x < g.nx && y >= 0 && y < g.ny)
            atomicAdd(&counts[s.co + x + (int64_t)y * g.nx], 1);
        else
            atomicOr(warn, FS_WARN_PARTICLE_OUTSIDE);
    }
};

// transferVelocityToGridSpread's normalisation (src/FluidSolver.cpp:898-917):
// faces whose weight is not above 1e-6 keep their previous back value.
struct P2GFinish
{
    const float *su, *wu, *sv, *wv;
    float *ub, *vb;
    __device__ void operator()(const Seg& s, int64_t c, int, int) const
    {
        const int64_t o = s.co + c;
        const float a = wu[o], b = wv[o];
        if ((double)a > 0.000001) ub[o] = fdiv(su[o], a);
        if ((double)b > 0.000001) vb[o] = fdiv(sv[o], b);
    }
};

struct Copy2
{
    const float *a0, *a1;
    float *b0, *b1;
    __device__ void operator()(const Seg& s, int64_t c, int, int) const
    {
        const int64_t o = s.co + c;
        b0[o] = a0[o];
        b1[o] = a1[o];
    }
};

// MacGrid::updateVelocityDiffBuffer (src/MacGrid.cpp:58-70).
struct Diff
{
    const float *uf, *vf, *up, *vp;
    float *ud, *vd;
    __device__ void operator()(const Seg& s, int64_t c, int, int) const
    {
        const int64_t o = s.co + c;
        ud[o] = fsub(uf[o], up[o]);
        vd[o] = fsub(vf[o], vp[o]);
    }
};

// FluidSolver::addExternalAcceleration (src/FluidSolver.cpp:276-295); a * dt
// is one float product, as :289-291.
struct Gravity
{
    const uint8_t* lab;
    float *uf, *vf;
    float dt;
    __device__ void operator()(const Seg& s, int64_t c, int, int) const
    {
        const int64_t o = s.co + c;
        if (lab[o] == LIQUID) {
            uf[o] = fadd(uf[o], fmul(s.gx, dt));
            vf[o] = fadd(vf[o], fmul(s.gy, dt));
        }
    }
};

// FluidSolver::enforceDirichlet (src/FluidSolver.cpp:297-321).
struct Dirichlet
{
    const uint8_t* lab;
    float *uf, *vf;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        const Geom& g = s.g;
        const uint8_t* L = lab + s.co;
        const int64_t o = s.co + c;
        const int im1 = clampi(i - 1, 0, g.nx - 1);
        const int jm1 = clampi(j - 1, 0, g.ny - 1);
        const bool here = L[c] == SOLID;
        const float u = uf[o];
        if ((cell_type(L, g, im1, j) == SOLID && u < 0) || (here && u > 0)) uf[o] = 0;
        const float v = vf[o];
        if ((cell_type(L, g, i, jm1) == SOLID && v < 0) || (here && v > 0)) vf[o] = 0;
    }
};

// extendVelocityIndividual, validity masks and buffer initialisation
// (src/FluidSolver.cpp:490-530).  The y-invalid branch zeroes the front x
// velocity (:527), as in the reference.
struct ExtendInit
{
    const uint8_t* lab;
    float *uf, *vf, *ub, *vb;
    uint8_t *mxf, *mxb, *myf, *myb;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        const uint8_t* L = lab + s.co;
        const int64_t o = s.co + c;
        const bool liq = L[c] == LIQUID;
        const bool vx = liq || cell_type(L, s.g, i - 1, j) == LIQUID;
        const bool vy = liq || cell_type(L, s.g, i, j - 1) == LIQUID;
        const float u = uf[o];
        mxf[o] = vx;
        mxb[o] = vx;
        ub[o] = vx ? u : 0.0f;
        myf[o] = vy;
        myb[o] = vy;
        vb[o] = vy ? vf[o] : 0.0f;
        if (!vx || !vy) uf[o] = 0.0f;
    }
};

// Gravity, Dirichlet and ExtendInit of one face in one pass, in the step's
// order (src/FluidSolver.cpp:230-232, 490-530): each reads and writes only
// its own face's velocities (and the labels), so the fusion changes nothing.
struct ForcesExtendInit
{
    Gravity gravity;
    Dirichlet dirichlet;
    ExtendInit init;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        gravity(s, c, i, j);
        dirichlet(s, c, i, j);
        init(s, c, i, j);
    }
};

// One extension sweep (src/FluidSolver.cpp:533-619): invalid non-solid faces
// take the average of their valid neighbours, in the neighbour order
// (i-1, j), (i, j-1), (i, j+1), (i+1, j).  Reads only faces valid in the
// front mask and writes only faces invalid in it, so the in-place update of
// the back velocities is race-free.
struct ExtendSweep
{
    const uint8_t* lab;
    float *ub, *vb;
    const uint8_t* mxf;
    uint8_t* mxb;
    const uint8_t* myf;
    uint8_t* myb;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        const Geom& g = s.g;
        const int nx = g.nx;
        // Faces on the grid border never pass the tests below when the border is
        // SOLID (as classification guarantees); for other label fields the
        // reference would read outside the grid, so they are left alone here.
        if (i == 0 || j == 0 || i == g.nx - 1 || j == g.ny - 1) return;
        const uint8_t* L = lab + s.co;
        const uint8_t* MX = mxf + s.co;
        const uint8_t* MY = myf + s.co;
        float* UB = ub + s.co;
        float* VB = vb + s.co;
        const bool here_solid = L[c] == SOLID;
        if (MX[c] == 0 && !here_solid && cell_type(L, g, i - 1, j) != SOLID) {
            float nv = 0.0f;
            int nn = 0;
            if (MX[c - 1] == 1) { nv = fadd(nv, UB[c - 1]); ++nn; }
            if (MX[c - nx] == 1) { nv = fadd(nv, UB[c - nx]); ++nn; }
            if (MX[c + nx] == 1) { nv = fadd(nv, UB[c + nx]); ++nn; }
            if (MX[c + 1] == 1) { nv = fadd(nv, UB[c + 1]); ++nn; }
            if (nn > 0) {
                UB[c] = fdiv(nv, (float)nn);
                mxb[s.co + c] = 1;
            }
        }
        if (MY[c] == 0 && !here_solid && cell_type(L, g, i, j - 1) != SOLID) {
            float nv = 0.0f;
            int nn = 0;
            if (MY[c - 1] == 1) { nv = fadd(nv, VB[c - 1]); ++nn; }
            if (MY[c - nx] == 1) { nv = fadd(nv, VB[c - nx]); ++nn; }
            if (MY[c + nx] == 1) { nv = fadd(nv, VB[c + nx]); ++nn; }
            if (MY[c + 1] == 1) { nv = fadd(nv, VB[c + 1]); ++nn; }
            if (nn > 0) {
                VB[c] = fdiv(nv, (float)nn);
                myb[s.co + c] = 1;
            }
        }
    }
};

// pressureSolve assembly (src/FluidSolver.cpp:363-416), thread t = fluid cell
// t: divergence b[t] (MacGrid::divVelX + divVelY, include/MacGrid.h:98-111)
// and the row of A (matrix_row).  Also the uint8 particle counts of all cells
// (:344, :359).
struct Assemble
{
    const uint8_t* lab;
    const int32_t *fidx, *cell_of, *nfluid;
    const float *uf, *vf;
    float* b;
    int32_t *down, *up;
    uint8_t* flags;
    const int32_t* counts32;
    uint8_t* counts8;
    __device__ void operator()(const Seg& s, int64_t t, int, int) const
    {
        const Geom& g = s.g;
        const int nf = nfluid[s.sim];
        const int64_t o = s.co;
        counts8[o + t] = nf > 0 ? (uint8_t)(counts32[o + t] & 255) : (uint8_t)0;
        if (t >= nf) return;
        const int64_t c = cell_of[o + t];
        const int i = (int)(c % g.nx), j = (int)(c / g.nx);
        matrix_row(lab + o, g, fidx + o, c, i, j, flags[o + t], down[o + t], up[o + t]);
        const float* U = uf + o;
        const float* V = vf + o;
        const float u1 = i < g.nx - 1 ? U[c + 1] : 0.0f;
        const float v1 = j < g.ny - 1 ? V[c + g.nx] : 0.0f;
        const float ddx = fdiv(fsub(u1, U[c]), g.dx);
        const float ddy = fdiv(fsub(v1, V[c]), g.dy);
        b[o + t] = fadd(ddx, ddy);
    }
};

// pressureSolve's velocity update (src/FluidSolver.cpp:428-482) into the back
// buffers on faces with a fluid cell on either side; the volume-loss term is
// multiplied by k = 0 and contributes +0; dt / density is formed first
// (:471-474).  With no fluid cell the reference returns before updating and
// swapping (:347-350); the buffers' contents are exchanged here so that the
// caller's unconditional swap leaves them as they were.
struct Project
{
    const int32_t *fidx, *nfluid;
    const float* x;
    float *uf, *vf, *ub, *vb;
    float dt;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        const Geom& g = s.g;
        const int64_t o = s.co + c;
        if (nfluid[s.sim] == 0) {
            const float a = uf[o], b = ub[o], cc = vf[o], d = vb[o];
            uf[o] = b;
            ub[o] = a;
            vf[o] = d;
            vb[o] = cc;
            return;
        }
        const int32_t* F = fidx + s.co;
        const float* X = x + s.co;
        const int im1 = clampi(i - 1, 0, g.nx - 1);
        const int jm1 = clampi(j - 1, 0, g.ny - 1);
        const int idx = F[c];
        const int idx_im1 = F[im1 + (int64_t)j * g.nx];
        const int idx_jm1 = F[i + (int64_t)jm1 * g.nx];
        if (idx >= 0 || idx_im1 >= 0 || idx_jm1 >= 0) {
            const float dt_over_rho = fdiv(dt, s.rho);
            const float p = idx >= 0 ? fadd(X[idx], 0.0f) : 0.0f;
            const float p_im1 = idx_im1 >= 0 ? fadd(X[idx_im1], 0.0f) : 0.0f;
            const float p_jm1 = idx_jm1 >= 0 ? fadd(X[idx_jm1], 0.0f) : 0.0f;
            const float dpx = fsub(p, p_im1);
            const float dpy = fsub(p, p_jm1);
            ub[o] = fsub(uf[o], fdiv(fmul(dt_over_rho, dpx), g.dx));
            vb[o] = fsub(vf[o], fdiv(fmul(dt_over_rho, dpy), g.dy));
        }
    }
};

struct PressureToGrid
{
    const int32_t *fidx, *nfluid;
    const float* x;
    float* out;
    __device__ void operator()(const Seg& s, int64_t c, int, int) const
    {
        const int k = fidx[s.co + c];
        out[s.co + c] = (k >= 0 && k < nfluid[s.sim]) ? x[s.co + k] : 0.0f;
    }
};

// A grid element by its linear index; 0 past the end of the array (where the
// reference's std::vector read is undefined).
__device__ __forceinline__ float at_lin(const float* a, int64_t idx, int64_t n) { return idx < n ? a[idx] : 0.0f; }

// FluidDomain::advectLevelSet (src/FluidDomain.cpp:104-125) as written: its
// loops run j < sizeX, i < sizeY, so for size_x != size_y several iterations
// can write one element; element e takes the last of them in loop order
// (largest j), whose linear index i + j * size_x is e itself.  MacGrid::velX /
// velY (include/MacGrid.h:30-39) average a face with the next one through the
// linear index; LevelSet::computeUpwindGradient{X,Y} (src/LevelSet.cpp:27-59)
// clamp through float.
struct AdvectLevelSet
{
    const float *ls, *uf, *vf;
    float* out;
    float dt;
    __device__ void operator()(const Seg& s, int64_t e, int, int) const
    {
        const Geom& g = s.g;
        const int64_t n = (int64_t)g.nx * g.ny;
        const int jt = (int)min((int64_t)(g.nx - 1), e / g.nx);
        const int it = (int)(e - (int64_t)jt * g.nx);
        if (it >= g.ny) {  // no iteration writes e: the new LevelSet's 0
            out[e] = 0.0f;
            return;
        }
        const float vel_x = fdiv(fadd(at_lin(uf, e, n), at_lin(uf, e + 1, n)), 2.0f);
        const float vel_y = fdiv(fadd(at_lin(vf, e, n), at_lin(vf, e + g.nx, n)), 2.0f);
        auto L = [&](int i, int j) { return ls[(int64_t)i + (int64_t)j * g.nx]; };
        const int i = clampi(it, 0, g.nx - 1), j = clampi(jt, 0, g.ny - 1);
        const int ip = clampi(it + 1, 0, g.nx - 1), im = clampi(it - 1, 0, g.nx - 1);
        const int jp = clampi(jt + 1, 0, g.ny - 1), jm = clampi(jt - 1, 0, g.ny - 1);
        const float gx = vel_x < 0 ? fsub(L(ip, j), L(i, j)) : fsub(L(i, j), L(im, j));
        const float gy = vel_y < 0 ? fsub(L(i, jp), L(i, j)) : fsub(L(i, j), L(i, jm));
        const float change = -fadd(fmul(vel_x, gx), fmul(vel_y, gy));
        out[e] = fadd(at_lin(ls, e, n), fmul(fmul(change, dt), 5.0f));
    }
};

// FluidDomain::classifyCells(LevelSet&) (src/FluidDomain.cpp:127-148), then
// the persistent solid mask.
struct ClassifyLevelSet
{
    const float* ls;
    uint8_t* lab;
    const uint8_t* solid;
    __device__ void operator()(const Seg& s, int64_t c, int i, int j) const
    {
        const bool border = i == 0 || j == 0 || i == s.g.nx - 1 || j == s.g.ny - 1;
        uint8_t t = ls[c] < 0 ? LIQUID : AIR;
        if (border || (solid && solid[c])) t = SOLID;
        lab[c] = t;
    }
};

}  // namespace

void advect_level_set(const Launch& L, const Domain& d, const float* ls, const float* uf, const float* vf, float dt,
                      float* out)
{
    each_cell(L, d, AdvectLevelSet{ls, uf, vf, out, dt});
}

void classify_level_set(const Launch& L, const Domain& d, const float* ls, uint8_t* lab, const uint8_t* solid)
{
    each_cell(L, d, ClassifyLevelSet{ls, lab, solid});
}

void labels_clear(const Launch& L, const Domain& d, uint8_t* lab) { each_cell(L, d, LabelsClear{lab}); }

void labels_from_particles(const Launch& L, const Domain& d, const float* px, const float* py, uint8_t* lab)
{
    each_particle(L, d, LabelsFromParticles{px, py, lab});
}

void labels_finalize(const Launch& L, const Domain& d, uint8_t* lab, const uint8_t* solid)
{
    each_cell(L, d, LabelsFinalize{lab, solid});
}

void labels_and_counts(const Launch& L, const Domain& d, const float* px, const float* py, uint8_t* lab,
                       int32_t* counts32, unsigned* warn)
{
    cudaMemsetAsync(counts32, 0, sizeof(int32_t) * (size_t)d.cells, L.stream);
    each_particle(L, d, LabelsAndCounts{px, py, lab, counts32, warn});
}

void forces_extend_init(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf, float dt,
                        float* ub, float* vb, uint8_t* mxf, uint8_t* mxb, uint8_t* myf, uint8_t* myb)
{
    each_cell(L, d,
              ForcesExtendInit{Gravity{lab, uf, vf, dt}, Dirichlet{lab, uf, vf},
                               ExtendInit{lab, uf, vf, ub, vb, mxf, mxb, myf, myb}});
}

void count_particles(const Launch& L, const Domain& d, const float* px, const float* py, int32_t* counts32,
                     unsigned* warn)
{
    cudaMemsetAsync(counts32, 0, sizeof(int32_t) * (size_t)d.cells, L.stream);
    each_particle(L, d, CountParticles{px, py, counts32, warn});
}

void p2g_finish(const Launch& L, const Domain& d, const float* su, const float* wu, const float* sv, const float* wv,
                float* ub, float* vb)
{
    each_cell(L, d, P2GFinish{su, wu, sv, wv, ub, vb});
}

void grid_copy2(const Launch& L, const Domain& d, const float* a0, const float* a1, float* b0, float* b1)
{
    each_cell(L, d, Copy2{a0, a1, b0, b1});
}

void grid_diff(const Launch& L, const Domain& d, const float* uf, const float* vf, const float* up, const float* vp,
               float* ud, float* vd)
{
    each_cell(L, d, Diff{uf, vf, up, vp, ud, vd});
}

void gravity(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf, float dt)
{
    each_cell(L, d, Gravity{lab, uf, vf, dt});
}

void dirichlet(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf)
{
    each_cell(L, d, Dirichlet{lab, uf, vf});
}

void extend_init(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf, float* ub, float* vb,
                 uint8_t* mxf, uint8_t* mxb, uint8_t* myf, uint8_t* myb)
{
    each_cell(L, d, ExtendInit{lab, uf, vf, ub, vb, mxf, mxb, myf, myb});
}

void extend_sweep(const Launch& L, const Domain& d, const uint8_t* lab, float* ub, float* vb, const uint8_t* mxf,
                  uint8_t* mxb, const uint8_t* myf, uint8_t* myb)
{
    each_cell(L, d, ExtendSweep{lab, ub, vb, mxf, mxb, myf, myb});
}

void assemble(const Launch& L, const Domain& d, const uint8_t* lab, const int32_t* fidx, const int32_t* cell_of,
              const int32_t* nfluid, const float* uf, const float* vf, float* b, int32_t* down, int32_t* up,
              uint8_t* flags, const int32_t* counts32, uint8_t* counts8)
{
    each_cell(L, d, Assemble{lab, fidx, cell_of, nfluid, uf, vf, b, down, up, flags, counts32, counts8});
}

void project(const Launch& L, const Domain& d, const int32_t* fidx, const int32_t* nfluid, const float* x, float* uf,
             float* vf, float* ub, float* vb, float dt)
{
    each_cell(L, d, Project{fidx, nfluid, x, uf, vf, ub, vb, dt});
}

void pressure_to_grid(const Launch& L, const Domain& d, const int32_t* fidx, const int32_t* nfluid, const float* x,
                      float* out)
{
    each_cell(L, d, PressureToGrid{fidx, nfluid, x, out});
}

}  // namespace fs
