// Per-cell (per-face) kernels of the step: labelling, transfer finishing,
// forces, Dirichlet conditions, velocity extension, pressure assembly and
// projection.  One thread per cell, row-major cell index c = i + j * nx.
#include "fs_internal.h"

namespace fs {
namespace {

constexpr int TPB = 256;

__device__ __forceinline__ bool cell_index(const Geom& g, int64_t& c, int& i, int& j)
{
    c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)g.nx * g.ny) return false;
    i = (int)(c % g.nx);
    j = (int)(c / g.nx);
    return true;
}

unsigned cell_blocks(const Geom& g) { return (unsigned)(((int64_t)g.nx * g.ny + TPB - 1) / TPB); }

// MacGrid::clearCellTypeBuffer (src/MacGrid.cpp:32-50): border SOLID, interior AIR.
__global__ void k_labels_clear(Geom g, uint8_t* __restrict__ lab)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    lab[c] = (i > 0 && j > 0 && i < g.nx - 1 && j < g.ny - 1) ? AIR : SOLID;
}

// FluidDomain::classifyCells (src/FluidDomain.cpp:157-167): the cell of each
// particle, x = (int)((px / lengthX) * sizeX), clamped, becomes LIQUID.
__global__ void k_labels_particles(Geom g, const float* __restrict__ px, const float* __restrict__ py, int64_t n,
                                   uint8_t* __restrict__ lab)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int x = trunc_i(fmul(fdiv(px[k], g.lx), (float)g.nx));
    int y = trunc_i(fmul(fdiv(py[k], g.ly), (float)g.ny));
    x = clampi(x, 0, g.nx - 1);
    y = clampi(y, 0, g.ny - 1);
    lab[x + (int64_t)y * g.nx] = LIQUID;
}

// Border reset (src/FluidDomain.cpp:169-179) and the persistent solid mask.
__global__ void k_labels_finalize(Geom g, uint8_t* __restrict__ lab, const uint8_t* __restrict__ solid)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    if (i == 0 || j == 0 || i == g.nx - 1 || j == g.ny - 1 || (solid && solid[c])) lab[c] = SOLID;
}

// pressureSolve's particle count (src/FluidSolver.cpp:353-360), unclamped.
__global__ void k_count_particles(Geom g, const float* __restrict__ px, const float* __restrict__ py, int64_t n,
                                  int32_t* __restrict__ counts, unsigned* __restrict__ warn)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int x = trunc_i(fmul(fdiv(px[k], g.lx), (float)g.nx));
    const int y = trunc_i(fmul(fdiv(py[k], g.ly), (float)g.ny));
    if (x >= 0 && x < g.nx && y >= 0 && y < g.ny)
        atomicAdd(&counts[x + (int64_t)y * g.nx], 1);
    else
        atomicOr(warn, FS_WARN_PARTICLE_OUTSIDE);
}

// transferVelocityToGridSpread's normalisation (src/FluidSolver.cpp:898-917):
// faces whose weight is not above 1e-6 keep their previous back value.
__global__ void k_p2g_finish(Geom g, const float* __restrict__ su, const float* __restrict__ wu,
                             const float* __restrict__ sv, const float* __restrict__ wv, float* __restrict__ ub,
                             float* __restrict__ vb)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    const float a = wu[c], b = wv[c];
    if ((double)a > 0.000001) ub[c] = fdiv(su[c], a);
    if ((double)b > 0.000001) vb[c] = fdiv(sv[c], b);
}

__global__ void k_copy2(Geom g, const float* __restrict__ a0, const float* __restrict__ a1, float* __restrict__ b0,
                        float* __restrict__ b1)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    b0[c] = a0[c];
    b1[c] = a1[c];
}

// MacGrid::updateVelocityDiffBuffer (src/MacGrid.cpp:58-70).
__global__ void k_diff(Geom g, const float* __restrict__ uf, const float* __restrict__ vf,
                       const float* __restrict__ up, const float* __restrict__ vp, float* __restrict__ ud,
                       float* __restrict__ vd)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    ud[c] = fsub(uf[c], up[c]);
    vd[c] = fsub(vf[c], vp[c]);
}

// FluidSolver::addExternalAcceleration (src/FluidSolver.cpp:276-295).
__global__ void k_gravity(Geom g, const uint8_t* __restrict__ lab, float* __restrict__ uf, float* __restrict__ vf,
                          float ax_dt, float ay_dt)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    if (lab[c] == LIQUID) {
        uf[c] = fadd(uf[c], ax_dt);
        vf[c] = fadd(vf[c], ay_dt);
    }
}

// FluidSolver::enforceDirichlet (src/FluidSolver.cpp:297-321).
__global__ void k_dirichlet(Geom g, const uint8_t* __restrict__ lab, float* __restrict__ uf, float* __restrict__ vf)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    const int im1 = clampi(i - 1, 0, g.nx - 1);
    const int jm1 = clampi(j - 1, 0, g.ny - 1);
    const bool here = lab[c] == SOLID;
    const float u = uf[c];
    if ((cell_type(lab, g, im1, j) == SOLID && u < 0) || (here && u > 0)) uf[c] = 0;
    const float v = vf[c];
    if ((cell_type(lab, g, i, jm1) == SOLID && v < 0) || (here && v > 0)) vf[c] = 0;
}

// extendVelocityIndividual, validity masks and buffer initialisation
// (src/FluidSolver.cpp:490-530).  The y-invalid branch zeroes the front x
// velocity (:527), as in the reference.
__global__ void k_extend_init(Geom g, const uint8_t* __restrict__ lab, float* __restrict__ uf,
                              float* __restrict__ vf, float* __restrict__ ub, float* __restrict__ vb,
                              uint8_t* __restrict__ mxf, uint8_t* __restrict__ mxb, uint8_t* __restrict__ myf,
                              uint8_t* __restrict__ myb)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    const bool liq = lab[c] == LIQUID;
    const bool vx = liq || cell_type(lab, g, i - 1, j) == LIQUID;
    const bool vy = liq || cell_type(lab, g, i, j - 1) == LIQUID;
    const float u = uf[c];
    mxf[c] = vx;
    mxb[c] = vx;
    ub[c] = vx ? u : 0.0f;
    myf[c] = vy;
    myb[c] = vy;
    vb[c] = vy ? vf[c] : 0.0f;
    if (!vx || !vy) uf[c] = 0.0f;
}

// One extension sweep (src/FluidSolver.cpp:533-619): invalid non-solid faces
// take the average of their valid neighbours, in the neighbour order
// (i-1, j), (i, j-1), (i, j+1), (i+1, j).  Reads only faces valid in the
// front mask and writes only faces invalid in it, so the in-place update of
// the back velocities is race-free.
__global__ void k_extend_sweep(Geom g, const uint8_t* __restrict__ lab, float* ub, float* vb,
                               const uint8_t* __restrict__ mxf, uint8_t* __restrict__ mxb,
                               const uint8_t* __restrict__ myf, uint8_t* __restrict__ myb)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    const int nx = g.nx;
    // Faces on the grid border never pass the tests below when the border is
    // SOLID (as classification guarantees); for other label fields the
    // reference would read outside the grid, so they are left alone here.
    if (i == 0 || j == 0 || i == g.nx - 1 || j == g.ny - 1) return;
    const bool here_solid = lab[c] == SOLID;
    if (mxf[c] == 0 && !here_solid && cell_type(lab, g, i - 1, j) != SOLID) {
        float nv = 0.0f;
        int nn = 0;
        if (mxf[c - 1] == 1) { nv = fadd(nv, ub[c - 1]); ++nn; }
        if (mxf[c - nx] == 1) { nv = fadd(nv, ub[c - nx]); ++nn; }
        if (mxf[c + nx] == 1) { nv = fadd(nv, ub[c + nx]); ++nn; }
        if (mxf[c + 1] == 1) { nv = fadd(nv, ub[c + 1]); ++nn; }
        if (nn > 0) {
            ub[c] = fdiv(nv, (float)nn);
            mxb[c] = 1;
        }
    }
    if (myf[c] == 0 && !here_solid && cell_type(lab, g, i, j - 1) != SOLID) {
        float nv = 0.0f;
        int nn = 0;
        if (myf[c - 1] == 1) { nv = fadd(nv, vb[c - 1]); ++nn; }
        if (myf[c - nx] == 1) { nv = fadd(nv, vb[c - nx]); ++nn; }
        if (myf[c + nx] == 1) { nv = fadd(nv, vb[c + nx]); ++nn; }
        if (myf[c + 1] == 1) { nv = fadd(nv, vb[c + 1]); ++nn; }
        if (nn > 0) {
            vb[c] = fdiv(nv, (float)nn);
            myb[c] = 1;
        }
    }
}

// pressureSolve assembly (src/FluidSolver.cpp:363-416), one thread per fluid
// cell k: divergence b[k] (MacGrid::divVelX + divVelY, include/MacGrid.h:98-111)
// and the row of A as flags: bit 0 / bit 1 = liquid left / right neighbour
// (fluid indices k-1 / k+1 in the j-major order), bits 2-4 = number of
// non-solid neighbours n (diagonal -n / dx^2); down / up fluid indices or -1.
// Also the uint8 particle counts of all cells (:344, :359).
__global__ void k_assemble(Geom g, const uint8_t* __restrict__ lab, const int32_t* __restrict__ fidx,
                           const int32_t* __restrict__ cell_of, const int32_t* __restrict__ nfluid,
                           const float* __restrict__ uf, const float* __restrict__ vf, float* __restrict__ b,
                           int32_t* __restrict__ down, int32_t* __restrict__ up, uint8_t* __restrict__ flags,
                           const int32_t* __restrict__ counts32, uint8_t* __restrict__ counts8)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ncell = (int64_t)g.nx * g.ny;
    const int nf = *nfluid;
    if (t < ncell) counts8[t] = nf > 0 ? (uint8_t)(counts32[t] & 255) : (uint8_t)0;
    if (t >= nf) return;
    const int64_t c = cell_of[t];
    const int i = (int)(c % g.nx), j = (int)(c / g.nx);
    matrix_row(lab, g, fidx, c, i, j, flags[t], down[t], up[t]);
    const float u1 = i < g.nx - 1 ? uf[c + 1] : 0.0f;
    const float v1 = j < g.ny - 1 ? vf[c + g.nx] : 0.0f;
    const float ddx = fdiv(fsub(u1, uf[c]), g.dx);
    const float ddy = fdiv(fsub(v1, vf[c]), g.dy);
    b[t] = fadd(ddx, ddy);
}

// pressureSolve's velocity update (src/FluidSolver.cpp:428-482) into the back
// buffers on faces with a fluid cell on either side; the volume-loss term is
// multiplied by k = 0 and contributes +0.  With no fluid cell the reference
// returns before updating and swapping (:347-350); the buffers' contents are
// exchanged here so that the caller's unconditional swap leaves them as they were.
__global__ void k_project(Geom g, const int32_t* __restrict__ fidx, const int32_t* __restrict__ nfluid,
                          const float* __restrict__ x, float* __restrict__ uf, float* __restrict__ vf,
                          float* __restrict__ ub, float* __restrict__ vb, float dt_over_rho)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    if (*nfluid == 0) {
        const float a = uf[c], b = ub[c], cc = vf[c], d = vb[c];
        uf[c] = b;
        ub[c] = a;
        vf[c] = d;
        vb[c] = cc;
        return;
    }
    const int im1 = clampi(i - 1, 0, g.nx - 1);
    const int jm1 = clampi(j - 1, 0, g.ny - 1);
    const int idx = fidx[c];
    const int idx_im1 = fidx[im1 + (int64_t)j * g.nx];
    const int idx_jm1 = fidx[i + (int64_t)jm1 * g.nx];
    if (idx >= 0 || idx_im1 >= 0 || idx_jm1 >= 0) {
        const float p = idx >= 0 ? fadd(x[idx], 0.0f) : 0.0f;
        const float p_im1 = idx_im1 >= 0 ? fadd(x[idx_im1], 0.0f) : 0.0f;
        const float p_jm1 = idx_jm1 >= 0 ? fadd(x[idx_jm1], 0.0f) : 0.0f;
        const float dpx = fsub(p, p_im1);
        const float dpy = fsub(p, p_jm1);
        ub[c] = fsub(uf[c], fdiv(fmul(dt_over_rho, dpx), g.dx));
        vb[c] = fsub(vf[c], fdiv(fmul(dt_over_rho, dpy), g.dy));
    }
}

__global__ void k_pressure_to_grid(Geom g, const int32_t* __restrict__ fidx, const int32_t* __restrict__ nfluid,
                                   const float* __restrict__ x, float* __restrict__ out)
{
    int64_t c;
    int i, j;
    if (!cell_index(g, c, i, j)) return;
    const int k = fidx[c];
    out[c] = (k >= 0 && k < *nfluid) ? x[k] : 0.0f;
}

}  // namespace

void labels_clear(const Launch& L, const Geom& g, uint8_t* lab)
{
    k_labels_clear<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab);
    L.count();
}

void labels_from_particles(const Launch& L, const Geom& g, const float* px, const float* py, int64_t n, uint8_t* lab)
{
    if (n <= 0) return;
    k_labels_particles<<<(unsigned)((n + TPB - 1) / TPB), TPB, 0, L.stream>>>(g, px, py, n, lab);
    L.count();
}

void labels_finalize(const Launch& L, const Geom& g, uint8_t* lab, const uint8_t* solid)
{
    k_labels_finalize<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab, solid);
    L.count();
}

void count_particles(const Launch& L, const Geom& g, const float* px, const float* py, int64_t n, int32_t* counts32,
                     unsigned* warn)
{
    cudaMemsetAsync(counts32, 0, sizeof(int32_t) * (size_t)g.nx * g.ny, L.stream);
    if (n <= 0) return;
    k_count_particles<<<(unsigned)((n + TPB - 1) / TPB), TPB, 0, L.stream>>>(g, px, py, n, counts32, warn);
    L.count();
}

void p2g_finish(const Launch& L, const Geom& g, const float* su, const float* wu, const float* sv, const float* wv,
                float* ub, float* vb)
{
    k_p2g_finish<<<cell_blocks(g), TPB, 0, L.stream>>>(g, su, wu, sv, wv, ub, vb);
    L.count();
}

void grid_copy2(const Launch& L, const Geom& g, const float* a0, const float* a1, float* b0, float* b1)
{
    k_copy2<<<cell_blocks(g), TPB, 0, L.stream>>>(g, a0, a1, b0, b1);
    L.count();
}

void grid_diff(const Launch& L, const Geom& g, const float* uf, const float* vf, const float* up, const float* vp,
               float* ud, float* vd)
{
    k_diff<<<cell_blocks(g), TPB, 0, L.stream>>>(g, uf, vf, up, vp, ud, vd);
    L.count();
}

void gravity(const Launch& L, const Geom& g, const uint8_t* lab, float* uf, float* vf, float ax_dt, float ay_dt)
{
    k_gravity<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab, uf, vf, ax_dt, ay_dt);
    L.count();
}

void dirichlet(const Launch& L, const Geom& g, const uint8_t* lab, float* uf, float* vf)
{
    k_dirichlet<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab, uf, vf);
    L.count();
}

void extend_init(const Launch& L, const Geom& g, const uint8_t* lab, float* uf, float* vf, float* ub, float* vb,
                 uint8_t* mxf, uint8_t* mxb, uint8_t* myf, uint8_t* myb)
{
    k_extend_init<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab, uf, vf, ub, vb, mxf, mxb, myf, myb);
    L.count();
}

void extend_sweep(const Launch& L, const Geom& g, const uint8_t* lab, float* ub, float* vb, const uint8_t* mxf,
                  uint8_t* mxb, const uint8_t* myf, uint8_t* myb)
{
    k_extend_sweep<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab, ub, vb, mxf, mxb, myf, myb);
    L.count();
}

void assemble(const Launch& L, const Geom& g, const uint8_t* lab, const int32_t* fidx, const int32_t* cell_of,
              const int32_t* nfluid, const float* uf, const float* vf, float* b, int32_t* down, int32_t* up,
              uint8_t* flags, const int32_t* counts32, uint8_t* counts8)
{
    k_assemble<<<cell_blocks(g), TPB, 0, L.stream>>>(g, lab, fidx, cell_of, nfluid, uf, vf, b, down, up, flags,
                                                     counts32, counts8);
    L.count();
}

void project(const Launch& L, const Geom& g, const int32_t* fidx, const int32_t* nfluid, const float* x, float* uf,
             float* vf, float* ub, float* vb, float dt_over_rho)
{
    k_project<<<cell_blocks(g), TPB, 0, L.stream>>>(g, fidx, nfluid, x, uf, vf, ub, vb, dt_over_rho);
    L.count();
}

void pressure_to_grid(const Launch& L, const Geom& g, const int32_t* fidx, const int32_t* nfluid, const float* x,
                      float* out)
{
    k_pressure_to_grid<<<cell_blocks(g), TPB, 0, L.stream>>>(g, fidx, nfluid, x, out);
    L.count();
}

}  // namespace fs
