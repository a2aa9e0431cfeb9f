// Multigrid-preconditioned conjugate gradient for the pressure system of
// FluidSolver::pressureSolve (src/FluidSolver.cpp:363-425): the same matrix
// (off-diagonal 1 / dx^2 to liquid neighbours, diagonal -(non-solid
// neighbours) / dx^2, AIR neighbours as p = 0), solved on the cell grid with
// a geometric V-cycle as preconditioner.  Not in the reference: it needs far
// fewer iterations than the Jacobi-preconditioned CG (the reference's, kept
// bit-exact elsewhere) and gives a different, equally converged, solution.
//
// Levels halve the grid until it is at most 16 cells a side.  A coarse cell
// is AIR if any of its (up to four) children is AIR, else LIQUID if any child
// is LIQUID, else SOLID; the operator is re-discretised with twice the
// spacing.  Smoothing is damped Jacobi (omega = 2/3; two sweeps before and
// after), restriction averages the children's residuals, prolongation copies
// the coarse correction to the children, and the coarsest level takes 64
// Jacobi sweeps in one CTA, so the V-cycle is a fixed symmetric linear
// operator.  The CG runs on -A (positive) with dot products accumulated in
// double along a fixed order; its scalars stay on the device and every kernel
// of an iteration returns at once after convergence, so chunks of iterations
// are replayed from one CUDA graph and the host only polls a flag.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fs_mg.h"

namespace fs {
namespace {

constexpr int TPB = 256;
constexpr int COARSE = 16;
constexpr int COARSE_SWEEPS = 64;
constexpr float OMEGA = 2.0f / 3.0f;
constexpr int CHUNK = 8;  // CG iterations per graph replay

unsigned nblk(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

struct Level
{
    int nx, ny;
    float inv_h2;   // 1 / h^2 of this level
    uint8_t* type;  // LIQUID / AIR / SOLID
    float *x, *b, *r;
};

// Scalars of the CG on the device.
struct Scal
{
    double pq, rr, rz, bb, thr;
    float alpha, beta;
    int it, done, maxit;
};

__device__ __forceinline__ uint8_t type_at(const Level& L, int i, int j)
{
    if (i < 0 || j < 0 || i >= L.nx || j >= L.ny) return SOLID;
    return L.type[i + (int64_t)j * L.nx];
}

// (-A x)_c for a LIQUID cell: (n x_c - sum of liquid neighbours) / h^2.
__device__ __forceinline__ float neg_apply(const Level& L, const float* __restrict__ x, int i, int j, float& diag)
{
    const int64_t c = i + (int64_t)j * L.nx;
    int n = 0;
    float s = 0.0f;
    const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint8_t t = type_at(L, i + di[k], j + dj[k]);
        if (t != SOLID) {
            ++n;
            if (t == LIQUID) s += x[c + di[k] + (int64_t)dj[k] * L.nx];
        }
    }
    diag = (float)n * L.inv_h2;
    return ((float)n * x[c] - s) * L.inv_h2;
}

__global__ void k_types0(int64_t n, const uint8_t* __restrict__ labels, uint8_t* __restrict__ type)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c < n) type[c] = labels[c];
}

__global__ void k_coarsen_types(Level F, Level C)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)C.nx * C.ny) return;
    const int I = (int)(c % C.nx), J = (int)(c / C.nx);
    bool air = false, liq = false;
    for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
            const int i = 2 * I + di, j = 2 * J + dj;
            if (i >= F.nx || j >= F.ny) continue;
            const uint8_t t = F.type[i + (int64_t)j * F.nx];
            air |= t == AIR;
            liq |= t == LIQUID;
        }
    C.type[c] = air ? AIR : liq ? LIQUID : SOLID;
}

// Damped Jacobi sweep: x_out = x_in + omega D^-1 (b - (-A) x_in) on LIQUID
// cells (x_in == nullptr: a zero initial guess); others 0.
__global__ void k_smooth(Level L, const float* __restrict__ xin, float* __restrict__ xout, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)L.nx * L.ny) return;
    if (L.type[c] != LIQUID) {
        xout[c] = 0.0f;
        return;
    }
    const int i = (int)(c % L.nx), j = (int)(c / L.nx);
    float diag = 0.0f, ax = 0.0f;
    if (xin) ax = neg_apply(L, xin, i, j, diag);
    else {
        int n = 0;
        const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
        for (int k = 0; k < 4; ++k) n += type_at(L, i + di[k], j + dj[k]) != SOLID;
        diag = (float)n * L.inv_h2;
    }
    const float x0 = xin ? xin[c] : 0.0f;
    xout[c] = diag > 0.0f ? x0 + OMEGA * (L.b[c] - ax) / diag : 0.0f;
}

// r = b - (-A) x
__global__ void k_residual(Level L, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)L.nx * L.ny) return;
    if (L.type[c] != LIQUID) {
        L.r[c] = 0.0f;
        return;
    }
    float diag;
    L.r[c] = L.b[c] - neg_apply(L, L.x, (int)(c % L.nx), (int)(c / L.nx), diag);
}

// Coarse right-hand side: the average of the LIQUID children's residuals.
__global__ void k_restrict(Level F, Level C, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)C.nx * C.ny) return;
    if (C.type[c] != LIQUID) {
        C.b[c] = 0.0f;
        return;
    }
    const int I = (int)(c % C.nx), J = (int)(c / C.nx);
    float s = 0.0f;
    for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
            const int i = 2 * I + di, j = 2 * J + dj;
            if (i < F.nx && j < F.ny && F.type[i + (int64_t)j * F.nx] == LIQUID) s += F.r[i + (int64_t)j * F.nx];
        }
    C.b[c] = 0.25f * s;
}

// x_fine += the coarse correction of the parent (LIQUID fine cells).
__global__ void k_prolong(Level F, Level C, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)F.nx * F.ny) return;
    if (F.type[c] != LIQUID) return;
    const int i = (int)(c % F.nx), j = (int)(c / F.nx);
    F.x[c] += C.x[(i / 2) + (int64_t)(j / 2) * C.nx];
}

// The coarsest level: COARSE_SWEEPS damped Jacobi sweeps from 0, one CTA.
__global__ void __launch_bounds__(1024) k_coarse(Level L, const Scal* __restrict__ S)
{
    if (S->done) return;
    __shared__ float xs[2][COARSE * COARSE];
    const int n = L.nx * L.ny;
    for (int c = threadIdx.x; c < n; c += blockDim.x) xs[0][c] = 0.0f;
    __syncthreads();
    for (int s = 0; s < COARSE_SWEEPS; ++s) {
        const float* xin = xs[s & 1];
        float* xout = xs[(s + 1) & 1];
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            if (L.type[c] != LIQUID) {
                xout[c] = 0.0f;
                continue;
            }
            float diag;
            const float ax = neg_apply(L, xin, c % L.nx, c / L.nx, diag);
            xout[c] = diag > 0.0f ? xin[c] + OMEGA * (L.b[c] - ax) / diag : 0.0f;
        }
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) L.x[c] = xs[COARSE_SWEEPS & 1][c];
}

// ---- CG kernels (level-0 cell vectors; every one returns once done) -------

// Block partial of sum a*b (double) over LIQUID cells: fixed tree per block.
__device__ __forceinline__ void block_partial(double v, double* __restrict__ part)
{
    __shared__ double sh[TPB];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = TPB / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__device__ __forceinline__ double fixed_sum(const double* __restrict__ part, int nb)
{
    __shared__ double sh[TPB];
    double acc = 0.0;
    for (int k = threadIdx.x; k < nb; k += TPB) acc += part[k];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = TPB / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    return sh[0];
}

// Start: x = 0, r = -b (the system -A x = -b), bb, threshold.
__global__ void k_cg_init(Level L, const float* __restrict__ b, float* __restrict__ x, float* __restrict__ r,
                          double* __restrict__ part)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    double v = 0.0;
    if (c < (int64_t)L.nx * L.ny) {
        const float rv = L.type[c] == LIQUID ? -b[c] : 0.0f;
        x[c] = 0.0f;
        r[c] = rv;
        v = (double)rv * rv;
    }
    block_partial(v, part);
}

__global__ void k_cg_init_final(const double* __restrict__ part, int nb, Scal* __restrict__ S, double tol, int maxit)
{
    const double bb = fixed_sum(part, nb);
    if (threadIdx.x == 0) {
        S->bb = bb;
        S->rr = bb;
        S->thr = tol * tol * bb;
        S->it = 0;
        S->maxit = maxit;
        S->beta = 0.0f;
        S->done = (bb == 0.0 || bb < S->thr || maxit == 0) ? 1 : 0;
    }
}

// rz partial (z = M^-1 r just computed).
__global__ void k_dot_rz(int64_t n, const float* __restrict__ r, const float* __restrict__ z, double* __restrict__ part,
                         const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    block_partial(c < n ? (double)r[c] * z[c] : 0.0, part);
}

__global__ void k_rz_final(const double* __restrict__ part, int nb, Scal* __restrict__ S)
{
    if (S->done) return;
    const double rz = fixed_sum(part, nb);
    if (threadIdx.x == 0) {
        S->beta = S->it == 0 ? 0.0f : (float)(rz / S->rz);
        S->rz = rz;
    }
}

// p = z + beta p, then q = (-A) p and the p.q partial (two kernels: q needs
// the neighbours' p).
__global__ void k_update_p(int64_t n, const float* __restrict__ z, float* __restrict__ p, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c < n) p[c] = S->it == 0 ? z[c] : z[c] + S->beta * p[c];
}

__global__ void k_spmv_pq(Level L, const float* __restrict__ p, float* __restrict__ q, double* __restrict__ part,
                          const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    double v = 0.0;
    if (c < (int64_t)L.nx * L.ny) {
        float qc = 0.0f;
        if (L.type[c] == LIQUID) {
            float diag;
            qc = neg_apply(L, p, (int)(c % L.nx), (int)(c / L.nx), diag);
        }
        q[c] = qc;
        v = (double)p[c] * qc;
    }
    block_partial(v, part);
}

__global__ void k_pq_final(const double* __restrict__ part, int nb, Scal* __restrict__ S)
{
    if (S->done) return;
    const double pq = fixed_sum(part, nb);
    if (threadIdx.x == 0) {
        S->pq = pq;
        S->alpha = pq != 0.0 ? (float)(S->rz / pq) : 0.0f;
    }
}

__global__ void k_update_xr(int64_t n, const float* __restrict__ p, const float* __restrict__ q, float* __restrict__ x,
                            float* __restrict__ r, double* __restrict__ part, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    double v = 0.0;
    if (c < n) {
        const float a = S->alpha;
        x[c] += a * p[c];
        const float rv = r[c] - a * q[c];
        r[c] = rv;
        v = (double)rv * rv;
    }
    block_partial(v, part);
}

__global__ void k_rr_final(const double* __restrict__ part, int nb, Scal* __restrict__ S)
{
    if (S->done) return;
    const double rr = fixed_sum(part, nb);
    if (threadIdx.x == 0) {
        S->rr = rr;
        S->it += 1;
        if (rr < S->thr || S->it >= S->maxit) S->done = 1;
    }
}

// Between the fluid-index order of the assembled system and the cell grid.
template <typename T>
__global__ void k_fluid_to_cells(int64_t n, const int32_t* __restrict__ fidx, const int32_t* __restrict__ nfluid,
                                 const T* __restrict__ src, float* __restrict__ dst)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= n) return;
    const int k = fidx[c];
    dst[c] = (k >= 0 && k < *nfluid) ? (float)src[k] : 0.0f;
}

template <typename T>
__global__ void k_cells_to_fluid(const int32_t* __restrict__ nfluid, const int32_t* __restrict__ cell_of,
                                 const float* __restrict__ src, T* __restrict__ dst)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k < *nfluid) dst[k] = (T)src[cell_of[k]];
}

}  // namespace

template <typename T>
void mg_fluid_to_cells(const Launch& L, int64_t ncell, const int32_t* fidx, const int32_t* nfluid, const T* src,
                       float* dst)
{
    k_fluid_to_cells<T><<<nblk(ncell), TPB, 0, L.stream>>>(ncell, fidx, nfluid, src, dst);
    L.count();
}

template <typename T>
void mg_cells_to_fluid(const Launch& L, int64_t ncell, const int32_t* nfluid, const int32_t* cell_of, const float* src,
                       T* dst)
{
    k_cells_to_fluid<T><<<nblk(ncell), TPB, 0, L.stream>>>(nfluid, cell_of, src, dst);
    L.count();
}

template void mg_fluid_to_cells<float>(const Launch&, int64_t, const int32_t*, const int32_t*, const float*, float*);
template void mg_fluid_to_cells<double>(const Launch&, int64_t, const int32_t*, const int32_t*, const double*, float*);
template void mg_cells_to_fluid<float>(const Launch&, int64_t, const int32_t*, const int32_t*, const float*, float*);
template void mg_cells_to_fluid<double>(const Launch&, int64_t, const int32_t*, const int32_t*, const float*, double*);

struct MgSolver
{
    int device = 0;
    int64_t n = 0;
    std::vector<Level> lv;
    float *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *tmp = nullptr;
    double* part = nullptr;
    Scal* S = nullptr;
    std::vector<void*> allocs;
    cudaGraphExec_t chunk = nullptr;
    const float* chunk_b = nullptr;
    cudaStream_t chunk_stream = nullptr;
};

namespace {

cudaError_t alloc(MgSolver* m, void** p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 4);
    if (e == cudaSuccess) m->allocs.push_back(*p);
    return e;
}

// One V-cycle from level l: lv[l].b given, lv[l].x out.
void vcycle(MgSolver* m, cudaStream_t st, int64_t* launches)
{
    const int nl = (int)m->lv.size();
    for (int l = 0; l < nl - 1; ++l) {
        Level& L = m->lv[l];
        const unsigned nb = nblk((int64_t)L.nx * L.ny);
        k_smooth<<<nb, TPB, 0, st>>>(L, nullptr, m->tmp, m->S);
        k_smooth<<<nb, TPB, 0, st>>>(L, m->tmp, L.x, m->S);
        k_residual<<<nb, TPB, 0, st>>>(L, m->S);
        k_restrict<<<nblk((int64_t)m->lv[l + 1].nx * m->lv[l + 1].ny), TPB, 0, st>>>(L, m->lv[l + 1], m->S);
        *launches += 4;
    }
    k_coarse<<<1, 1024, 0, st>>>(m->lv[nl - 1], m->S);
    *launches += 1;
    for (int l = nl - 2; l >= 0; --l) {
        Level& L = m->lv[l];
        const unsigned nb = nblk((int64_t)L.nx * L.ny);
        k_prolong<<<nb, TPB, 0, st>>>(L, m->lv[l + 1], m->S);
        k_smooth<<<nb, TPB, 0, st>>>(L, L.x, m->tmp, m->S);
        k_smooth<<<nb, TPB, 0, st>>>(L, m->tmp, L.x, m->S);
        *launches += 3;
    }
}

// One CG iteration (z = M^-1 r first): every kernel returns once S->done.
void cg_iteration(MgSolver* m, cudaStream_t st, int64_t* launches)
{
    Level& L0 = m->lv[0];
    const int64_t n = m->n;
    const unsigned nb = nblk(n);
    // z = V-cycle(r): level 0's right-hand side is r, its solution z
    vcycle(m, st, launches);
    k_dot_rz<<<nb, TPB, 0, st>>>(n, m->r, m->z, m->part, m->S);
    k_rz_final<<<1, TPB, 0, st>>>(m->part, (int)nb, m->S);
    k_update_p<<<nb, TPB, 0, st>>>(n, m->z, m->p, m->S);
    k_spmv_pq<<<nb, TPB, 0, st>>>(L0, m->p, m->q, m->part, m->S);
    k_pq_final<<<1, TPB, 0, st>>>(m->part, (int)nb, m->S);
    k_update_xr<<<nb, TPB, 0, st>>>(n, m->p, m->q, m->x, m->r, m->part, m->S);
    k_rr_final<<<1, TPB, 0, st>>>(m->part, (int)nb, m->S);
    *launches += 7;
}

}  // namespace

int mg_create(MgSolver** out, int nx, int ny, float dx, int device)
{
    *out = nullptr;
    MgSolver* m = new MgSolver();
    m->device = device;
    m->n = (int64_t)nx * ny;
    cudaError_t e = cudaSetDevice(device);
    const double h0 = dx;
    int lx = nx, ly = ny;
    double h = h0;
    for (;;) {
        Level L{};
        L.nx = lx;
        L.ny = ly;
        L.inv_h2 = (float)(1.0 / (h * h));
        const size_t N = (size_t)lx * ly;
        if (e == cudaSuccess) e = alloc(m, (void**)&L.type, N);
        if (e == cudaSuccess) e = alloc(m, (void**)&L.x, 4 * N);
        if (e == cudaSuccess) e = alloc(m, (void**)&L.b, 4 * N);
        if (e == cudaSuccess) e = alloc(m, (void**)&L.r, 4 * N);
        m->lv.push_back(L);
        if (std::max(lx, ly) <= COARSE) break;
        lx = (lx + 1) / 2;
        ly = (ly + 1) / 2;
        h *= 2.0;
    }
    const size_t N = (size_t)m->n;
    for (float** v : {&m->x, &m->p, &m->q, &m->tmp})
        if (e == cudaSuccess) e = alloc(m, (void**)v, 4 * N);
    if (e == cudaSuccess) e = alloc(m, (void**)&m->part, 8 * (size_t)nblk(m->n));
    if (e == cudaSuccess) e = alloc(m, (void**)&m->S, sizeof(Scal));
    // level 0 of the V-cycle: right-hand side = the CG residual, solution = z
    m->r = m->lv[0].b;
    m->z = m->lv[0].x;
    if (e != cudaSuccess) {
        mg_destroy(m);
        return -1;
    }
    *out = m;
    return 0;
}

void mg_destroy(MgSolver* m)
{
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->chunk) cudaGraphExecDestroy(m->chunk);
    for (void* p : m->allocs) cudaFree(p);
    delete m;
}

void mg_set_labels(MgSolver* m, cudaStream_t st, const uint8_t* labels, int64_t* launches)
{
    k_types0<<<nblk(m->n), TPB, 0, st>>>(m->n, labels, m->lv[0].type);
    for (size_t l = 1; l < m->lv.size(); ++l)
        k_coarsen_types<<<nblk((int64_t)m->lv[l].nx * m->lv[l].ny), TPB, 0, st>>>(m->lv[l - 1], m->lv[l]);
    *launches += (int64_t)m->lv.size();
}

cudaError_t mg_solve(MgSolver* m, cudaStream_t st, const float* b, double tol, int maxit, int64_t* launches,
                     int* iterations, double* rr, double* bb, float** x_out)
{
    const unsigned nb = nblk(m->n);
    k_cg_init<<<nb, TPB, 0, st>>>(m->lv[0], b, m->x, m->r, m->part);
    k_cg_init_final<<<1, TPB, 0, st>>>(m->part, (int)nb, m->S, tol, maxit);
    *launches += 2;
    // chunks of CHUNK iterations, recorded once per stream
    if (!m->chunk || m->chunk_stream != st) {
        if (m->chunk) cudaGraphExecDestroy(m->chunk);
        m->chunk = nullptr;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        int64_t dummy = 0;
        for (int k = 0; k < CHUNK; ++k) cg_iteration(m, st, &dummy);
        e = cudaStreamEndCapture(st, &g);
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&m->chunk, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return e;
        m->chunk_stream = st;
    }
    const int64_t per_iter = 7 * ((int64_t)m->lv.size() - 1) + 8;  // kernels of one cg_iteration
    Scal s{};
    for (;;) {
        cudaError_t e = cudaGraphLaunch(m->chunk, st);
        if (e != cudaSuccess) return e;
        *launches += per_iter * CHUNK;
        e = cudaMemcpyAsync(&s, m->S, sizeof(Scal), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        if (s.done) break;
    }
    *iterations = s.it;
    *rr = s.rr;
    *bb = s.bb;
    *x_out = m->x;
    return cudaSuccess;
}

}  // namespace fs
