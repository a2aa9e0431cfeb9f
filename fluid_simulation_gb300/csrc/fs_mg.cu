// Multigrid-preconditioned conjugate gradient for the pressure system of
// FluidSolver::pressureSolve (src/FluidSolver.cpp:363-425): the same matrix
// (off-diagonal 1 / dx^2 to liquid neighbours, diagonal -(non-solid
// neighbours) / dx^2, AIR neighbours as p = 0), solved on the cell grid with
// a geometric V-cycle as preconditioner.  Not in the reference: it needs far
// fewer iterations than the Jacobi-preconditioned CG (the reference's, kept
// bit-exact elsewhere) and gives a different, equally converged, solution.
//
// Levels halve the grid until it is at most 8 cells a side.  A coarse cell
// is AIR if any of its (up to four) children is AIR, else LIQUID if any child
// is LIQUID, else SOLID; the operator is re-discretised with twice the
// spacing.  Smoothing is damped Jacobi (omega = 2/3; two sweeps before and
// after), restriction averages the children's residuals, prolongation copies
// the coarse correction to the children, and the coarsest level takes 16
// Jacobi sweeps, so the V-cycle is a fixed symmetric linear operator.  The CG
// runs on -A (positive) with dot products accumulated in double along a fixed
// order; its scalars stay on the device and every kernel of an iteration
// returns at once after convergence, so iterations are replayed from a CUDA
// graph and the host only polls a flag.
//
// Launches are few and fused: a cell's neighbour types are one precomputed
// byte per level; on a level finer than 64 cells a side the two pre-smoothing
// sweeps (the first is pointwise, from zero) are one kernel, the residual is
// computed inside restriction, and prolongation inside the first
// post-smoothing sweep; all levels of at most 64 cells a side run in one CTA
// in shared memory; the CG's p update and SpMV are one kernel, and each
// reduction finishes in the last block of its kernel.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fs_mg.h"

namespace fs {
namespace {

constexpr int TPB = 256;
constexpr int RTPB = 512;  // threads of the reducing kernels (grid-stride, two blocks per SM)
constexpr int COARSE = 8;          // the coarsest level is at most this many cells a side
constexpr int COARSE_SWEEPS = 16;
constexpr int FUSE = 64;           // levels at most this many cells a side run in one CTA
constexpr int FUSED_THREADS = 1024;
constexpr int MAX_FUSED = 8;
constexpr float OMEGA = 2.0f / 3.0f;

unsigned nblk(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

// nbi byte of a cell: bits 0-3 its left, right, down, up neighbour is LIQUID;
// bits 4-6 the number of non-SOLID neighbours; bit 7 the cell is LIQUID.
struct Level
{
    int nx, ny;
    float inv_h2;   // 1 / h^2 of this level
    uint8_t* type;  // LIQUID / AIR / SOLID
    uint8_t* nbi;
    float *x, *b, *tmp;
};

// Scalars of the CG on the device.
struct Scal
{
    double pq, rr, rz, bb, thr;
    float alpha, beta;
    int it, done, maxit;
    int cur;          // p_old is p[cur], p_new p[cur ^ 1]
    unsigned ticket;  // blocks of the running kernel done with their partial
};

struct Fused
{
    Level lv[MAX_FUSED];
    int n;
};

__device__ __forceinline__ bool liquid(uint8_t m) { return (m & 0x80u) != 0; }
__device__ __forceinline__ int nsolid_free(uint8_t m) { return (m >> 4) & 7; }

// Stencil accessors take the direction of the value they return: the cell
// itself, or its left, right, down or up neighbour.
enum Dir { CTR = 0, LEFT, RIGHT, DOWN, UP };

// Values of an array around cell c of a level nx cells wide.
struct Around
{
    const float* a;
    int c, nx;
    __device__ __forceinline__ float operator()(int d) const
    {
        return a[d == CTR ? c : d == LEFT ? c - 1 : d == RIGHT ? c + 1 : d == DOWN ? c - nx : c + nx];
    }
};

// (-A x)_c of a LIQUID cell from its neighbour byte: (n x_c - sum of the
// LIQUID neighbours, in the order left, right, down, up) / h^2.
template <class X>
__device__ __forceinline__ float neg_apply(uint8_t m, float inv_h2, X xv)
{
    float s = 0.0f;
    if (m & 1u) s += xv(LEFT);
    if (m & 2u) s += xv(RIGHT);
    if (m & 4u) s += xv(DOWN);
    if (m & 8u) s += xv(UP);
    return ((float)nsolid_free(m) * xv(CTR) - s) * inv_h2;
}

// One damped Jacobi sweep at a cell from the input values xv around it: 0 off
// LIQUID cells (and where no neighbour is non-SOLID).
template <class X>
__device__ __forceinline__ float sweep_at(uint8_t m, float inv_h2, float bc, X xv)
{
    if (!liquid(m)) return 0.0f;
    const float d = (float)nsolid_free(m) * inv_h2;
    if (!(d > 0.0f)) return 0.0f;
    return xv(CTR) + OMEGA * (bc - neg_apply(m, inv_h2, xv)) / d;
}

// The first sweep from a zero guess, which is pointwise.
__device__ __forceinline__ float first_sweep(uint8_t m, float inv_h2, float bc)
{
    if (!liquid(m)) return 0.0f;
    const float d = (float)nsolid_free(m) * inv_h2;
    return d > 0.0f ? 0.0f + OMEGA * (bc - 0.0f) / d : 0.0f;
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

__device__ __forceinline__ uint8_t type_at(const Level& L, int i, int j)
{
    if (i < 0 || j < 0 || i >= L.nx || j >= L.ny) return SOLID;
    return L.type[i + (int64_t)j * L.nx];
}

__global__ void k_nbi(Level L)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)L.nx * L.ny) return;
    const int i = (int)(c % L.nx), j = (int)(c / L.nx);
    const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
    unsigned m = 0, n = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint8_t t = type_at(L, i + di[k], j + dj[k]);
        if (t != SOLID) ++n;
        if (t == LIQUID) m |= 1u << k;
    }
    m |= n << 4;
    if (L.type[c] == LIQUID) m |= 0x80u;
    L.nbi[c] = (uint8_t)m;
}

// ---- V-cycle kernels of the levels finer than FUSE cells a side ------------

// The two pre-smoothing sweeps from zero: x = sweep(sweep_0(b)).
__global__ void k_pre(Level L, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c64 = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c64 >= (int64_t)L.nx * L.ny) return;
    const int c = (int)c64;
    const uint8_t m = L.nbi[c];
    const Around nbi_b{L.b, c, L.nx};
    auto x1 = [&](int d) {
        const int k = d == CTR ? c : d == LEFT ? c - 1 : d == RIGHT ? c + 1 : d == DOWN ? c - L.nx : c + L.nx;
        return first_sweep(L.nbi[k], L.inv_h2, nbi_b(d));
    };
    L.x[c] = sweep_at(m, L.inv_h2, L.b[c], x1);
}

// Coarse right-hand side: the average of the LIQUID children's residuals
// b - (-A) x, computed here.
__global__ void k_restrict(Level F, Level C, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c64 = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c64 >= (int64_t)C.nx * C.ny) return;
    const int c = (int)c64;
    if (!liquid(C.nbi[c])) {
        C.b[c] = 0.0f;
        return;
    }
    const int J = c / C.nx, I = c - J * C.nx;
    float s = 0.0f;
    for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
            const int i = 2 * I + di, j = 2 * J + dj;
            if (i >= F.nx || j >= F.ny) continue;
            const int f = i + j * F.nx;
            const uint8_t m = F.nbi[f];
            if (liquid(m)) s += F.b[f] - neg_apply(m, F.inv_h2, Around{F.x, f, F.nx});
        }
    C.b[c] = 0.25f * s;
}

// x + the parent's coarse correction at the neighbour (di, dj) of fine cell
// (i, j) (di, dj in {-1, 0, 1}, the neighbour inside the grid).
__device__ __forceinline__ float prolonged(const float* __restrict__ xf, const float* __restrict__ xc, int nxf, int nxc,
                                           int i, int j, int di, int dj)
{
    const int fi = i + di, fj = j + dj;
    return xf[fi + fj * nxf] + xc[(fi >> 1) + (fj >> 1) * nxc];
}

// One sweep of x + P xc at fine cell (i, j) (the neighbours read are those
// the neighbour byte marks LIQUID, so inside the grid).
__device__ __forceinline__ float post1_at(uint8_t m, int i, int j, int nx, int nxc, float inv_h2, float bc,
                                          const float* __restrict__ xf, const float* __restrict__ xc)
{
    auto xv = [&](int d) {
        return prolonged(xf, xc, nx, nxc, i, j, d == LEFT ? -1 : d == RIGHT ? 1 : 0,
                         d == DOWN ? -1 : d == UP ? 1 : 0);
    };
    return sweep_at(m, inv_h2, bc, xv);
}

// First post-smoothing sweep of x + (the parent's coarse correction) into tmp.
__global__ void k_post1(Level F, Level C, const Scal* __restrict__ S)
{
    if (S->done) return;
    const int64_t c64 = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c64 >= (int64_t)F.nx * F.ny) return;
    const int c = (int)c64;
    const int j = c / F.nx, i = c - j * F.nx;
    F.tmp[c] = post1_at(F.nbi[c], i, j, F.nx, C.nx, F.inv_h2, F.b[c], F.x, C.x);
}

// ---- reductions: a fixed tree per block, the last block sums the blocks ----

// Adds v over the block (fixed tree), stores the block partial and returns
// true in the last block of the grid to do so, with the fixed-order sum of all
// partials in *total (every thread of that block).  Threads and warps add in
// double-single pairs; each warp's pair becomes a double (hi + lo) once, and
// the levels above are double.  GB300 executes FP64 at about two lanes per
// clock per SM, where a double product and add per cell bound these kernels.
__device__ __forceinline__ bool block_reduce(ds v, double* __restrict__ part, unsigned* ticket, double* total)
{
    __shared__ double sh[32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1)
        v = ds_add(v, ds{__shfl_down_sync(0xffffffffu, v.hi, s), __shfl_down_sync(0xffffffffu, v.lo, s)});
    if (lane == 0) sh[warp] = dadd((double)v.hi, (double)v.lo);
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < nw; ++w) b += sh[w];
        part[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    // (grids of at most 2 * blockDim.x blocks: both loads are issued before the add)
    const int k0 = threadIdx.x, k1 = threadIdx.x + blockDim.x;
    const double a0 = k0 < (int)gridDim.x ? __ldcg(&part[k0]) : 0.0;
    const double a1 = k1 < (int)gridDim.x ? __ldcg(&part[k1]) : 0.0;
    double acc = a0 + a1;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
    __syncthreads();
    if (lane == 0) sh[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += sh[w];
        sh[0] = t;
        *ticket = 0;
    }
    __syncthreads();
    *total = sh[0];
    return true;
}

// The reducing kernels walk the cells grid-stride (cell c of thread t of
// block b: c = b * blockDim + t + k * gridDim * blockDim), so a reduction has
// one partial per block, and its order is fixed by the launch shape.

// Last post-smoothing sweep; at level 0 (z = M^-1 r) also r.z and beta.
__global__ void k_post2(Level L, const float* __restrict__ r0, double* __restrict__ part, Scal* __restrict__ S)
{
    if (S->done) return;
    const int n = L.nx * L.ny;
    ds v{0.0f, 0.0f};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const float z = sweep_at(L.nbi[c], L.inv_h2, L.b[c], Around{L.tmp, c, L.nx});
        L.x[c] = z;
        if (r0) v = ds_add(v, ds_prod(r0[c], z));
    }
    if (!r0) return;  // uniform over the grid
    double rz;
    if (block_reduce(v, part, &S->ticket, &rz) && threadIdx.x == 0) {
        S->beta = S->it == 0 ? 0.0f : (float)(rz / S->rz);
        S->rz = rz;
    }
}

// ---- the levels of at most FUSE cells a side, in one CTA -------------------

__global__ void __launch_bounds__(FUSED_THREADS, 1)
    k_fused(Fused fu, const float* __restrict__ r0, Scal* __restrict__ S)
{
    if (S->done) return;
    extern __shared__ __align__(16) unsigned char smem[];
    float* X[MAX_FUSED];
    float* T[MAX_FUSED];
    float* B[MAX_FUSED];
    uint8_t* M[MAX_FUSED];
    {
        float* f = reinterpret_cast<float*>(smem);
        for (int k = 0; k < fu.n; ++k) {
            const int n = fu.lv[k].nx * fu.lv[k].ny;
            X[k] = f;
            T[k] = f + n;
            B[k] = f + 2 * n;
            f += 3 * n;
        }
        uint8_t* u = reinterpret_cast<uint8_t*>(f);
        for (int k = 0; k < fu.n; ++k) {
            M[k] = u;
            u += fu.lv[k].nx * fu.lv[k].ny;
        }
    }
    const int tid = threadIdx.x;
    for (int k = 0; k < fu.n; ++k) {
        const int n = fu.lv[k].nx * fu.lv[k].ny;
        for (int c = tid; c < n; c += FUSED_THREADS) M[k][c] = fu.lv[k].nbi[c];
    }
    {
        const int n = fu.lv[0].nx * fu.lv[0].ny;
        for (int c = tid; c < n; c += FUSED_THREADS) B[0][c] = fu.lv[0].b[c];
    }
    __syncthreads();
    // down: pre-smoothing and restriction (each level's sizes and shared
    // arrays held in registers for its loops)
    for (int k = 0; k + 1 < fu.n; ++k) {
        const int lnx = fu.lv[k].nx, lny = fu.lv[k].ny, cnx = fu.lv[k + 1].nx, cny = fu.lv[k + 1].ny;
        const float inv_h2 = fu.lv[k].inv_h2;
        float* const Xk = X[k];
        float* const Tk = T[k];
        float* const Bk = B[k];
        float* const Bc = B[k + 1];
        const uint8_t* const Mk = M[k];
        const uint8_t* const Mc = M[k + 1];
        const int n = lnx * lny;
        for (int c = tid; c < n; c += FUSED_THREADS) Tk[c] = first_sweep(Mk[c], inv_h2, Bk[c]);
        __syncthreads();
        for (int c = tid; c < n; c += FUSED_THREADS) Xk[c] = sweep_at(Mk[c], inv_h2, Bk[c], Around{Tk, c, lnx});
        __syncthreads();
        const int nc = cnx * cny;
        for (int c = tid; c < nc; c += FUSED_THREADS) {
            float s = 0.0f;
            if (liquid(Mc[c])) {
                const int J = c / cnx, I = c - J * cnx;
                for (int dj = 0; dj < 2; ++dj)
                    for (int di = 0; di < 2; ++di) {
                        const int i = 2 * I + di, j = 2 * J + dj;
                        if (i >= lnx || j >= lny) continue;
                        const int f = i + j * lnx;
                        const uint8_t m = Mk[f];
                        if (liquid(m)) s += Bk[f] - neg_apply(m, inv_h2, Around{Xk, f, lnx});
                    }
                s = 0.25f * s;
            }
            Bc[c] = s;
        }
        __syncthreads();
    }
    // the coarsest level: COARSE_SWEEPS sweeps from 0
    {
        const int k = fu.n - 1;
        const int lnx = fu.lv[k].nx, n = fu.lv[k].nx * fu.lv[k].ny;
        const float inv_h2 = fu.lv[k].inv_h2;
        float* const Xk = X[k];
        float* const Tk = T[k];
        const float* const Bk = B[k];
        const uint8_t* const Mk = M[k];
        for (int c = tid; c < n; c += FUSED_THREADS) Xk[c] = 0.0f;
        __syncthreads();
        for (int s = 0; s < COARSE_SWEEPS; ++s) {
            const float* xin = (s & 1) ? Tk : Xk;
            float* xout = (s & 1) ? Xk : Tk;
            for (int c = tid; c < n; c += FUSED_THREADS) xout[c] = sweep_at(Mk[c], inv_h2, Bk[c], Around{xin, c, lnx});
            __syncthreads();
        }
        static_assert((COARSE_SWEEPS & 1) == 0, "the coarse result ends in X");
    }
    // up: prolongation and post-smoothing
    for (int k = fu.n - 2; k >= 0; --k) {
        const int lnx = fu.lv[k].nx, cnx = fu.lv[k + 1].nx, n = fu.lv[k].nx * fu.lv[k].ny;
        const float inv_h2 = fu.lv[k].inv_h2;
        float* const Xk = X[k];
        float* const Tk = T[k];
        const float* const Xc = X[k + 1];
        const float* const Bk = B[k];
        const uint8_t* const Mk = M[k];
        for (int c = tid; c < n; c += FUSED_THREADS) {
            const int j = c / lnx, i = c - j * lnx;
            Tk[c] = post1_at(Mk[c], i, j, lnx, cnx, inv_h2, Bk[c], Xk, Xc);
        }
        __syncthreads();
        for (int c = tid; c < n; c += FUSED_THREADS) Xk[c] = sweep_at(Mk[c], inv_h2, Bk[c], Around{Tk, c, lnx});
        __syncthreads();
    }
    const int n0 = fu.lv[0].nx * fu.lv[0].ny;
    for (int c = tid; c < n0; c += FUSED_THREADS) fu.lv[0].x[c] = X[0][c];
    if (!r0) return;
    // the whole V-cycle ran here: r.z and beta over level 0, fixed order
    __shared__ double sh[32];
    double v = 0.0;
    for (int c = tid; c < n0; c += FUSED_THREADS) v += (double)r0[c] * X[0][c];
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
        double rz = 0.0;
        for (int w = 0; w < FUSED_THREADS / 32; ++w) rz += sh[w];
        S->beta = S->it == 0 ? 0.0f : (float)(rz / S->rz);
        S->rz = rz;
    }
}

// ---- CG kernels (level-0 cell vectors; every one returns once done) -------

// Start: x = 0, r = -b (the system -A x = -b), bb, threshold.
__global__ void k_cg_init(Level L, const float* __restrict__ b, float* __restrict__ x, float* __restrict__ r,
                          double* __restrict__ part, Scal* __restrict__ S, double tol, int maxit)
{
    const int n = L.nx * L.ny;
    ds v{0.0f, 0.0f};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const float rv = L.type[c] == LIQUID ? -b[c] : 0.0f;
        x[c] = 0.0f;
        r[c] = rv;
        v = ds_add(v, ds_prod(rv, rv));
    }
    double bb;
    if (block_reduce(v, part, &S->ticket, &bb) && threadIdx.x == 0) {
        S->bb = bb;
        S->rr = bb;
        S->thr = tol * tol * bb;
        S->it = 0;
        S->maxit = maxit;
        S->beta = 0.0f;
        S->cur = 0;
        S->done = (bb == 0.0 || bb < S->thr || maxit == 0) ? 1 : 0;
    }
}

// p_new = z + beta p_old (first iteration: z), q = (-A) p_new, p.q and alpha.
__global__ void k_p_spmv(Level L, const float* __restrict__ z, float* __restrict__ p0, float* __restrict__ p1,
                         float* __restrict__ q, double* __restrict__ part, Scal* __restrict__ S)
{
    if (S->done) return;
    const int n = L.nx * L.ny;
    const bool first = S->it == 0;
    const float beta = S->beta;
    const float* pold = S->cur ? p1 : p0;
    float* pnew = S->cur ? p0 : p1;
    ds v{0.0f, 0.0f};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const uint8_t m = L.nbi[c];
        const Around zs{z, c, L.nx}, ps{pold, c, L.nx};
        auto pn = [&](int d) { return first ? zs(d) : zs(d) + beta * ps(d); };
        const float pc = pn(CTR);
        const float qc = liquid(m) ? neg_apply(m, L.inv_h2, pn) : 0.0f;
        pnew[c] = pc;
        q[c] = qc;
        v = ds_add(v, ds_prod(pc, qc));
    }
    double pq;
    if (block_reduce(v, part, &S->ticket, &pq) && threadIdx.x == 0) {
        S->pq = pq;
        S->alpha = pq != 0.0 ? (float)(S->rz / pq) : 0.0f;
    }
}

// x += alpha p_new, r -= alpha q, r.r, convergence; p_new becomes p_old.
__global__ void k_update_xr(int64_t n, const float* __restrict__ p0, const float* __restrict__ p1,
                            const float* __restrict__ q, float* __restrict__ x, float* __restrict__ r,
                            double* __restrict__ part, Scal* __restrict__ S)
{
    if (S->done) return;
    const float* pnew = S->cur ? p0 : p1;
    const float a = S->alpha;
    ds v{0.0f, 0.0f};
    for (int64_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        x[c] += a * pnew[c];
        const float rv = r[c] - a * q[c];
        r[c] = rv;
        v = ds_add(v, ds_prod(rv, rv));
    }
    double rr;
    if (block_reduce(v, part, &S->ticket, &rr) && threadIdx.x == 0) {
        S->rr = rr;
        S->it += 1;
        S->cur ^= 1;
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
    int fuse0 = 0;            // first level of the fused kernel
    size_t fused_bytes = 0;   // its dynamic shared memory
    float *x = nullptr, *r = nullptr, *z = nullptr, *p0 = nullptr, *p1 = nullptr, *q = nullptr;
    double* part = nullptr;
    Scal* S = nullptr;
    std::vector<void*> allocs;
    cudaGraphExec_t iteration = nullptr;  // one CG iteration, recorded once per stream
    cudaStream_t iteration_stream = nullptr;
    int64_t per_iteration = 0;            // kernels of one CG iteration
    unsigned rgrid = 1;                   // blocks of the reducing kernels
    int expect = 8;                       // iterations to launch before the first poll
};

namespace {

cudaError_t alloc(MgSolver* m, void** p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 4);
    if (e == cudaSuccess) m->allocs.push_back(*p);
    return e;
}

Fused fused_levels(const MgSolver* m)
{
    Fused f{};
    f.n = (int)m->lv.size() - m->fuse0;
    for (int k = 0; k < f.n; ++k) f.lv[k] = m->lv[m->fuse0 + k];
    return f;
}

// z = V-cycle(r), with r.z and beta (level 0's right-hand side is r, its solution z).
void vcycle(MgSolver* m, cudaStream_t st, int64_t* launches)
{
    const int F = m->fuse0;
    for (int l = 0; l < F; ++l) {
        Level& L = m->lv[l];
        k_pre<<<nblk((int64_t)L.nx * L.ny), TPB, 0, st>>>(L, m->S);
        k_restrict<<<nblk((int64_t)m->lv[l + 1].nx * m->lv[l + 1].ny), TPB, 0, st>>>(L, m->lv[l + 1], m->S);
        *launches += 2;
    }
    k_fused<<<1, FUSED_THREADS, m->fused_bytes, st>>>(fused_levels(m), F == 0 ? m->r : nullptr, m->S);
    *launches += 1;
    for (int l = F - 1; l >= 0; --l) {
        Level& L = m->lv[l];
        const unsigned nb = nblk((int64_t)L.nx * L.ny);
        k_post1<<<nb, TPB, 0, st>>>(L, m->lv[l + 1], m->S);
        if (l == 0) k_post2<<<m->rgrid, RTPB, 0, st>>>(L, m->r, m->part, m->S);
        else k_post2<<<nb, TPB, 0, st>>>(L, nullptr, m->part, m->S);
        *launches += 2;
    }
}

void cg_iteration(MgSolver* m, cudaStream_t st, int64_t* launches)
{
    vcycle(m, st, launches);
    k_p_spmv<<<m->rgrid, RTPB, 0, st>>>(m->lv[0], m->z, m->p0, m->p1, m->q, m->part, m->S);
    k_update_xr<<<m->rgrid, RTPB, 0, st>>>(m->n, m->p0, m->p1, m->q, m->x, m->r, m->part, m->S);
    *launches += 2;
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
        if (e == cudaSuccess) e = alloc(m, (void**)&L.nbi, N);
        if (e == cudaSuccess) e = alloc(m, (void**)&L.x, 4 * N);
        if (e == cudaSuccess) e = alloc(m, (void**)&L.b, 4 * N);
        if (e == cudaSuccess) e = alloc(m, (void**)&L.tmp, 4 * N);
        m->lv.push_back(L);
        if (std::max(lx, ly) <= COARSE) break;
        lx = (lx + 1) / 2;
        ly = (ly + 1) / 2;
        h *= 2.0;
    }
    // the fused kernel takes every level of at most FUSE cells a side
    m->fuse0 = (int)m->lv.size() - 1;
    while (m->fuse0 > 0 && std::max(m->lv[m->fuse0 - 1].nx, m->lv[m->fuse0 - 1].ny) <= FUSE &&
           (int)m->lv.size() - (m->fuse0 - 1) <= MAX_FUSED)
        --m->fuse0;
    for (size_t k = m->fuse0; k < m->lv.size(); ++k) m->fused_bytes += (size_t)13 * m->lv[k].nx * m->lv[k].ny;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)m->fused_bytes);
    const size_t N = (size_t)m->n;
    for (float** v : {&m->x, &m->p0, &m->p1, &m->q})
        if (e == cudaSuccess) e = alloc(m, (void**)v, 4 * N);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    m->rgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(2 * (int64_t)sms, (m->n + RTPB - 1) / RTPB));
    m->rgrid = std::min(m->rgrid, (unsigned)(2 * RTPB));  // the last block loads two partials per thread
    if (e == cudaSuccess) e = alloc(m, (void**)&m->part, 8 * (size_t)m->rgrid);
    if (e == cudaSuccess) e = alloc(m, (void**)&m->S, sizeof(Scal));
    if (e == cudaSuccess) e = cudaMemset(m->S, 0, sizeof(Scal));
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
    if (m->iteration) cudaGraphExecDestroy(m->iteration);
    for (void* p : m->allocs) cudaFree(p);
    delete m;
}

void mg_set_labels(MgSolver* m, cudaStream_t st, const uint8_t* labels, int64_t* launches)
{
    k_types0<<<nblk(m->n), TPB, 0, st>>>(m->n, labels, m->lv[0].type);
    for (size_t l = 1; l < m->lv.size(); ++l)
        k_coarsen_types<<<nblk((int64_t)m->lv[l].nx * m->lv[l].ny), TPB, 0, st>>>(m->lv[l - 1], m->lv[l]);
    for (size_t l = 0; l < m->lv.size(); ++l)
        k_nbi<<<nblk((int64_t)m->lv[l].nx * m->lv[l].ny), TPB, 0, st>>>(m->lv[l]);
    *launches += 2 * (int64_t)m->lv.size();
}

cudaError_t mg_solve(MgSolver* m, cudaStream_t st, const float* b, double tol, int maxit, int64_t* launches,
                     int* iterations, double* rr, double* bb, float** x_out)
{
    k_cg_init<<<m->rgrid, RTPB, 0, st>>>(m->lv[0], b, m->x, m->r, m->part, m->S, tol, maxit);
    *launches += 1;
    if (!m->iteration || m->iteration_stream != st) {
        if (m->iteration) cudaGraphExecDestroy(m->iteration);
        m->iteration = nullptr;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        m->per_iteration = 0;
        cg_iteration(m, st, &m->per_iteration);
        e = cudaStreamEndCapture(st, &g);
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&m->iteration, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return e;
        m->iteration_stream = st;
    }
    // Launch as many iterations as the last solve needed, then poll; after
    // convergence the remaining kernels return at once.
    Scal s{};
    int launched = 0;
    int batch = std::max(1, std::min(m->expect, maxit));
    for (;;) {
        for (int k = 0; k < batch; ++k) {
            const cudaError_t e = cudaGraphLaunch(m->iteration, st);
            if (e != cudaSuccess) return e;
        }
        launched += batch;
        *launches += m->per_iteration * batch;
        cudaError_t e = cudaMemcpyAsync(&s, m->S, sizeof(Scal), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        if (s.done || launched >= maxit) break;
        batch = 2;
    }
    m->expect = std::max(1, s.it);
    *iterations = s.it;
    *rr = s.rr;
    *bb = s.bb;
    *x_out = m->x;
    return cudaSuccess;
}

}  // namespace fs
