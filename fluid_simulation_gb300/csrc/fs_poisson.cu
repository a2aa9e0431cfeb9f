// Pressure projection alone (no particles): the Poisson system of
// FluidSolver::pressureSolve (src/FluidSolver.cpp:363-425) built from a label
// grid, with the right-hand side given in double, solved three ways:
//
//   FS_POISSON_FP32   the step's CG (float vectors; float or double dots);
//   FS_POISSON_FP64   conjugate gradient with double vectors, double SpMV
//                     and double dots (k_cg64 below);
//   FS_POISSON_MIXED  FP64 iterative refinement: x and r = b - A x in double,
//                     each correction d from A d = r solved by the float CG to
//                     a loose tolerance, x += d, until ||b - A x|| / ||b|| is
//                     below the tolerance.
//
// On GB300 the FP64 rate is a small fraction of the FP32 rate, so the FP64 CG
// is bound by FP64 issue while the mixed form spends FP64 only once per
// refinement step.  Every method is deterministic (fixed reduction trees) and
// restated on the CPU in oracle/fs_oracle.c (fso_poisson_solve).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fs_mg.h"

namespace fs {
namespace {

constexpr int T = 1024;  // threads per CTA and elements per chunk
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;
constexpr int MAX_CHUNKS64 = 32 * 1024;

// ---- setup -------------------------------------------------------------

__global__ void k_poisson_rows(Geom g, const uint8_t* __restrict__ lab, const int32_t* __restrict__ fidx,
                               const int32_t* __restrict__ cell_of, const int32_t* __restrict__ nfluid,
                               const double* __restrict__ rhs, double* __restrict__ b, int32_t* __restrict__ down,
                               int32_t* __restrict__ up, uint8_t* __restrict__ flags)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= *nfluid) return;
    const int64_t c = cell_of[t];
    const int i = (int)(c % g.nx), j = (int)(c / g.nx);
    matrix_row(lab, g, fidx, c, i, j, flags[t], down[t], up[t]);
    b[t] = rhs[c];
}

// b[t] = rhs[cell of fluid cell t] (right-hand side given per cell on the device)
__global__ void k_gather_rhs(const int32_t* __restrict__ cell_of, const int32_t* __restrict__ nfluid,
                             const double* __restrict__ rhs, double* __restrict__ b)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < *nfluid) b[t] = rhs[cell_of[t]];
}

// ---- double vectors ----------------------------------------------------

struct Mat64
{
    const int32_t* down;
    const int32_t* up;
    const uint8_t* flags;
    double off;
    double dtab[5];
    double itab[5];
};

// (A v)_k summed in ascending column order from +0, in double.  v_at(n)
// supplies the vector entry of fluid cell n.
template <class VA>
__device__ __forceinline__ double row64(const Mat64& m, const double* dtab, int k, double vk, unsigned fl, int dn,
                                        int up, VA v_at)
{
    double acc = 0.0;
    if (dn >= 0) acc = dadd(acc, dmul(m.off, v_at(dn)));
    if (fl & 1u) acc = dadd(acc, dmul(m.off, v_at(k - 1)));
    acc = dadd(acc, dmul(dtab[fl >> 2], vk));
    if (fl & 2u) acc = dadd(acc, dmul(m.off, v_at(k + 1)));
    if (up >= 0) acc = dadd(acc, dmul(m.off, v_at(up)));
    return acc;
}

// r = b - A x
__global__ void k_residual64(Mat64 m, const int32_t* __restrict__ nfluid, const double* __restrict__ b,
                             const double* __restrict__ x, double* __restrict__ r)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *nfluid) return;
    auto v_at = [&](int n) { return x[n]; };
    r[k] = b[k] - row64(m, m.dtab, k, x[k], m.flags[k], m.down[k], m.up[k], v_at);
}

__global__ void k_to_f32(const int32_t* __restrict__ nfluid, const double* __restrict__ a, float* __restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < *nfluid) out[k] = (float)a[k];
}

// x = d (assign) or x += d, d converted exactly from float.
__global__ void k_add_f32(const int32_t* __restrict__ nfluid, const float* __restrict__ d, double* __restrict__ x,
                          int assign)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *nfluid) return;
    x[k] = assign ? (double)d[k] : x[k] + (double)d[k];
}

__global__ void k_copy64(const int32_t* __restrict__ nfluid, const double* __restrict__ a, double* __restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < *nfluid) out[k] = a[k];
}

__global__ void k_scatter64(Geom g, const int32_t* __restrict__ fidx, const int32_t* __restrict__ nfluid,
                            const double* __restrict__ x, double* __restrict__ out)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)g.nx * g.ny) return;
    const int k = fidx[c];
    out[c] = (k >= 0 && k < *nfluid) ? x[k] : 0.0;
}

__device__ __forceinline__ double warp_tree64(double v)
{
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) v = dadd(v, __shfl_down_sync(0xffffffffu, v, s));
    return v;
}

// Chunk partials (levels 1-2) of the fixed 32-ary tree over a[k] * b[k].
__global__ void __launch_bounds__(T) k_dot64_chunks(const int32_t* __restrict__ nfluid, const double* __restrict__ a,
                                                   const double* __restrict__ b, double* __restrict__ part)
{
    __shared__ double w[32];
    const int nf = *nfluid;
    if ((int)blockIdx.x * T >= nf) return;
    const int k = blockIdx.x * T + threadIdx.x;
    double v = k < nf ? dmul(a[k], b[k]) : 0.0;
    v = warp_tree64(v);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        const double t = warp_tree64(w[threadIdx.x]);
        if (threadIdx.x == 0) part[blockIdx.x] = t;
    }
}

// Levels 3+ over n chunk partials, one CTA; the result in *out.
__device__ void tree_over_partials(const double* part, int n, double* lvlA, double* lvlB, double* out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (n <= 1) {
        if (threadIdx.x == 0) *out = n == 1 ? part[0] : 0.0;
        return;
    }
    const int n3 = (n + 31) / 32;
    for (int g = warp; g < n3; g += T / 32) {
        const int e = g * 32 + lane;
        const double t = warp_tree64(e < n ? part[e] : 0.0);
        if (lane == 0) lvlA[g] = t;
    }
    __syncthreads();
    if (n3 == 1) {
        if (threadIdx.x == 0) *out = lvlA[0];
        return;
    }
    const int n4 = (n3 + 31) / 32;
    if (warp < n4) {
        const int e = warp * 32 + lane;
        const double t = warp_tree64(e < n3 ? lvlA[e] : 0.0);
        if (lane == 0) lvlB[warp] = t;
    }
    __syncthreads();
    if (warp == 0) {
        const double t = n4 == 1 ? lvlB[0] : warp_tree64(lane < n4 ? lvlB[lane] : 0.0);
        if (lane == 0) *out = t;
    }
}

__global__ void __launch_bounds__(T) k_dot64_final(const int32_t* __restrict__ nfluid,
                                                  const double* __restrict__ part, double* __restrict__ out)
{
    __shared__ double lvlA[T];
    __shared__ double lvlB[32];
    const int n = (*nfluid + T - 1) / T;
    tree_over_partials(part, n, lvlA, lvlB, out);
}

// ---- the FP64 conjugate gradient (persistent, cooperative) --------------

struct Cg64Args
{
    const int32_t* nfluid;
    const double* b;
    Mat64 m;
    double tol;
    int maxit;
    double *x, *r, *z, *p, *q;
    double* partials;  // [2 buffers][2 values][max chunks]
    int max_chunks;
    double* groups;    // [2 buffers][2 values][max_groups] group partials, or null
    int max_groups;
    unsigned* barrier;
    unsigned* status;
    CgResult* result;
};

struct Smem64
{
    double red[32][2];   // level-1 results of one chunk: [warp][value]
    double lvlA[T][2];
    double lvlB[32][2];
    double dtab[5];
    double itab[5];
    int flag;
};

// Grid barrier + levels 3+ over all chunk partials of buffer buf (NV values).
// When the group trees (32 chunk partials each) are many, the CTAs divide
// them among themselves and publish them behind a second barrier, as the
// float-vector CG's reduction does: the same tree, one more exchange, and a
// fraction of the FP64 work in each CTA.
constexpr int SPLIT_MIN64 = 64;  // group trees x values from which the CTAs divide them
template <int NV>
__device__ bool exchange64(const Cg64Args& a, int buf, int nchunks, unsigned& target, Smem64& sm, double (&out)[NV])
{
    auto barrier = [&]() -> bool {
        __syncthreads();
        if (threadIdx.x == 0) {
            int ok = 1;
            target += gridDim.x;
            red_release_add_u32(a.barrier, 1u);
            if (!count_reached(ld_acquire_u32(a.barrier), target)) {
                const uint64_t t0 = globaltimer_ns();
                while (!count_reached(ld_acquire_u32(a.barrier), target)) {
                    if (globaltimer_ns() - t0 > WAIT_LIMIT_NS) {
                        atomicOr(a.status, ST_TIMEOUT);
                        ok = 0;
                        break;
                    }
                }
            }
            sm.flag = ok;
        }
        __syncthreads();
        return sm.flag != 0;
    };
    if (!barrier()) return false;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double* src = a.partials + (size_t)buf * 2 * a.max_chunks;
    if (nchunks == 1) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = __ldcg(&src[(size_t)k * a.max_chunks]);
        return true;
    }
    const int n3 = (nchunks + 31) / 32;
    if (a.groups && n3 * NV >= SPLIT_MIN64 && gridDim.x > 1) {
        double* grp = a.groups + (size_t)buf * 2 * a.max_groups;
        for (int g = (int)blockIdx.x + warp * (int)gridDim.x; g < n3; g += 32 * (int)gridDim.x) {
            const int e = g * 32 + lane;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double t = warp_tree64(e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : 0.0);
                if (lane == 0) __stcg(&grp[(size_t)k * a.max_groups + g], t);
            }
        }
        if (!barrier()) return false;
        for (int i = threadIdx.x; i < n3 * NV; i += T)
            sm.lvlA[i / NV][i % NV] = __ldcg(&grp[(size_t)(i % NV) * a.max_groups + i / NV]);
    } else {
        for (int g = warp; g < n3; g += 32) {
            const int e = g * 32 + lane;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double t = warp_tree64(e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : 0.0);
                if (lane == 0) sm.lvlA[g][k] = t;
            }
        }
    }
    __syncthreads();
    if (n3 == 1) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = sm.lvlA[0][k];
    } else {
        const int n4 = (n3 + 31) / 32;
        if (warp < n4) {
            const int e = warp * 32 + lane;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double t = warp_tree64(e < n3 ? sm.lvlA[e][k] : 0.0);
                if (lane == 0) sm.lvlB[warp][k] = t;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double t = n4 == 1 ? sm.lvlB[0][k] : warp_tree64(lane < n4 ? sm.lvlB[lane][k] : 0.0);
            out[k] = __shfl_sync(0xffffffffu, t, 0);
        }
    }
    __syncthreads();
    return true;
}

// Levels 1-2 of NV values of one chunk -> partial slot `chunk` of buffer buf.
template <int NV>
__device__ void chunk_partial64(const Cg64Args& a, int buf, int chunk, const double (&v)[NV], Smem64& sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const double t = warp_tree64(v[k]);
        if (lane == 0) sm.red[warp][k] = t;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double t = warp_tree64(sm.red[lane][k]);
            if (lane == 0) __stcg(&a.partials[((size_t)buf * 2 + k) * a.max_chunks + chunk], t);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ double remote_p64(const Cg64Args& a, int n, bool first, double beta)
{
    const double zn = __ldcg(&a.z[n]);
    return first ? zn : dadd(zn, dmul(beta, __ldcg(&a.p[n])));
}

__global__ void __launch_bounds__(T, 1) k_cg64(Cg64Args a)
{
    __shared__ Smem64 sm;
    const int nf = *a.nfluid;
    const int nchunks = (nf + T - 1) / T;
    if (threadIdx.x < 5) {
        sm.dtab[threadIdx.x] = a.m.dtab[threadIdx.x];
        sm.itab[threadIdx.x] = a.m.itab[threadIdx.x];
    }
    if (nchunks == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.result = CgResult{0, 0, 0.0, 0.0};
        return;
    }
    if (nchunks > a.max_chunks || nchunks > MAX_CHUNKS64) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.status, ST_TOO_LARGE);
        return;
    }
    __syncthreads();
    const int tid = threadIdx.x;
    const int c0 = (int)(((int64_t)blockIdx.x * nchunks) / gridDim.x);
    const int c1 = (int)(((int64_t)(blockIdx.x + 1) * nchunks) / gridDim.x);
    unsigned target = 0;
    const Mat64& m = a.m;

    for (int c = c0; c < c1; ++c) {
        const int e = c * T + tid;
        double v[2] = {0.0, 0.0};
        if (e < nf) {
            const double r = a.b[e];
            const double z = dmul(sm.itab[m.flags[e] >> 2], r);
            __stcg(&a.x[e], 0.0);
            __stcg(&a.r[e], r);
            __stcg(&a.z[e], z);
            v[0] = dmul(r, r);
            v[1] = dmul(r, z);
        }
        chunk_partial64<2>(a, 0, c, v, sm);
    }
    double red2[2];
    if (!exchange64<2>(a, 0, nchunks, target, sm, red2)) return;
    const double bb = red2[0];
    double rz = red2[1], rr = bb;
    int iters = 0;
    bool done = bb == 0.0;
    double thr = dmul(dmul(a.tol, a.tol), bb);
    if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
    if (!done && rr < thr) done = true;
    bool first = true;
    double beta = 0.0;
    auto pv = [&](int n) { return remote_p64(a, n, first, beta); };
    for (int it = 1; !done && it <= a.maxit; ++it) {
        for (int c = c0; c < c1; ++c) {
            const int e = c * T + tid;
            double v[1] = {0.0};
            if (e < nf) {
                const double pe = remote_p64(a, e, first, beta);
                const double q = row64(m, sm.dtab, e, pe, m.flags[e], m.down[e], m.up[e], pv);
                __stcg(&a.q[e], q);
                v[0] = dmul(pe, q);
            }
            chunk_partial64<1>(a, 1, c, v, sm);
        }
        double red1[1];
        if (!exchange64<1>(a, 1, nchunks, target, sm, red1)) return;
        const double alpha = rz / red1[0];
        for (int c = c0; c < c1; ++c) {
            const int e = c * T + tid;
            double v[2] = {0.0, 0.0};
            if (e < nf) {
                const double pn = remote_p64(a, e, first, beta);
                const double x = dadd(__ldcg(&a.x[e]), dmul(alpha, pn));
                const double r = __ldcg(&a.r[e]) - dmul(alpha, __ldcg(&a.q[e]));
                const double z = dmul(sm.itab[m.flags[e] >> 2], r);
                __stcg(&a.x[e], x);
                __stcg(&a.r[e], r);
                __stcg(&a.z[e], z);
                __stcg(&a.p[e], pn);
                v[0] = dmul(r, r);
                v[1] = dmul(r, z);
            }
            chunk_partial64<2>(a, 0, c, v, sm);
        }
        if (!exchange64<2>(a, 0, nchunks, target, sm, red2)) return;
        rr = red2[0];
        iters = it;
        if (rr < thr) break;
        beta = red2[1] / rz;
        rz = red2[1];
        first = false;
    }
    if (blockIdx.x == 0 && tid == 0) *a.result = CgResult{iters, 0, rr, bb};
}

unsigned blocks(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace
}  // namespace fs

// ---------------------------------------------------------------- C ABI

using namespace fs;

struct fs_poisson
{
    Geom g{};
    int device = 0;
    int64_t ncell = 0;
    cudaStream_t stream = nullptr;
    uint8_t* labels = nullptr;
    int32_t *fidx = nullptr, *cell_of = nullptr, *down = nullptr, *up = nullptr, *scan_tmp = nullptr;
    int32_t* nfluid = nullptr;
    uint8_t* flags = nullptr;
    double *rhs = nullptr, *b = nullptr, *x = nullptr, *r = nullptr, *part = nullptr, *scal = nullptr;
    double *cx = nullptr, *cr = nullptr, *cz = nullptr, *cp = nullptr, *cq = nullptr, *cpart = nullptr;
    float* b32 = nullptr;
    unsigned* status = nullptr;
    unsigned* barrier64 = nullptr;
    CgResult* result64 = nullptr;
    CgWork cg{};
    float off32 = 0.0f;
    float diag32[5] = {};
    Mat64 m{};
    int grid64 = 0;
    bool ready = false;
    MgSolver* mg = nullptr;  // FS_POISSON_MGPCG, made on first use
    float* mg_b = nullptr;   // its right-hand side on the cells
    bool mg_labels = false;  // its cell types are those of the current problem
    int64_t launches = 0;
    cudaEvent_t ev[2] = {};
};

namespace {

int fail(int code, const std::string& msg)
{
    set_thread_error(msg.c_str());
    return code;
}

int cuda_check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return FS_OK;
    return fail(e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

void destroy(fs_poisson* p)
{
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    void* ptrs[] = {p->labels, p->fidx, p->cell_of, p->down, p->up, p->scan_tmp, p->nfluid, p->flags, p->rhs, p->b,
                    p->x, p->r, p->part, p->scal, p->cx, p->cr, p->cz, p->cp, p->cq, p->cpart, p->b32, p->status,
                    p->barrier64, p->result64, p->cg.x, p->cg.r, p->cg.z, p->cg.p, p->cg.q, p->cg.partials,
                    p->cg.barrier, p->cg.result, p->cg.route};
    for (void* q : ptrs) cudaFree(q);
    for (auto& e : p->ev)
        if (e) cudaEventDestroy(e);
    mg_destroy(p->mg);
    cudaFree(p->mg_b);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

// ||a||.||b|| style dot along the fixed tree; result in p->scal[slot].
void dot64(fs_poisson* p, const double* a, const double* b, int slot)
{
    const unsigned nch = (unsigned)((p->ncell + T - 1) / T);
    k_dot64_chunks<<<nch, T, 0, p->stream>>>(p->nfluid, a, b, p->part);
    k_dot64_final<<<1, T, 0, p->stream>>>(p->nfluid, p->part, p->scal + slot);
    p->launches += 2;
}

double read_scalar(fs_poisson* p, int slot)
{
    double v = 0.0;
    cudaMemcpyAsync(&v, p->scal + slot, sizeof(double), cudaMemcpyDeviceToHost, p->stream);
    cudaStreamSynchronize(p->stream);
    return v;
}

// The three methods on the assembled system (right-hand side in p->b), the
// solution in p->x (fluid-index order).
int solve_impl(fs_poisson* p, int method, double tol, int max_iterations, double inner_tolerance,
               int inner_precision, fs_poisson_stats* stats)
{
    const Launch L{p->stream, &p->launches, 0};
    const unsigned nb = blocks(p->ncell);
    fs_poisson_stats st{};
    cudaMemsetAsync(p->status, 0, 4, p->stream);
    cudaEventRecord(p->ev[0], p->stream);
    const int fp64dots = inner_precision == FS_CG_DOUBLE ? 1 : inner_precision == FS_CG_DS ? 2 : 0;
    const bool use_mg = method == FS_POISSON_MGPCG || method == FS_POISSON_MIXED_MG;
    if (use_mg) {
        if (!p->mg) {
            if (mg_create(&p->mg, p->g.nx, p->g.ny, p->g.dx, p->device) != 0)
                return fail(FS_ERR_OUT_OF_MEMORY, "multigrid levels");
            if (cudaMalloc(&p->mg_b, 4 * (size_t)p->ncell) != cudaSuccess)
                return fail(FS_ERR_OUT_OF_MEMORY, "multigrid right-hand side");
            p->mg_labels = false;
        }
        if (!p->mg_labels) {
            mg_set_labels(p->mg, p->stream, p->labels, &p->launches);
            p->mg_labels = true;
        }
    }
    if (method == FS_POISSON_MGPCG) {
        mg_fluid_to_cells<double>(L, p->ncell, p->fidx, p->nfluid, p->b, p->mg_b);
        int iters = 0;
        double rr = 0, bb = 0;
        float* xc = nullptr;
        const cudaError_t e = mg_solve(p->mg, p->stream, p->mg_b, tol, max_iterations, &p->launches, &iters, &rr, &bb, &xc);
        if (e != cudaSuccess) return cuda_check(e, "multigrid solve");
        mg_cells_to_fluid<double>(L, p->ncell, p->nfluid, p->cell_of, xc, p->x);
        st.inner_iterations = iters;
        st.outer_iterations = 1;
    } else if (method == FS_POISSON_FP32) {
        k_to_f32<<<nb, 256, 0, p->stream>>>(p->nfluid, p->b, p->b32);
        cg_solve(L, p->cg, p->nfluid, p->b32, p->diag32, p->down, p->up, p->flags, p->off32, tol, max_iterations,
                 fp64dots, p->status);
        k_add_f32<<<nb, 256, 0, p->stream>>>(p->nfluid, p->cg.x, p->x, 1);
        p->launches += 2;
        CgResult r{};
        cudaMemcpyAsync(&r, p->cg.result, sizeof(r), cudaMemcpyDeviceToHost, p->stream);
        cudaStreamSynchronize(p->stream);
        st.inner_iterations = r.iterations;
        st.outer_iterations = 1;
    } else if (method == FS_POISSON_FP64) {
        Cg64Args a{};
        a.nfluid = p->nfluid;
        a.b = p->b;
        a.m = p->m;
        a.tol = tol;
        a.maxit = max_iterations;
        a.x = p->x;
        a.r = p->cr;
        a.z = p->cz;
        a.p = p->cp;
        a.q = p->cq;
        a.partials = p->cpart;
        a.max_chunks = (int)((p->ncell + T - 1) / T);
        a.groups = p->cpart + 4 * (size_t)a.max_chunks;
        a.max_groups = (a.max_chunks + 31) / 32;
        a.barrier = p->barrier64;
        a.status = p->status;
        a.result = p->result64;
        cudaMemsetAsync(p->barrier64, 0, 4, p->stream);
        void* args[] = {&a};
        cudaLaunchCooperativeKernel((const void*)k_cg64, dim3(p->grid64), dim3(T), args, 0, p->stream);
        p->launches += 1;
        CgResult r{};
        cudaMemcpyAsync(&r, p->result64, sizeof(r), cudaMemcpyDeviceToHost, p->stream);
        cudaStreamSynchronize(p->stream);
        st.inner_iterations = r.iterations;
        st.outer_iterations = 1;
    } else {
        // FP64 iterative refinement around float-vector corrections (the
        // Jacobi-preconditioned CG, or the multigrid one for MIXED_MG).
        cudaMemsetAsync(p->x, 0, 8 * (size_t)p->ncell, p->stream);
        k_copy64<<<nb, 256, 0, p->stream>>>(p->nfluid, p->b, p->r);
        p->launches += 1;
        dot64(p, p->b, p->b, 0);
        const double bb = read_scalar(p, 0);
        const double thr = tol * tol * bb;
        double rr = bb;
        for (int outer = 0; outer < 64; ++outer) {
            if (!(rr >= thr) || bb == 0.0) break;
            CgResult r{};
            if (method == FS_POISSON_MIXED_MG) {
                mg_fluid_to_cells<double>(L, p->ncell, p->fidx, p->nfluid, p->r, p->mg_b);
                double rr_in = 0, bb_in = 0;
                float* xc = nullptr;
                const cudaError_t e = mg_solve(p->mg, p->stream, p->mg_b, inner_tolerance, max_iterations, &p->launches,
                                               &r.iterations, &rr_in, &bb_in, &xc);
                if (e != cudaSuccess) return cuda_check(e, "multigrid correction");
                mg_cells_to_fluid<float>(L, p->ncell, p->nfluid, p->cell_of, xc, p->cg.x);
            } else {
                k_to_f32<<<nb, 256, 0, p->stream>>>(p->nfluid, p->r, p->b32);
                cg_solve(L, p->cg, p->nfluid, p->b32, p->diag32, p->down, p->up, p->flags, p->off32, inner_tolerance,
                         max_iterations, fp64dots, p->status);
                p->launches += 1;
            }
            k_add_f32<<<nb, 256, 0, p->stream>>>(p->nfluid, p->cg.x, p->x, 0);
            k_residual64<<<nb, 256, 0, p->stream>>>(p->m, p->nfluid, p->b, p->x, p->r);
            p->launches += 2;
            dot64(p, p->r, p->r, 1);
            if (method != FS_POISSON_MIXED_MG)
                cudaMemcpyAsync(&r, p->cg.result, sizeof(r), cudaMemcpyDeviceToHost, p->stream);
            const double rr_new = read_scalar(p, 1);
            st.inner_iterations += r.iterations;
            st.outer_iterations = outer + 1;
            if (r.iterations == 0) break;  // no progress possible
            rr = rr_new;
        }
    }
    // final FP64 residual of the solution, whatever the method
    k_residual64<<<nb, 256, 0, p->stream>>>(p->m, p->nfluid, p->b, p->x, p->r);
    p->launches += 1;
    dot64(p, p->r, p->r, 1);
    dot64(p, p->b, p->b, 0);
    cudaEventRecord(p->ev[1], p->stream);
    unsigned status = 0;
    cudaMemcpyAsync(&status, p->status, 4, cudaMemcpyDeviceToHost, p->stream);
    const double rr = read_scalar(p, 1), bb = read_scalar(p, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_check(e, "fs_poisson_solve");
    if (status & ST_TIMEOUT) return fail(FS_ERR_TIMEOUT, "a device-side wait of a CG kernel timed out");
    if (status & ST_TOO_LARGE) return fail(FS_ERR_TOO_LARGE, "too many fluid cells");
    st.residual = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    cudaEventElapsedTime(&st.ms, p->ev[0], p->ev[1]);
    if (stats) *stats = st;
    return FS_OK;
}

}  // namespace

extern "C" {

FS_API int fs_poisson_create(int size_x, int size_y, float length_x, float length_y, int device, fs_poisson** out)
{
    set_thread_error("");
    if (!out || size_x < 3 || size_y < 3 || !(length_x > 0) || !(length_y > 0))
        return fail(FS_ERR_INVALID_ARGUMENT, "invalid Poisson grid");
    const int64_t n = (int64_t)size_x * size_y;
    if (n > (int64_t)4096 * 4096) return fail(FS_ERR_TOO_LARGE, "grid larger than 16777216 cells");
    fs_poisson* p = new fs_poisson();
    p->device = device;
    p->ncell = n;
    int rc = cuda_check(cudaSetDevice(device), "cudaSetDevice");
    if (rc) {
        delete p;
        return rc;
    }
    Geom& g = p->g;
    g.nx = size_x;
    g.ny = size_y;
    g.dx = length_x / (float)size_x;
    g.dy = length_y / (float)size_y;
    g.lx = (float)g.nx * g.dx;
    g.ly = (float)g.ny * g.dy;
    g.pdx = g.pdy = g.dx;
    // float coefficients as the step (src/FluidSolver.cpp:381-410); double
    // coefficients for the FP64 forms, from the same dx in double.
    const double dx2 = std::pow((double)g.dx, 2);
    p->off32 = (float)(1 / dx2);
    p->m.off = 1.0 / dx2;
    for (int k = 0; k < 5; ++k) {
        p->diag32[k] = (float)(-k / dx2);
        p->m.dtab[k] = -k / dx2;
        p->m.itab[k] = k ? 1.0 / p->m.dtab[k] : 1.0;
    }
    const size_t N = (size_t)n;
    const int64_t max_chunks = (n + T - 1) / T;
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    auto A = [&](void** ptr, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(ptr, bytes ? bytes : 1);
    };
    A((void**)&p->labels, N);
    A((void**)&p->fidx, 4 * N);
    A((void**)&p->cell_of, 4 * N);
    // The FP32 CG kernel copies whole 1024-element chunks of its system
    // arrays, so they are allocated to the last chunk's end.
    const size_t NP = (size_t)max_chunks * T;
    A((void**)&p->down, 4 * NP);
    A((void**)&p->up, 4 * NP);
    A((void**)&p->scan_tmp, 4 * scan_tmp_ints(n + 2));
    A((void**)&p->nfluid, 4);
    A((void**)&p->flags, NP);
    for (double** d : {&p->rhs, &p->b, &p->x, &p->r, &p->cx, &p->cr, &p->cz, &p->cp, &p->cq}) A((void**)d, 8 * N);
    A((void**)&p->part, 8 * max_chunks);
    A((void**)&p->scal, 8 * 4);
    A((void**)&p->cpart, 8 * 8 * max_chunks);  // chunk partials, then the group partials
    A((void**)&p->b32, 4 * N);
    A((void**)&p->status, 4);
    A((void**)&p->barrier64, 4);
    A((void**)&p->result64, sizeof(CgResult));
    for (float** f : {&p->cg.x, &p->cg.r, &p->cg.z, &p->cg.p, &p->cg.q}) A((void**)f, 4 * NP);
    A((void**)&p->cg.partials, 8 * 8 * max_chunks);  // chunk partials, then the group partials
    A((void**)&p->cg.barrier, 4);
    A((void**)&p->cg.result, sizeof(CgResult));
    A((void**)&p->cg.route, 8);
    for (auto& ev : p->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->status, 0, 4, p->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->nfluid, 0, 4, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    p->cg.max_cells = n;
    if (p->cg.partials) p->cg.groups = p->cg.partials + 4 * max_chunks;
    if (e == cudaSuccess && cg_prepare(p->cg, device) != 0) e = cudaErrorInvalidConfiguration;
    if (e == cudaSuccess) {
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        p->grid64 = sms;
    }
    if (e != cudaSuccess) {
        rc = cuda_check(e, "fs_poisson_create");
        destroy(p);
        return rc;
    }
    *out = p;
    return FS_OK;
}

FS_API int fs_poisson_destroy(fs_poisson* p)
{
    destroy(p);
    return FS_OK;
}

FS_API int fs_poisson_set_problem(fs_poisson* p, const uint8_t* labels, const double* rhs)
{
    if (!p || !labels || !rhs) return fail(FS_ERR_INVALID_ARGUMENT, "null argument");
    cudaSetDevice(p->device);
    const size_t N = (size_t)p->ncell;
    cudaMemcpyAsync(p->labels, labels, N, cudaMemcpyHostToDevice, p->stream);
    cudaMemcpyAsync(p->rhs, rhs, 8 * N, cudaMemcpyHostToDevice, p->stream);
    const Launch L{p->stream, &p->launches, 0};
    fluid_index(L, p->labels, p->ncell, p->fidx, p->cell_of, p->nfluid, p->scan_tmp);
    k_poisson_rows<<<blocks(p->ncell), 256, 0, p->stream>>>(p->g, p->labels, p->fidx, p->cell_of, p->nfluid, p->rhs,
                                                            p->b, p->down, p->up, p->flags);
    p->launches += 1;
    p->m.down = p->down;
    p->m.up = p->up;
    p->m.flags = p->flags;
    p->ready = true;
    p->mg_labels = false;
    return cuda_check(cudaStreamSynchronize(p->stream), "fs_poisson_set_problem");
}

FS_API int fs_poisson_solve(fs_poisson* p, int method, double tol, int max_iterations, double inner_tolerance,
                            int inner_precision, fs_poisson_stats* stats)
{
    if (!p || !p->ready || !(tol >= 0) || max_iterations < 0 ||
        (method != FS_POISSON_FP32 && method != FS_POISSON_FP64 && method != FS_POISSON_MIXED &&
         method != FS_POISSON_MGPCG && method != FS_POISSON_MIXED_MG))
        return fail(FS_ERR_INVALID_ARGUMENT, "invalid Poisson solve");
    cudaSetDevice(p->device);
    return solve_impl(p, method, tol, max_iterations, inner_tolerance, inner_precision, stats);
}

FS_API int fs_poisson_get_solution(fs_poisson* p, double* out)
{
    if (!p || !out || !p->ready) return fail(FS_ERR_INVALID_ARGUMENT, "no solution");
    cudaSetDevice(p->device);
    double* tmp = p->cx;  // scratch grid-sized double buffer of the FP64 CG
    k_scatter64<<<blocks(p->ncell), 256, 0, p->stream>>>(p->g, p->fidx, p->nfluid, p->x, tmp);
    p->launches += 1;
    cudaMemcpyAsync(out, tmp, 8 * (size_t)p->ncell, cudaMemcpyDeviceToHost, p->stream);
    return cuda_check(cudaStreamSynchronize(p->stream), "fs_poisson_get_solution");
}

FS_API int64_t fs_poisson_kernel_launches(const fs_poisson* p) { return p ? p->launches : 0; }

}  // extern "C"

// ---- device-side use by the other solvers of this library ------------------

namespace fs {

cudaStream_t poisson_stream(const fs_poisson* p) { return p->stream; }

int poisson_set_labels_device(fs_poisson* p, const uint8_t* d_labels)
{
    const size_t N = (size_t)p->ncell;
    cudaMemcpyAsync(p->labels, d_labels, N, cudaMemcpyDeviceToDevice, p->stream);
    cudaMemsetAsync(p->rhs, 0, 8 * N, p->stream);
    const Launch L{p->stream, &p->launches, 0};
    fluid_index(L, p->labels, p->ncell, p->fidx, p->cell_of, p->nfluid, p->scan_tmp);
    k_poisson_rows<<<blocks(p->ncell), 256, 0, p->stream>>>(p->g, p->labels, p->fidx, p->cell_of, p->nfluid, p->rhs,
                                                            p->b, p->down, p->up, p->flags);
    p->launches += 1;
    p->m.down = p->down;
    p->m.up = p->up;
    p->m.flags = p->flags;
    p->ready = true;
    p->mg_labels = false;
    return cuda_check(cudaStreamSynchronize(p->stream), "Poisson labels");
}

int poisson_solve_device(fs_poisson* p, const double* d_rhs, double* d_x, int method, double tol, int max_iterations,
                         double inner_tolerance, int inner_precision, fs_poisson_stats* stats)
{
    if (!p->ready) return fail(FS_ERR_INVALID_ARGUMENT, "Poisson labels not set");
    k_gather_rhs<<<blocks(p->ncell), 256, 0, p->stream>>>(p->cell_of, p->nfluid, d_rhs, p->b);
    p->launches += 1;
    const int rc = solve_impl(p, method, tol, max_iterations, inner_tolerance, inner_precision, stats);
    if (rc) return rc;
    k_scatter64<<<blocks(p->ncell), 256, 0, p->stream>>>(p->g, p->fidx, p->nfluid, p->x, d_x);
    p->launches += 1;
    return cuda_check(cudaGetLastError(), "Poisson solve");
}

int64_t poisson_launches(const fs_poisson* p) { return p->launches; }

}  // namespace fs
