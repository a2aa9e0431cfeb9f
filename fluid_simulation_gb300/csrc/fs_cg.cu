// Jacobi-preconditioned conjugate gradient for the pressure Poisson system of
// FluidSolver::pressureSolve (src/FluidSolver.cpp:363-425), where the
// reference assembles an Eigen::SparseMatrix and calls
// Eigen::ConjugateGradient (zero initial guess, diagonal preconditioner,
// stop when ||r||^2 < tol^2 ||b||^2 or after maxit updates).
//
// One persistent cooperative kernel runs the whole solve.  The matrix is never
// stored: row k of A is rebuilt from the fluid-cell flags (liquid left/right
// neighbours are k-1/k+1 in the j-major fluid order), the down/up fluid
// indices and the count of non-solid neighbours.  Floating point follows the
// oracle exactly:
//   * vectors and SpMV in float, each product and sum rounded on its own; a
//     row sums its terms in ascending column order (down, left, centre,
//     right, up) starting from +0;
//   * dot products sum their terms along the fixed "32-ary stride-halving
//     tree" (groups of 32 consecutive elements, s = 16..1: a[l] += a[l+s],
//     repeated on the group results) -- a warp shuffle tree, then a tree over
//     warps (one 1024-element chunk per CTA pass), then a tree over chunk
//     partials that every CTA evaluates redundantly after a grid barrier
//     (double trees over many chunks first divide their widest level among
//     the CTAs, behind a second barrier).  The result does not depend on the
//     launch shape.  Three precisions (template parameter R): float products,
//     sums, alpha, beta and threshold -- the precision of the reference's
//     Eigen VectorXf CG, and the default; exact float*float products summed
//     in double with alpha and beta rounded once to float; or the same with
//     the warp level in double-single pairs (DSD).  GB300's FP64 rate is a
//     small fraction of its FP32 rate, so the double variants cost FP64 issue
//     slots in every reduction.
//
// Per iteration there are two grid barriers (after p.q and after r.r, r.z).
// The search direction p_new = z + beta p_old is not exchanged through a third
// barrier: z and p_old of every cell are published to global memory in the
// previous phase, and each CTA recomputes p_new of the neighbours it needs
// with the same float operations.  A CTA that owns at most KREG chunks of 1024
// cells keeps their state in registers and shared memory and stages the p_new
// values its rows read from other CTAs into a shared-memory halo once per
// iteration; larger systems stream the state from global memory.  With float
// dot products, systems of more than KREG chunks per CTA run in k_cg_large
// instead (k_cg_route picks the kernel on the device): up to KBIG chunks per
// CTA in the register-resident form with 4-byte rows, from PIPE_MIN_CHUNKS on
// in a streaming form that copies each slot's operands into shared memory
// with cp.async several slots ahead of their use, in between streaming as in
// k_cg.  Waits are bounded: a CTA that waits longer than about two seconds
// sets ST_TIMEOUT and every CTA returns.
#include <type_traits>

#include "fs_internal.h"
#include "fs_pipeline.h"

namespace fs {
namespace {

constexpr int CG_THREADS = 1024;
constexpr int CHUNK = CG_THREADS;
constexpr int KREG = 8;                   // most chunks per CTA in the register-resident form
constexpr size_t DYN_BYTES = 204800;      // dynamic shared memory of k_cg: 12 B (16 B above 4 chunks) per cell + halo
constexpr int KBIG = 12;                  // most chunks per CTA in k_cg_large's register-resident form
// Dynamic shared memory of k_cg_large: 227 KB per CTA less the static Smem;
// 16 B per resident cell (p, row, x, r) + halo, or the pipeline's stages.
constexpr size_t LARGE_DYN_BYTES = 215040;
constexpr int SINGLE_CTA_CHUNKS = 16;       // systems this small run in one CTA
constexpr int MAX_CHUNKS = 32 * 1024;       // all-read reduction limit (33.5M cells)
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;

// Dynamic shared memory of the cluster kernel with K chunks per CTA.
__host__ __device__ constexpr size_t cluster_dyn_bytes(int K) { return (size_t)K * CHUNK * 25; }

struct CgArgs
{
    const int32_t* nfluid;
    const float* b;
    const int32_t* down;
    const int32_t* up;
    const uint8_t* flags;  // bit 0 left liquid, bit 1 right liquid, bits 2-4 non-solid neighbours
    float dtab[5];         // diagonal by non-solid count: (float)(-n / dx^2)
    float itab[5];         // 1 / diagonal, or 1 where the diagonal is 0
    float off;             // (float)(1 / dx^2)
    double tol;
    int maxit;
    int fp64;                  // 0: float dot products, 1: double
    float *x, *r, *z, *p, *q;  // fluid-index vectors (global)
    double* partials;          // [2 buffers][2 values][MAX chunks]
    int max_chunks;
    unsigned* barrier;
    unsigned* status;
    CgResult* result;
    unsigned missing;          // arrivals the grid barrier waits for beyond the grid (test hook; normally 0)
    uint64_t wait_ns;          // bound of a barrier wait
    int dyn_bytes;             // dynamic shared memory of the launch
    double* groups;            // [2 buffers][2 values][max_groups] group partials, or null
    int max_groups;
};

struct Smem
{
    union {
        double red[32][32][2];  // level-1 results: [chunk slot][warp][value]
        double lvlA[1024][2];
        float redf[32][32][2];
        float lvlAf[1024][2];
        float2 redp[32][32][2];  // level-1 results as double-single pairs
    };
    union {
        double lvlB[32][2];
        float lvlBf[32][2];
    };
    float dtab[5];
    float itab[5];
    int flag;
    int hlo, hhi;  // halo extent of the register-resident body
};

// Arithmetic of the reduction type R, each operation rounded on its own.
template <typename R> struct Ar;
template <> struct Ar<float>
{
    using Acc = float;
    using Elem = float;
    static __device__ __forceinline__ float add(float a, float b) { return fadd(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return fmul(a, b); }
    static __device__ __forceinline__ float prod(float a, float b) { return fmul(a, b); }
    static __device__ __forceinline__ float ratio(float a, float b) { return fdiv(a, b); }
    static __device__ __forceinline__ float tiny() { return 1.17549435e-38f; }
    using Lv1 = float;
    static __device__ __forceinline__ void put1(Smem& s, int a, int b, int k, float t) { s.redf[a][b][k] = t; }
    static __device__ __forceinline__ float get1(Smem& s, int a, int b, int k) { return s.redf[a][b][k]; }
    static __device__ __forceinline__ float& lvlA(Smem& s, int a, int k) { return s.lvlAf[a][k]; }
    static __device__ __forceinline__ float& lvlB(Smem& s, int a, int k) { return s.lvlBf[a][k]; }
};
template <> struct Ar<double>
{
    using Acc = double;
    using Elem = double;
    static __device__ __forceinline__ double add(double a, double b) { return dadd(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return dmul(a, b); }
    static __device__ __forceinline__ double prod(float a, float b) { return dmul((double)a, (double)b); }
    static __device__ __forceinline__ float ratio(double a, double b) { return (float)(a / b); }
    static __device__ __forceinline__ double tiny() { return 2.2250738585072014e-308; }
    using Lv1 = double;
    static __device__ __forceinline__ void put1(Smem& s, int a, int b, int k, double t) { s.red[a][b][k] = t; }
    static __device__ __forceinline__ double get1(Smem& s, int a, int b, int k) { return s.red[a][b][k]; }
    static __device__ __forceinline__ double& lvlA(Smem& s, int a, int k) { return s.lvlA[a][k]; }
    static __device__ __forceinline__ double& lvlB(Smem& s, int a, int k) { return s.lvlB[a][k]; }
};

// Double-single dot products (FS_CG_DS): each float*float product exactly,
// as an unevaluated pair of floats (fmul, then fmaf for its rounding error),
// the first tree level -- the 32 elements of one warp -- added in such pairs
// (TwoSum of the high parts, then the error and both low parts added in float;
// the pair is not renormalised between levels), the warp's root pair turned
// into a double (hi + lo, one double addition), and every level above in
// double, as FS_CG_DOUBLE.  The pairs carry about 48 bits, so the sums stay
// close to FP64 while GB300's FP64 pipe, where the double variant spends its
// time, does almost nothing per element.  (ds, ds_prod, ds_add: fs_common.cuh.)
struct DSD
{
};
template <> struct Ar<DSD> : Ar<double>
{
    using Elem = ds;
    static __device__ __forceinline__ ds prod(float a, float b) { return ds_prod(a, b); }
    // A warp's root pair is kept as a pair and becomes a double where the
    // level-2 tree reads 32 of them, one per lane: one conversion instruction
    // per 32 warp trees instead of one per tree, on a pipe that does about two
    // FP64 lanes per clock per SM.
    using Lv1 = ds;
    static __device__ __forceinline__ void put1(Smem& s, int a, int b, int k, ds t)
    {
        s.redp[a][b][k] = make_float2(t.hi, t.lo);
    }
    static __device__ __forceinline__ double get1(Smem& s, int a, int b, int k)
    {
        const float2 t = s.redp[a][b][k];
        return dadd((double)t.x, (double)t.y);
    }
};
template <typename R> using Acc = typename Ar<R>::Acc;
template <typename R> using Elem = typename Ar<R>::Elem;

template <typename R>
__device__ __forceinline__ R warp_tree(R v)
{
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) v = Ar<R>::add(v, __shfl_down_sync(0xffffffffu, v, s));
    return v;
}

// The warp trees of NV values in place; with PACK, two floats share one tree
// of packed adds (add.rn.f32x2: each half rounded as its own fadd).  Level-1
// trees pack in every kernel; level 2 and the cross-CTA reduction only in the
// grid-synchronised ones (in the cluster kernel their paired values spill).
template <typename A, int NV, bool PACK = true>
__device__ __forceinline__ void warp_trees(A (&v)[NV])
{
    if constexpr (PACK && std::is_same<A, float>::value && NV == 2) {
        float2 t = make_float2(v[0], v[1]);
#pragma unroll
        for (int s = 16; s >= 1; s >>= 1) {
            const float2 o = make_float2(__shfl_down_sync(0xffffffffu, t.x, s), __shfl_down_sync(0xffffffffu, t.y, s));
            t = __fadd2_rn(t, o);
        }
        v[0] = t.x;
        v[1] = t.y;
    } else {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = warp_tree<A>(v[k]);
    }
}

// Barrier over the active CTAs.  Thread 0 arrives with a release reduction on
// the counter (bar.sync first makes the CTA's writes part of what it
// releases) and spins with acquire loads; the closing bar.sync hands the
// acquired view to the other threads, which read shared data with ld.cg.
// Returns false if this CTA gave up waiting (after a.wait_ns); a CTA that
// gives up returns, so every other CTA also gives up at its next barrier.
__device__ __forceinline__ bool cta_barrier(const CgArgs& a, bool grid, unsigned arrivals, unsigned& target, Smem& sm)
{
    // (callers come straight from level2, whose closing bar.sync orders the CTA's writes)
    if (grid && threadIdx.x == 0) {
        target += arrivals;
        unsigned old;
        asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(a.barrier) : "memory");
        int ok = 1;
        const unsigned want = target + a.missing;
        if (!count_reached(old + 1u, want) && !count_reached(ld_acquire_u32(a.barrier), want)) {
            const uint64_t t0 = globaltimer_ns();
            while (!count_reached(ld_acquire_u32(a.barrier), want)) {
                if (globaltimer_ns() - t0 > a.wait_ns) {
                    atomicOr(a.status, ST_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        sm.flag = ok;
    }
    __syncthreads();
    return !grid || sm.flag != 0;
}

// The CTAs that share one solve: every CTA of the cooperative grid (or the
// first CTA alone, for small systems) ...
struct GridSync
{
    bool grid;
    unsigned target;
    int active;  // CTAs taking part: the fewest that keep the most chunks per CTA unchanged
    __device__ int rank() const { return grid ? (int)blockIdx.x : 0; }
    __device__ int size() const { return grid ? active : 1; }
    __device__ bool barrier(const CgArgs& a, Smem& sm) { return cta_barrier(a, grid, (unsigned)active, target, sm); }
};

// ... or the CTAs of one thread-block cluster, which the hardware schedules
// together; its barrier releases and acquires at cluster scope, which covers
// the global-memory partials and published z, p that the CTAs exchange.
struct ClusterSync
{
    __device__ int rank() const
    {
        unsigned r;
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
        return (int)r;
    }
    __device__ int size() const
    {
        unsigned n;
        asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
        return (int)n;
    }
    __device__ bool barrier(const CgArgs&, Smem&)
    {
        asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
        return true;
    }
};

// The level-1 tree of one warp's elements (lane 0's value is the result).
template <typename R>
__device__ __forceinline__ typename Ar<R>::Lv1 elem_tree(Elem<R> v)
{
    if constexpr (std::is_same<R, DSD>::value) {
#pragma unroll
        for (int s = 16; s >= 1; s >>= 1) {
            const ds o{__shfl_down_sync(0xffffffffu, v.hi, s), __shfl_down_sync(0xffffffffu, v.lo, s)};
            v = ds_add(v, o);
        }
        return v;
    } else {
        return warp_tree<R>(v);
    }
}

// Level-1 (warp) tree of NV values for chunk slot `slot`; lane 0 keeps it.
// Two float values go through one tree of packed adds (add.rn.f32x2: each
// half rounded as its own fadd), the same sums with half the add instructions;
// with PACK_DS two double-single values likewise (the register-resident
// forms spill with it, so only the pipelined form asks for it).
template <typename R, int NV, bool PACK_DS = false>
__device__ __forceinline__ void level1(const Elem<R> (&v)[NV], int slot, Smem& sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if constexpr (std::is_same<R, float>::value && NV == 2) {
        float t[2] = {v[0], v[1]};
        warp_trees<float, 2>(t);
        if (lane == 0) {
            Ar<R>::put1(sm, slot, warp, 0, t[0]);
            Ar<R>::put1(sm, slot, warp, 1, t[1]);
        }
        return;
    }
    if constexpr (PACK_DS && std::is_same<R, DSD>::value && NV == 2) {
        // both values' pairs in packed arithmetic: ds_add on each half, its
        // subtractions as additions of the negation (exact in round-to-nearest)
        auto sub2 = [](float2 x, float2 y) { return __fadd2_rn(x, make_float2(-y.x, -y.y)); };
        float2 hi = make_float2(v[0].hi, v[1].hi), lo = make_float2(v[0].lo, v[1].lo);
#pragma unroll
        for (int s = 16; s >= 1; s >>= 1) {
            const float2 ohi =
                make_float2(__shfl_down_sync(0xffffffffu, hi.x, s), __shfl_down_sync(0xffffffffu, hi.y, s));
            const float2 olo =
                make_float2(__shfl_down_sync(0xffffffffu, lo.x, s), __shfl_down_sync(0xffffffffu, lo.y, s));
            const float2 sum = __fadd2_rn(hi, ohi);
            const float2 vv = sub2(sum, hi);
            float2 e = __fadd2_rn(sub2(hi, sub2(sum, vv)), sub2(ohi, vv));
            e = __fadd2_rn(e, lo);
            e = __fadd2_rn(e, olo);
            hi = sum;
            lo = e;
        }
        if (lane == 0) {
            Ar<R>::put1(sm, slot, warp, 0, ds{hi.x, lo.x});
            Ar<R>::put1(sm, slot, warp, 1, ds{hi.y, lo.y});
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const typename Ar<R>::Lv1 t = elem_tree<R>(v[k]);
        if (lane == 0) Ar<R>::put1(sm, slot, warp, k, t);
    }
}

// Level-1 trees of one float value of two slots at once (packed adds).
__device__ __forceinline__ void level1_pair(float v0, float v1, int slot0, Smem& sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float t[2] = {v0, v1};
    warp_trees<float, 2>(t);
    if (lane == 0) {
        Ar<float>::put1(sm, slot0, warp, 0, t[0]);
        Ar<float>::put1(sm, slot0 + 1, warp, 0, t[1]);
    }
}

// Level-2 trees for slots [0, nslots) -> chunk partials part[buf][k][chunk0 + slot].
template <typename R, int NV, bool PACK = true>
__device__ __forceinline__ void level2(const CgArgs& a, int buf, int chunk0, int nslots, Smem& sm)
{
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Acc<R>* part = reinterpret_cast<Acc<R>*>(a.partials);
    if (warp < nslots) {
        if constexpr (PACK && std::is_same<Acc<R>, float>::value && NV == 2) {
            Acc<R> t[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) t[k] = Ar<R>::get1(sm, warp, lane, k);
            warp_trees<Acc<R>, NV>(t);
#pragma unroll
            for (int k = 0; k < NV; ++k)
                if (lane == 0) __stcg(&part[((size_t)buf * 2 + k) * a.max_chunks + chunk0 + warp], t[k]);
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const Acc<R> t = warp_tree<Acc<R>>(Ar<R>::get1(sm, warp, lane, k));
                if (lane == 0) __stcg(&part[((size_t)buf * 2 + k) * a.max_chunks + chunk0 + warp], t);
            }
        }
    }
    __syncthreads();
}

// Levels 3+: every CTA reduces all chunk partials of buffer buf, one value
// after the other.
template <typename R, int NV>
__device__ __forceinline__ void reduce_chunks_one(const CgArgs& a, int buf, int nchunks, Smem& sm, Acc<R> (&out)[NV])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const Acc<R>* src = reinterpret_cast<const Acc<R>*>(a.partials) + (size_t)buf * 2 * a.max_chunks;
    if (nchunks == 1) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = __ldcg(&src[(size_t)k * a.max_chunks]);
        return;
    }
    int n = (nchunks + 31) / 32;
    if (n <= 32) {
        // group trees into lvlB, then every warp evaluates the tree over the
        // groups itself (lvlB is not reused before the next reduction's
        // group trees, so no trailing barrier)
        if (warp < n) {
            const int e = warp * 32 + lane;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const Acc<R> v = e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : Acc<R>(0);
                const Acc<R> t = warp_tree<Acc<R>>(v);
                if (lane == 0) Ar<R>::lvlB(sm, warp, k) = t;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if (n == 1) {
                out[k] = Ar<R>::lvlB(sm, 0, k);
            } else {
                const Acc<R> t = warp_tree<Acc<R>>(lane < n ? Ar<R>::lvlB(sm, lane, k) : Acc<R>(0));
                out[k] = __shfl_sync(0xffffffffu, t, 0);
            }
        }
        return;
    }
    for (int g = warp; g < n; g += 32) {
        const int e = g * 32 + lane;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const Acc<R> v = e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : Acc<R>(0);
            const Acc<R> t = warp_tree<Acc<R>>(v);
            if (lane == 0) Ar<R>::lvlA(sm, g, k) = t;
        }
    }
    __syncthreads();
    bool inA = true;
    while (n > 1) {
        const int m = (n + 31) / 32;
        if (warp < m) {
            const int e = warp * 32 + lane;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                Acc<R> v;
                if (inA) v = e < n ? Ar<R>::lvlA(sm, e, k) : Acc<R>(0);
                else v = e < n ? Ar<R>::lvlB(sm, e, k) : Acc<R>(0);
                const Acc<R> t = warp_tree<Acc<R>>(v);
                if (lane == 0) {
                    if (inA) Ar<R>::lvlB(sm, warp, k) = t;
                    else Ar<R>::lvlA(sm, warp, k) = t;
                }
            }
        }
        __syncthreads();
        inA = !inA;
        n = m;
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = inA ? Ar<R>::lvlA(sm, 0, k) : Ar<R>::lvlB(sm, 0, k);
    if (inA) __syncthreads();  // lvlA shares storage with the next phase's level-1 results
}

// The same with the two values of a float reduction in packed trees (PACK),
// else reduce_chunks_one.
template <typename R, int NV, bool PACK = true>
__device__ __forceinline__ void reduce_chunks(const CgArgs& a, int buf, int nchunks, Smem& sm, Acc<R> (&out)[NV])
{
    if constexpr (!(PACK && std::is_same<Acc<R>, float>::value && NV == 2)) {
        reduce_chunks_one<R, NV>(a, buf, nchunks, sm, out);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const Acc<R>* src = reinterpret_cast<const Acc<R>*>(a.partials) + (size_t)buf * 2 * a.max_chunks;
    if (nchunks == 1) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = __ldcg(&src[(size_t)k * a.max_chunks]);
        return;
    }
    int n = (nchunks + 31) / 32;
    if (n <= 32) {
        // group trees into lvlB, then every warp evaluates the tree over the
        // groups itself (lvlB is not reused before the next reduction's
        // group trees, so no trailing barrier)
        if (warp < n) {
            const int e = warp * 32 + lane;
            Acc<R> t[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) t[k] = e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : Acc<R>(0);
            warp_trees<Acc<R>, NV>(t);
#pragma unroll
            for (int k = 0; k < NV; ++k)
                if (lane == 0) Ar<R>::lvlB(sm, warp, k) = t[k];
        }
        __syncthreads();
        if (n == 1) {
#pragma unroll
            for (int k = 0; k < NV; ++k) out[k] = Ar<R>::lvlB(sm, 0, k);
        } else {
            Acc<R> t[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) t[k] = lane < n ? Ar<R>::lvlB(sm, lane, k) : Acc<R>(0);
            warp_trees<Acc<R>, NV>(t);
#pragma unroll
            for (int k = 0; k < NV; ++k) out[k] = __shfl_sync(0xffffffffu, t[k], 0);
        }
        return;
    }
    for (int g = warp; g < n; g += 32) {
        const int e = g * 32 + lane;
        Acc<R> t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] = e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : Acc<R>(0);
        warp_trees<Acc<R>, NV>(t);
#pragma unroll
        for (int k = 0; k < NV; ++k)
            if (lane == 0) Ar<R>::lvlA(sm, g, k) = t[k];
    }
    __syncthreads();
    bool inA = true;
    while (n > 1) {
        const int m = (n + 31) / 32;
        if (warp < m) {
            const int e = warp * 32 + lane;
            Acc<R> t[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                if (inA) t[k] = e < n ? Ar<R>::lvlA(sm, e, k) : Acc<R>(0);
                else t[k] = e < n ? Ar<R>::lvlB(sm, e, k) : Acc<R>(0);
            }
            warp_trees<Acc<R>, NV>(t);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                if (lane == 0) {
                    if (inA) Ar<R>::lvlB(sm, warp, k) = t[k];
                    else Ar<R>::lvlA(sm, warp, k) = t[k];
                }
            }
        }
        __syncthreads();
        inA = !inA;
        n = m;
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = inA ? Ar<R>::lvlA(sm, 0, k) : Ar<R>::lvlB(sm, 0, k);
    if (inA) __syncthreads();  // lvlA shares storage with the next phase's level-1 results
}

// Levels 3+ over the chunk partials of buffer buf, after the barrier that
// published them.  Every CTA evaluates the whole tree itself; when the tree is
// double and its widest level (the group trees over 32 chunk partials each)
// is wide, the CTAs first divide the group trees among themselves, publish
// them behind one more barrier and evaluate only the levels above: the same
// tree and the same operations, traded for one more exchange (~2.4 us)
// against the group trees' FP64 work, which GB300 executes at about two
// lanes per clock per SM (~40 ns per group and value in every CTA).
// Returns false if a barrier gave up.
constexpr int SPLIT_MIN = 64;  // group trees x values from which the CTAs divide them
template <typename R, int NV, class Sync>
__device__ __forceinline__ bool reduce_all(const CgArgs& a, int buf, int nchunks, Smem& sm, Acc<R> (&out)[NV],
                                           Sync& sync)
{
    if constexpr (std::is_same<Acc<R>, double>::value && std::is_same<Sync, GridSync>::value) {
        const double* src = a.partials + (size_t)buf * 2 * a.max_chunks;
        const int ngroups = (nchunks + 31) / 32;
        if (a.groups && ngroups * NV >= SPLIT_MIN && sync.size() > 1) {
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            const int rank = sync.rank(), size = sync.size();
            double* grp = a.groups + (size_t)buf * 2 * a.max_groups;
            for (int g = rank + warp * size; g < ngroups; g += 32 * size) {
                const int e = g * 32 + lane;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    const double v = e < nchunks ? __ldcg(&src[(size_t)k * a.max_chunks + e]) : 0.0;
                    const double t = warp_tree<double>(v);
                    if (lane == 0) __stcg(&grp[(size_t)k * a.max_groups + g], t);
                }
            }
            __syncthreads();  // the CTA's group stores precede thread 0's release
            if (!sync.barrier(a, sm)) return false;
            // the levels above, as reduce_chunks over the group partials
            CgArgs ag = a;
            ag.partials = a.groups;
            ag.max_chunks = a.max_groups;
            reduce_chunks<R, NV>(ag, buf, ngroups, sm, out);
            return true;
        }
    }
    reduce_chunks<R, NV, std::is_same<Sync, GridSync>::value>(a, buf, nchunks, sm, out);
    return true;
}

// Levels 2+ when one CTA owns all of at most 32 chunks: one warp reduces each
// chunk's 32 level-1 results and then the chunk partials, the same tree as
// level2 + reduce_all (a lone chunk's partial is the result as it stands),
// without the round trip of the partials through global memory.
template <typename R, int NV>
__device__ __forceinline__ void local_reduce(int nchunks, Smem& sm, Acc<R> (&out)[NV])
{
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            Acc<R> mine = Acc<R>(0);
            for (int s = 0; s < nchunks; ++s) {
                Acc<R> t = warp_tree<Acc<R>>(Ar<R>::get1(sm, s, lane, k));
                t = __shfl_sync(0xffffffffu, t, 0);
                if (lane == s) mine = t;
            }
            const Acc<R> res = nchunks == 1 ? mine : warp_tree<Acc<R>>(lane < nchunks ? mine : Acc<R>(0));
            if (lane == 0) Ar<R>::lvlB(sm, 0, k) = res;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = Ar<R>::lvlB(sm, 0, k);
}

// p_new of a cell outside this CTA's range, from its published z and p_old.
__device__ __forceinline__ float remote_p(const CgArgs& a, int n, bool first, float beta)
{
    const float zn = __ldcg(&a.z[n]);
    return first ? zn : fadd(zn, fmul(beta, __ldcg(&a.p[n])));
}

// One CG solve with the state streamed from global memory: the form for
// CTAs whose cells do not fit the register-resident form below.
template <typename R, class Sync>
__device__ __forceinline__ void cg_stream(const CgArgs& a, Smem& sm, int nf, int nchunks, Sync& sync)
{
    const int tid = threadIdx.x;
    const int ncta = sync.size();
    const int cta = sync.rank();
    const int c0 = (int)(((int64_t)cta * nchunks) / ncta);
    const int c1 = (int)(((int64_t)(cta + 1) * nchunks) / ncta);
    const int kb = c1 - c0;                // chunks owned
    const int e0 = c0 * CHUNK;             // owned element range [e0, e1)
    const int e1 = min(c1 * CHUNK, nf);
    // One CTA owning every chunk keeps the reductions in shared memory.
    const bool local = ncta == 1 && nchunks <= 32;
    const float* dtab = sm.dtab;
    const float* itab = sm.itab;
    (void)e0;
    (void)e1;

    // ---- initialisation: x = 0, r = b, z = M^-1 r; bb = r.r, rz = r.z
    for (int base = 0; base < kb; base += 32) {
        const int nslot = min(32, kb - base);
        for (int sl = 0; sl < nslot; ++sl) {
            const int s = base + sl;
            const int e = (c0 + s) * CHUNK + tid;
            Elem<R> v[2] = {Elem<R>(), Elem<R>()};
            if (e < nf) {
                const float r = a.b[e];
                const uint8_t fl = a.flags[e];
                const float z = fmul(itab[fl >> 2], r);
                __stcg(&a.z[e], z);
                v[0] = Ar<R>::prod(r, r);
                v[1] = Ar<R>::prod(r, z);
                __stcg(&a.x[e], 0.0f);
                __stcg(&a.r[e], r);
            }
            level1<R, 2>(v, sl, sm);
        }
        if (!local) level2<R, 2, std::is_same<Sync, GridSync>::value>(a, 0, c0 + base, nslot, sm);
    }
    Acc<R> red2[2];
    if (local) {
        local_reduce<R, 2>(nchunks, sm, red2);
    } else {
        if (!sync.barrier(a, sm)) return;
        if (!reduce_all<R, 2>(a, 0, nchunks, sm, red2, sync)) return;
    }
    const Acc<R> bb = red2[0];
    Acc<R> rz = red2[1];
    Acc<R> rr = bb;
    int iters = 0;
    bool done = bb == Acc<R>(0);
    const Acc<R> tolr = (Acc<R>)a.tol;
    Acc<R> thr = Ar<R>::mul(Ar<R>::mul(tolr, tolr), bb);
    if (thr < Ar<R>::tiny()) thr = Ar<R>::tiny();
    if (!done && rr < thr) done = true;

    bool first = true;
    float beta = 0.0f;
    for (int it = 1; !done && it <= a.maxit; ++it) {
        // ---- phase A: p_new = z + beta p, q = A p_new, partial p.q
        for (int base = 0; base < kb; base += 32) {
            const int nslot = min(32, kb - base);
            for (int sl = 0; sl < nslot; ++sl) {
                const int s = base + sl;
                const int e = (c0 + s) * CHUNK + tid;
                Elem<R> v[1] = {Elem<R>()};
                if (e < nf) {
                    const float pe = remote_p(a, e, first, beta);
                    const unsigned fl = a.flags[e];
                    const int dn = a.down[e], up = a.up[e];
                    float acc = 0.0f;
                    if (dn >= 0) acc = fadd(acc, fmul(a.off, remote_p(a, dn, first, beta)));
                    if (fl & 1u) acc = fadd(acc, fmul(a.off, remote_p(a, e - 1, first, beta)));
                    acc = fadd(acc, fmul(dtab[fl >> 2], pe));
                    if (fl & 2u) acc = fadd(acc, fmul(a.off, remote_p(a, e + 1, first, beta)));
                    if (up >= 0) acc = fadd(acc, fmul(a.off, remote_p(a, up, first, beta)));
                    v[0] = Ar<R>::prod(pe, acc);
                    __stcg(&a.q[e], acc);
                }
                level1<R, 1>(v, sl, sm);
            }
            if (!local) level2<R, 1, std::is_same<Sync, GridSync>::value>(a, 1, c0 + base, nslot, sm);
        }
        Acc<R> red1[1];
        if (local) {
            local_reduce<R, 1>(nchunks, sm, red1);
        } else {
            if (!sync.barrier(a, sm)) return;
            if (!reduce_all<R, 1>(a, 1, nchunks, sm, red1, sync)) return;
        }
        const float alpha = Ar<R>::ratio(rz, red1[0]);

        // ---- phase B: x += alpha p, r -= alpha q, z = M^-1 r; publish z, p; partial r.r, r.z
        for (int base = 0; base < kb; base += 32) {
            const int nslot = min(32, kb - base);
            for (int sl = 0; sl < nslot; ++sl) {
                const int s = base + sl;
                const int e = (c0 + s) * CHUNK + tid;
                Elem<R> v[2] = {Elem<R>(), Elem<R>()};
                if (e < nf) {
                    const float pn = remote_p(a, e, first, beta);
                    float x = __ldcg(&a.x[e]);
                    float r = __ldcg(&a.r[e]);
                    const float q = __ldcg(&a.q[e]);
                    const unsigned fl = a.flags[e];
                    x = fadd(x, fmul(alpha, pn));
                    r = fsub(r, fmul(alpha, q));
                    const float z = fmul(itab[fl >> 2], r);
                    __stcg(&a.x[e], x);
                    __stcg(&a.r[e], r);
                    __stcg(&a.z[e], z);
                    __stcg(&a.p[e], pn);
                    v[0] = Ar<R>::prod(r, r);
                    v[1] = Ar<R>::prod(r, z);
                }
                level1<R, 2>(v, sl, sm);
            }
            if (!local) level2<R, 2, std::is_same<Sync, GridSync>::value>(a, 0, c0 + base, nslot, sm);
        }
        if (local) {
            local_reduce<R, 2>(nchunks, sm, red2);
        } else {
            if (!sync.barrier(a, sm)) return;
            if (!reduce_all<R, 2>(a, 0, nchunks, sm, red2, sync)) return;
        }
        rr = red2[0];
        iters = it;
        if (rr < thr) break;
        beta = Ar<R>::ratio(red2[1], rz);
        rz = red2[1];
        first = false;
    }
    if (cta == 0 && tid == 0) {
        a.result->iterations = iters;
        a.result->rr = (double)rr;
        a.result->bb = (double)bb;
        a.result->status = 0;
    }
}

// ---- asynchronous copies into shared memory (cp.async: generic proxy, the
// copying thread waits for its own groups).  Shared destinations are
// shared-window addresses, global sources global-window addresses.
__device__ __forceinline__ unsigned long long gaddr(const void* p)
{
    return (unsigned long long)__cvta_generic_to_global(p);
}
__device__ __forceinline__ void cp_async16(unsigned dst, unsigned long long src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(unsigned dst, unsigned long long src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// Until at most N of this thread's most recent groups are pending.
template <int N>
__device__ __forceinline__ void cp_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
template <int N>
using IntC = std::integral_constant<int, N>;

// The pipelined streaming form's copy schedule (fs_pipeline.h).
constexpr int PIPE_MIN_CHUNKS = pipe::MIN_CHUNKS;
constexpr int PIPE_WARP_BYTES = pipe::WARP_BYTES;
using pipe::PA_AHEAD;
using pipe::PA_ENTRY;
using pipe::PA_PEEL;
using pipe::PA_STAGES;
using pipe::PB_AHEAD;
using pipe::PB_ENTRY;
using pipe::PB_STAGES;
using pipe::PG_AHEAD;
using pipe::PG_ENTRY;
using pipe::PG_STAGES;
using pipe::pa_wait1;
using pipe::pa_wait2;
static_assert(32 * PIPE_WARP_BYTES <= (int)LARGE_DYN_BYTES, "the warps' regions fit k_cg_large's shared memory");

// The streaming solve (state in global memory) with the cells' operands
// copied into shared memory several slots ahead of their use.  The
// arithmetic, the reduction tree and the exchanges are those of cg_stream;
// only where each operand is read from differs.  Used by grid launches only
// (every chunk partial goes through global memory).  The system arrays are
// read in whole 1024-cell chunks, so they must be allocated to the last
// chunk's end.
template <typename R, class Sync>
__device__ __forceinline__ void cg_pipe(const CgArgs& a, Smem& sm, unsigned char* dyn, int nf, int nchunks,
                                        Sync& sync)
{
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int ncta = sync.size();
    const int cta = sync.rank();
    const int c0 = (int)(((int64_t)cta * nchunks) / ncta);
    const int c1 = (int)(((int64_t)(cta + 1) * nchunks) / ncta);
    const int kb = c1 - c0;
    const int e0 = c0 * CHUNK;
    const int e_end = c1 * CHUNK;  // first element of the next CTA's chunks
    const int NONE = 0x7fffffff;   // slot base of a slot past the CTA's last
    const float* dtab = sm.dtab;
    const float* itab = sm.itab;
    const float off = a.off;
    unsigned char* const wb = dyn + (size_t)warp * PIPE_WARP_BYTES;
    const unsigned swb = (unsigned)__cvta_generic_to_shared(wb);
    unsigned char* const gring = wb + PA_STAGES * PA_ENTRY;
    const unsigned sgring = swb + PA_STAGES * PA_ENTRY;
    bool first = true;
    float beta = 0.0f;
    auto slot_base = [&](int k) { return k < kb ? (c0 + k) * CHUNK + warp * 32 : NONE; };

    // This lane's copies, fixed for the solve: source = base + slot base x
    // scale, destination = entry + offset.  Phase A: 16 bytes of z, p, down or
    // up (lane / 8, piece lane % 8), then lanes 0-1 the flags, 2-3 z and p of
    // the 4 cells before the warp's, 4-5 z and p of the 4 after them.  Phase
    // B: 16 bytes of z, p, x or r, then lanes 0-7 q and 8-9 the flags.
    const int arr = lane >> 3, piece = lane & 7;
    const unsigned long long gz = gaddr(a.z), gp = gaddr(a.p), gfl = gaddr(a.flags);
    const unsigned long long a1_src =
        (arr == 0 ? gz : arr == 1 ? gp : arr == 2 ? gaddr(a.down) : gaddr(a.up)) + piece * 16;
    const int a2_kind = lane < 2 ? 0 : lane < 4 ? 1 : lane < 6 ? 2 : 3;  // flags, before, after, none
    const unsigned long long a2_src = a2_kind == 0   ? gfl + lane * 16
                                      : a2_kind == 1 ? (lane == 2 ? gz : gp) - 16
                                                     : (lane == 4 ? gz : gp) + 128;
    const unsigned a2_scale = a2_kind == 0 ? 1u : 4u;
    const unsigned a2_dst = a2_kind == 0 ? 512 + lane * 16 : 544 + (lane - 2) * 16;
    const unsigned long long b1_src =
        (arr == 0 ? gz : arr == 1 ? gp : arr == 2 ? gaddr(a.x) : gaddr(a.r)) + piece * 16;
    const bool b2_on = lane < 10;
    const unsigned long long b2_src = lane < 8 ? gaddr(a.q) + lane * 16 : gfl + (lane - 8) * 16;
    const unsigned b2_scale = lane < 8 ? 4u : 1u;

    // Stage 1 of phase A for the slot at element base eb into the entry at
    // shared address dst.  Before the barrier that publishes the other CTAs'
    // z and p (post == false), the piece before the CTA's first cell is left
    // out; fix_edge copies it after the barrier.
    auto issue_a1 = [&](int eb, unsigned dst, bool post) {
        if (eb >= nf) return;
        cp_async16(dst + lane * 16, a1_src + (unsigned)eb * 4u);
        const bool on = a2_kind == 0 || (a2_kind == 1 && eb > 0 && (post || eb != e0)) ||
                        (a2_kind == 2 && eb + 32 < nf && (post || eb + 32 != e_end));
        if (on) cp_async16(dst + a2_dst, a2_src + (unsigned long long)((unsigned)eb * a2_scale));
    };
    auto fix_edge = [&]() {
        if (warp == 0 && (lane == 2 || lane == 3) && e0 > 0)
            cp_async16(swb + a2_dst, a2_src + (unsigned long long)((unsigned)e0 * 4u));
    };
    // Stage 2 of phase A for the slot at element base eb (indices in its
    // stage-1 entry en): z and p of the down and up neighbours into the gather
    // entry at dst.
    auto issue_gather = [&](int eb, const unsigned char* en, unsigned dst) {
        if (eb >= nf || eb + lane >= nf) return;
        const int dn = reinterpret_cast<const int*>(en + 256)[lane];
        const int up = reinterpret_cast<const int*>(en + 384)[lane];
        if (dn >= 0) {
            cp_async4(dst + lane * 4, gz + (unsigned)dn * 4u);
            if (!first) cp_async4(dst + 128 + lane * 4, gp + (unsigned)dn * 4u);
        }
        if (up >= 0) {
            cp_async4(dst + 256 + lane * 4, gz + (unsigned)up * 4u);
            if (!first) cp_async4(dst + 384 + lane * 4, gp + (unsigned)up * 4u);
        }
    };
    auto issue_b = [&](int eb, unsigned dst) {
        if (eb >= nf) return;
        cp_async16(dst + lane * 16, b1_src + (unsigned)eb * 4u);
        if (b2_on) cp_async16(dst + 512 + lane * 16, b2_src + (unsigned long long)((unsigned)eb * b2_scale));
    };
    auto prologue_a = [&]() {
        for (int k = 0; k < PA_AHEAD; ++k) {
            issue_a1(slot_base(k), swb + k * PA_ENTRY, false);
            cp_commit();
        }
    };
    auto prologue_b = [&]() {
        for (int k = 0; k < PB_AHEAD; ++k) {
            issue_b(slot_base(k), swb + k * PB_ENTRY);
            cp_commit();
        }
    };
    auto pnew = [&](float z, float p) { return first ? z : fadd(z, fmul(beta, p)); };
    auto wrap = [](int o, int stride, int end) { return o + stride == end ? 0 : o + stride; };

    // ---- initialisation: x = 0, r = b, z = M^-1 r; bb = r.r, rz = r.z
    for (int base = 0; base < kb; base += 32) {
        const int nslot = min(32, kb - base);
        for (int sl = 0; sl < nslot; ++sl) {
            const int e = (c0 + base + sl) * CHUNK + tid;
            Elem<R> v[2] = {Elem<R>(), Elem<R>()};
            if (e < nf) {
                const float r = a.b[e];
                const uint8_t fl = a.flags[e];
                const float z = fmul(itab[fl >> 2], r);
                __stcg(&a.z[e], z);
                v[0] = Ar<R>::prod(r, r);
                v[1] = Ar<R>::prod(r, z);
                __stcg(&a.x[e], 0.0f);
                __stcg(&a.r[e], r);
            }
            level1<R, 2>(v, sl, sm);
        }
        level2<R, 2>(a, 0, c0 + base, nslot, sm);
    }
    prologue_a();
    Acc<R> red2[2];
    if (!sync.barrier(a, sm)) {
        cp_wait_all();
        return;
    }
    if (!reduce_all<R, 2>(a, 0, nchunks, sm, red2, sync)) {
        cp_wait_all();
        return;
    }
    const Acc<R> bb = red2[0];
    Acc<R> rz = red2[1];
    Acc<R> rr = bb;
    int iters = 0;
    bool done = bb == Acc<R>(0);
    const Acc<R> tolr = (Acc<R>)a.tol;
    Acc<R> thr = Ar<R>::mul(Ar<R>::mul(tolr, tolr), bb);
    if (thr < Ar<R>::tiny()) thr = Ar<R>::tiny();
    if (!done && rr < thr) done = true;

    constexpr int A_END = PA_STAGES * PA_ENTRY, G_END = PG_STAGES * PG_ENTRY, B_END = PB_STAGES * PB_ENTRY;
    for (int it = 1; !done && it <= a.maxit; ++it) {
        // ---- phase A: p_new = z + beta p, q = A p_new, partial p.q
        // Ring offsets: oa / og of slot k's entries, oa_g of slot
        // k + PG_AHEAD's stage-1 entry; slot k + PA_AHEAD reuses slot k - 1's
        // stage-1 entry (oa_prev), and slot k + PG_AHEAD slot k - 1's gather
        // entry (og_prev).
        fix_edge();
        for (int j = 0; j < PG_AHEAD; ++j) {
            cp_wait<pipe::PA_WAIT_PROLOGUE>();  // G1(j)
            __syncwarp();
            issue_gather(slot_base(j), wb + j * PA_ENTRY, sgring + j * PG_ENTRY);
            cp_commit();
        }
        int oa = 0, oa_prev = A_END - PA_ENTRY, oa_g = PG_AHEAD * PA_ENTRY, og = 0, og_prev = G_END - PG_ENTRY;
        auto step_a = [&](int k, auto w1, auto w2) {
            cp_wait<decltype(w1)::value>();  // G1(k + PG_AHEAD)
            __syncwarp();
            issue_gather(slot_base(k + PG_AHEAD), wb + oa_g, sgring + og_prev);
            cp_commit();
            issue_a1(slot_base(k + PA_AHEAD), swb + oa_prev, true);
            cp_commit();
            cp_wait<decltype(w2)::value>();  // G2(k)
            __syncwarp();
            const unsigned char* en = wb + oa;
            const float* ez = reinterpret_cast<const float*>(en);
            const float* edge = reinterpret_cast<const float*>(en + 544);
            const float* g = reinterpret_cast<const float*>(gring + og);
            const int e = (c0 + k) * CHUNK + warp * 32 + lane;
            float pe = 0.0f;
            if (e < nf) pe = pnew(ez[lane], ez[32 + lane]);
            float pl = __shfl_up_sync(0xffffffffu, pe, 1);
            float pr = __shfl_down_sync(0xffffffffu, pe, 1);
            Elem<R> v[1] = {Elem<R>()};
            if (e < nf) {
                const unsigned fl = en[512 + lane];
                const int dn = reinterpret_cast<const int*>(en + 256)[lane];
                const int up = reinterpret_cast<const int*>(en + 384)[lane];
                if (lane == 0 && (fl & 1u)) pl = pnew(edge[3], edge[7]);
                if (lane == 31 && (fl & 2u)) pr = pnew(edge[8], edge[12]);
                float acc = 0.0f;
                if (dn >= 0) acc = fadd(acc, fmul(off, pnew(g[lane], g[32 + lane])));
                if (fl & 1u) acc = fadd(acc, fmul(off, pl));
                acc = fadd(acc, fmul(dtab[fl >> 2], pe));
                if (fl & 2u) acc = fadd(acc, fmul(off, pr));
                if (up >= 0) acc = fadd(acc, fmul(off, pnew(g[64 + lane], g[96 + lane])));
                v[0] = Ar<R>::prod(pe, acc);
                __stcg(&a.q[e], acc);
            }
            level1<R, 1>(v, k & 31, sm);
            if ((k & 31) == 31 || k == kb - 1) level2<R, 1>(a, 1, c0 + (k & ~31), (k & 31) + 1, sm);
            oa_prev = oa;
            oa = wrap(oa, PA_ENTRY, A_END);
            oa_g = wrap(oa_g, PA_ENTRY, A_END);
            og_prev = og;
            og = wrap(og, PG_ENTRY, G_END);
        };
        step_a(0, IntC<pa_wait1(0)>{}, IntC<pa_wait2(0)>{});
        step_a(1, IntC<pa_wait1(1)>{}, IntC<pa_wait2(1)>{});
        step_a(2, IntC<pa_wait1(2)>{}, IntC<pa_wait2(2)>{});
        static_assert(PA_PEEL == 3, "three peeled slots above");
        for (int k = PA_PEEL; k < kb; ++k) step_a(k, IntC<pa_wait1(PA_PEEL)>{}, IntC<pa_wait2(PA_PEEL)>{});
        prologue_b();
        Acc<R> red1[1];
        if (!sync.barrier(a, sm)) {
            cp_wait_all();
            return;
        }
        if (!reduce_all<R, 1>(a, 1, nchunks, sm, red1, sync)) {
            cp_wait_all();
            return;
        }
        const float alpha = Ar<R>::ratio(rz, red1[0]);

        // ---- phase B: x += alpha p, r -= alpha q, z = M^-1 r; publish z, p; partial r.r, r.z
        // Groups: GB(0..PB_AHEAD-1) before the barrier, then GB(k + PB_AHEAD)
        // per slot k, into slot k - 1's entry.
        int ob = 0, ob_prev = B_END - PB_ENTRY;
        for (int k = 0; k < kb; ++k) {
            issue_b(slot_base(k + PB_AHEAD), swb + ob_prev);
            cp_commit();
            cp_wait<pipe::PB_WAIT>();  // GB(k)
            __syncwarp();
            const float* en = reinterpret_cast<const float*>(wb + ob);
            const unsigned char* efl = wb + ob + 640;
            const int e = (c0 + k) * CHUNK + warp * 32 + lane;
            Elem<R> v[2] = {Elem<R>(), Elem<R>()};
            if (e < nf) {
                const float pn = pnew(en[lane], en[32 + lane]);
                float x = en[64 + lane];
                float r = en[96 + lane];
                const float q = en[128 + lane];
                const unsigned fl = efl[lane];
                x = fadd(x, fmul(alpha, pn));
                r = fsub(r, fmul(alpha, q));
                const float z = fmul(itab[fl >> 2], r);
                __stcg(&a.x[e], x);
                __stcg(&a.r[e], r);
                __stcg(&a.z[e], z);
                __stcg(&a.p[e], pn);
                v[0] = Ar<R>::prod(r, r);
                v[1] = Ar<R>::prod(r, z);
            }
            level1<R, 2, true>(v, k & 31, sm);
            if ((k & 31) == 31 || k == kb - 1) level2<R, 2>(a, 0, c0 + (k & ~31), (k & 31) + 1, sm);
            ob_prev = ob;
            ob = wrap(ob, PB_ENTRY, B_END);
        }
        prologue_a();
        if (!sync.barrier(a, sm)) {
            cp_wait_all();
            return;
        }
        if (!reduce_all<R, 2>(a, 0, nchunks, sm, red2, sync)) {
            cp_wait_all();
            return;
        }
        rr = red2[0];
        iters = it;
        if (rr < thr) break;
        beta = Ar<R>::ratio(red2[1], rz);
        rz = red2[1];
        first = false;
    }
    cp_wait_all();
    if (cta == 0 && tid == 0) {
        a.result->iterations = iters;
        a.result->rr = (double)rr;
        a.result->bb = (double)bb;
        a.result->status = 0;
    }
}

// Register-resident form of the solve, for CTAs that own at most K chunks.
// The owned cells' z (q between the SpMV and the update) live in registers,
// and r and p too for K <= 4 (slot s of thread t is element
// (c0 + s) * CHUNK + t); shared memory holds what other threads read, x, and
// r for K > 4:
//   pv[K * CHUNK + hcap + 1]: p of the owned cells at [s * CHUNK + t], then
//     the halo -- p_new of the remote cells the rows read, which lie in
//     [lo, e0) and [e1, hi) of the fluid order, staged once per iteration from
//     the published z and p_old -- then one +0 that absent neighbours index;
//   nb[K * CHUNK]: the pv indices of each row's down, left, right and up
//     neighbours, 16 bits each;
//   xs[K * CHUNK]: x;  rsm[K * CHUNK]: r (K > 4).
// A row adds its five terms in the same order as cg_stream; an absent
// neighbour contributes off * (+0) = +0, and adding +0 leaves the running sum
// unchanged because the sum starts at +0 and so is never -0.  Returns false,
// before any exchange with other CTAs, when the halo does not fit; the caller
// then runs the streaming body, whose arithmetic and exchanges are the same.
__device__ __forceinline__ int lean_halo_cap(int K, int dyn_bytes)
{
    const int cells = K * CHUNK;
    const int per_cell = K <= 4 ? 12 : K <= 8 ? 16 : 12;  // nb (8 or 4 bytes), x, r above 4 chunks
    const int cap = (dyn_bytes - per_cell * cells - 8) / 4 - cells - 1;
    return min(cap, (K > 8 ? 32767 : 65535) - cells);
}

template <int K, typename R, class Sync>
__device__ __forceinline__ bool cg_lean(const CgArgs& a, Smem& sm, unsigned char* dyn, int nf, int nchunks,
                                        Sync& sync)
{
    const int tid = threadIdx.x;
    const int ncta = sync.size();
    const int cta = sync.rank();
    const int c0 = (int)(((int64_t)cta * nchunks) / ncta);
    const int c1 = (int)(((int64_t)(cta + 1) * nchunks) / ncta);
    const int kb = c1 - c0;
    const int e0 = c0 * CHUNK;
    const int e1 = min(c1 * CHUNK, nf);
    const bool local = ncta == 1 && nchunks <= 32;
    const bool publish = !local;
    constexpr int OWN = K * CHUNK;
    // Above 8 chunks a row is one 32-bit word: the down and up indices (15
    // bits each), bit 15 left and bit 31 right neighbour liquid.  Those two
    // are the adjacent cells of the fluid order: the adjacent entries of pv,
    // or at the ends of the CTA's range the nearest halo cells.
    constexpr bool NB4 = K > 8;
    const int hcap = lean_halo_cap(K, a.dyn_bytes);
    float* pv = reinterpret_cast<float*>(dyn);
    unsigned char* const nbp = dyn + (((size_t)(OWN + hcap + 1) * 4 + 7) & ~(size_t)7);
    uint2* nb = reinterpret_cast<uint2*>(nbp);
    unsigned* nb4 = reinterpret_cast<unsigned*>(nbp);
    float* xs = reinterpret_cast<float*>(nbp + (size_t)OWN * (NB4 ? 4 : 8));
    float* rsm = xs + OWN;
    constexpr bool PREG = K <= 4;  // p of the owned cells in registers (else read back from pv)
    const float* dtab = sm.dtab;
    const float* itab = sm.itab;
    const float off = a.off;

    // ---- halo extent: the lowest down/left and highest up/right neighbour outside [e0, e1)
    if (tid == 0) {
        sm.hlo = e0;
        sm.hhi = e1;
    }
    __syncthreads();
    {
        int lo = e0, hi = e1;
#pragma unroll
        for (int s = 0; s < K; ++s) {
            const int e = (c0 + s) * CHUNK + tid;
            if (s < kb && e < nf) {
                const int dn = a.down[e], up = a.up[e];
                const unsigned fl = a.flags[e];
                if (dn >= 0 && dn < e0) lo = min(lo, dn);
                if ((fl & 1u) && e - 1 < e0) lo = min(lo, e - 1);
                if (up >= e1) hi = max(hi, up + 1);
                if ((fl & 2u) && e + 1 >= e1) hi = max(hi, e + 2);
            }
        }
        if (lo < e0) atomicMin(&sm.hlo, lo);
        if (hi > e1) atomicMax(&sm.hhi, hi);
    }
    __syncthreads();
    const int lo = sm.hlo, hi = sm.hhi;
    const int nbelow = e0 - lo;
    const int nhalo = nbelow + (hi - e1);
    if (nhalo > hcap) return false;  // uniform over the CTA
    const unsigned zero_i = (unsigned)(OWN + hcap);
    auto slot_of = [&](int n) -> unsigned {
        if (n < 0) return zero_i;
        if (n >= e0 && n < e1) return (unsigned)(n - e0);
        if (n < e0) return (unsigned)(OWN + n - lo);
        return (unsigned)(OWN + nbelow + n - e1);
    };

    // ---- initialisation: x = 0, r = b, z = M^-1 r; bb = r.r, rz = r.z
    float rreg[PREG ? K : 1], zq[K], pn[PREG ? K : 1];
    using Cnt = std::conditional_t<(K > 8), unsigned long long, unsigned>;
    Cnt cnts = 0;  // non-solid neighbour count of slot s in bits 4s..4s+2
    if (tid == 0) pv[zero_i] = 0.0f;
#pragma unroll
    for (int s = 0; s < K; ++s) {
        if constexpr (PREG) rreg[s] = 0.0f;
        zq[s] = 0.0f;
        if constexpr (PREG) pn[s] = 0.0f;
        if (s < kb) {
            const int e = (c0 + s) * CHUNK + tid;
            Elem<R> v[2] = {Elem<R>(), Elem<R>()};
            if (e < nf) {
                const float rb = a.b[e];
                const unsigned fl = a.flags[e];
                const float z = fmul(itab[fl >> 2], rb);
                if (publish) __stcg(&a.z[e], z);
                v[0] = Ar<R>::prod(rb, rb);
                v[1] = Ar<R>::prod(rb, z);
                if constexpr (PREG) rreg[s] = rb;
                else rsm[s * CHUNK + tid] = rb;
                zq[s] = z;
                xs[s * CHUNK + tid] = 0.0f;
                if constexpr (!PREG) pv[s * CHUNK + tid] = 0.0f;
                cnts |= (Cnt)(fl >> 2) << (4 * s);
                const unsigned i_dn = slot_of(a.down[e]);
                const unsigned i_up = slot_of(a.up[e]);
                if constexpr (NB4) {
                    nb4[s * CHUNK + tid] = i_dn | (i_up << 16) | ((fl & 1u) << 15) | ((fl & 2u) << 30);
                } else {
                    const unsigned i_l = (fl & 1u) ? slot_of(e - 1) : zero_i;
                    const unsigned i_r = (fl & 2u) ? slot_of(e + 1) : zero_i;
                    nb[s * CHUNK + tid] = make_uint2(i_dn | (i_l << 16), i_r | (i_up << 16));
                }
            }
            level1<R, 2>(v, s, sm);
        }
    }
    // Across the grid, the first HALO_PRE halo cells' z and p_old are loaded
    // right after the barrier that publishes them, so that their round trip
    // overlaps the partial-sum loads of reduce_all instead of following it.
    // (A cluster barrier has no such round trip to hide behind.)
    constexpr int HALO_PRE = std::is_same<Sync, GridSync>::value ? 2 : 0;
    float hz[HALO_PRE > 0 ? HALO_PRE : 1], hp[HALO_PRE > 0 ? HALO_PRE : 1];
    auto prefetch = [&](bool with_p) {
#pragma unroll
        for (int j = 0; j < HALO_PRE; ++j) {
            const int h = tid + j * CHUNK;
            if (h < nhalo) {
                const int n = h < nbelow ? lo + h : e1 + (h - nbelow);
                hz[j] = __ldcg(&a.z[n]);
                if (with_p) hp[j] = __ldcg(&a.p[n]);
            }
        }
    };
    if (!local) level2<R, 2, std::is_same<Sync, GridSync>::value>(a, 0, c0, kb, sm);
    Acc<R> red2[2];
    if (local) {
        local_reduce<R, 2>(nchunks, sm, red2);
    } else {
        if (!sync.barrier(a, sm)) return true;
        prefetch(false);
        if (!reduce_all<R, 2>(a, 0, nchunks, sm, red2, sync)) return true;
    }
    const Acc<R> bb = red2[0];
    Acc<R> rz = red2[1];
    Acc<R> rr = bb;
    int iters = 0;
    bool done = bb == Acc<R>(0);
    const Acc<R> tolr = (Acc<R>)a.tol;
    Acc<R> thr = Ar<R>::mul(Ar<R>::mul(tolr, tolr), bb);
    if (thr < Ar<R>::tiny()) thr = Ar<R>::tiny();
    if (!done && rr < thr) done = true;

    bool first = true;
    float beta = 0.0f;
    for (int it = 1; !done && it <= a.maxit; ++it) {
        // ---- phase A: p_new = z + beta p (own cells and halo), q = A p_new, partial p.q
#pragma unroll
        for (int s = 0; s < K; ++s) {
            if (s < kb && (c0 + s) * CHUNK + tid < nf) {
                float& ps = PREG ? pn[s] : pv[s * CHUNK + tid];
                const float np = first ? zq[s] : fadd(zq[s], fmul(beta, ps));
                if constexpr (PREG) pn[s] = np;
                pv[s * CHUNK + tid] = np;
            }
        }
#pragma unroll
        for (int j = 0; j < HALO_PRE; ++j) {
            const int h = tid + j * CHUNK;
            if (h < nhalo) pv[OWN + h] = first ? hz[j] : fadd(hz[j], fmul(beta, hp[j]));
        }
        for (int h = tid + HALO_PRE * CHUNK; h < nhalo; h += CHUNK) {
            const int n = h < nbelow ? lo + h : e1 + (h - nbelow);
            const float zn = __ldcg(&a.z[n]);
            pv[OWN + h] = first ? zn : fadd(zn, fmul(beta, __ldcg(&a.p[n])));
        }
        __syncthreads();
        // with float dots, the p.q trees of slots 2i and 2i + 1 share one tree
        // of packed adds (a slot past the CTA's range adds zeros into a level-1
        // entry nothing reads)
        constexpr bool PAIR_A = std::is_same<R, float>::value && K % 2 == 0;
        float held = 0.0f;
#pragma unroll
        for (int s = 0; s < K; ++s) {
            if (PAIR_A || s < kb) {
                Elem<R> v[1] = {Elem<R>()};
                if (s < kb && (c0 + s) * CHUNK + tid < nf) {
                    const float ps = PREG ? pn[s] : pv[s * CHUNK + tid];
                    float acc = 0.0f;
                    if constexpr (NB4) {
                        const unsigned w = nb4[s * CHUNK + tid];
                        const int l = s * CHUNK + tid;  // = e - e0
                        const unsigned il = !(w & 0x8000u) ? zero_i
                                            : l > 0        ? (unsigned)(l - 1)
                                                           : (unsigned)(OWN + nbelow - 1);
                        const unsigned ir = !(w & 0x80000000u) ? zero_i
                                            : l + 1 < e1 - e0  ? (unsigned)(l + 1)
                                                               : (unsigned)(OWN + nbelow);
                        acc = fadd(acc, fmul(off, pv[w & 0x7fffu]));
                        acc = fadd(acc, fmul(off, pv[il]));
                        acc = fadd(acc, fmul(dtab[(unsigned)(cnts >> (4 * s)) & 7u], ps));
                        acc = fadd(acc, fmul(off, pv[ir]));
                        acc = fadd(acc, fmul(off, pv[(w >> 16) & 0x7fffu]));
                    } else {
                        const uint2 w = nb[s * CHUNK + tid];
                        acc = fadd(acc, fmul(off, pv[w.x & 0xffffu]));
                        acc = fadd(acc, fmul(off, pv[w.x >> 16]));
                        acc = fadd(acc, fmul(dtab[(cnts >> (4 * s)) & 7u], ps));
                        acc = fadd(acc, fmul(off, pv[w.y & 0xffffu]));
                        acc = fadd(acc, fmul(off, pv[w.y >> 16]));
                    }
                    v[0] = Ar<R>::prod(ps, acc);
                    zq[s] = acc;
                }
                if constexpr (PAIR_A) {
                    if (s % 2 == 0) held = v[0];
                    else if (s - 1 < kb) level1_pair(held, v[0], s - 1, sm);
                } else {
                    level1<R, 1>(v, s, sm);
                }
            }
        }
        if (!local) level2<R, 1, std::is_same<Sync, GridSync>::value>(a, 1, c0, kb, sm);
        Acc<R> red1[1];
        if (local) {
            local_reduce<R, 1>(nchunks, sm, red1);
        } else {
            if (!sync.barrier(a, sm)) return true;
            if (!reduce_all<R, 1>(a, 1, nchunks, sm, red1, sync)) return true;
        }
        const float alpha = Ar<R>::ratio(rz, red1[0]);

        // ---- phase B: x += alpha p, r -= alpha q, z = M^-1 r; publish z, p; partial r.r, r.z
#pragma unroll
        for (int s = 0; s < K; ++s) {
            if (s < kb) {
                const int e = (c0 + s) * CHUNK + tid;
                Elem<R> v[2] = {Elem<R>(), Elem<R>()};
                if (e < nf) {
                    const float ps = PREG ? pn[s] : pv[s * CHUNK + tid];
                    const int l = s * CHUNK + tid;
                    xs[l] = fadd(xs[l], fmul(alpha, ps));
                    float& rr_ = PREG ? rreg[s] : rsm[l];
                    const float rn = fsub(rr_, fmul(alpha, zq[s]));
                    rr_ = rn;
                    const float z = fmul(itab[(unsigned)(cnts >> (4 * s)) & 7u], rn);
                    zq[s] = z;
                    if (publish) {
                        __stcg(&a.z[e], z);
                        __stcg(&a.p[e], ps);
                    }
                    v[0] = Ar<R>::prod(rn, rn);
                    v[1] = Ar<R>::prod(rn, z);
                }
                level1<R, 2>(v, s, sm);
            }
        }
        if (!local) level2<R, 2, std::is_same<Sync, GridSync>::value>(a, 0, c0, kb, sm);
        if (local) {
            local_reduce<R, 2>(nchunks, sm, red2);
        } else {
            if (!sync.barrier(a, sm)) return true;
            prefetch(true);
            if (!reduce_all<R, 2>(a, 0, nchunks, sm, red2, sync)) return true;
        }
        rr = red2[0];
        iters = it;
        if (rr < thr) break;
        beta = Ar<R>::ratio(red2[1], rz);
        rz = red2[1];
        first = false;
    }
#pragma unroll
    for (int s = 0; s < K; ++s) {
        const int e = (c0 + s) * CHUNK + tid;
        if (s < kb && e < nf) a.x[e] = xs[s * CHUNK + tid];
    }
    if (cta == 0 && tid == 0) {
        a.result->iterations = iters;
        a.result->rr = (double)rr;
        a.result->bb = (double)bb;
        a.result->status = 0;
    }
    return true;
}

// Whether k_cg_large solves a system of nchunks chunks on `grid` CTAs: from
// KREG + 1 to KBIG chunks per CTA (the register-resident form with 4-byte
// rows) and from PIPE_MIN_CHUNKS on (the pipelined streaming form).
__device__ __forceinline__ bool large_takes(int nchunks, int grid)
{
    const int per_cta = (nchunks + grid - 1) / grid;
    return nchunks > SINGLE_CTA_CHUNKS && ((per_cta > KREG && per_cta <= KBIG) || per_cta >= PIPE_MIN_CHUNKS);
}

// Splits a solve between k_cg and k_cg_large: route[0] = the fluid cells k_cg
// solves, route[1] = those k_cg_large solves; one of the two is 0 (k_cg keeps
// the systems it rejects, to report them).
__global__ void k_cg_route(const int32_t* __restrict__ nfluid, int max_chunks, int grid, int32_t* __restrict__ route)
{
    const int nf = *nfluid;
    const int nchunks = (nf + CHUNK - 1) / CHUNK;
    const bool large = nchunks <= max_chunks && nchunks <= MAX_CHUNKS && large_takes(nchunks, grid);
    route[0] = large ? 0 : nf;
    route[1] = large ? nf : 0;
}

// Large systems with float (R = float) or double-single (R = DSD) dot
// products, on the system k_cg_route gave it (none: return without a result;
// k_cg wrote it): up to KBIG chunks per CTA in registers and shared memory,
// from PIPE_MIN_CHUNKS on streamed through the cp.async pipeline.
template <typename R>
__global__ void __launch_bounds__(CG_THREADS, 1) k_cg_large(CgArgs a)
{
    __shared__ Smem sm;
    extern __shared__ __align__(16) unsigned char dyn[];
    const int nf = *a.nfluid;
    if (nf == 0) return;
    const int nchunks = (nf + CHUNK - 1) / CHUNK;
    const int per_cta = (nchunks + gridDim.x - 1) / gridDim.x;
    const int active = (nchunks + per_cta - 1) / per_cta;
    if ((int)blockIdx.x >= active) return;
    if (threadIdx.x < 5) {
        sm.dtab[threadIdx.x] = a.dtab[threadIdx.x];
        sm.itab[threadIdx.x] = a.itab[threadIdx.x];
    }
    __syncthreads();
    GridSync sync{true, 0u, active};
    if (per_cta <= KBIG) {
        if (!cg_lean<KBIG, R>(a, sm, dyn, nf, nchunks, sync)) cg_stream<R>(a, sm, nf, nchunks, sync);
    } else {
        cg_pipe<R>(a, sm, dyn, nf, nchunks, sync);
    }
}

template <typename R>
__global__ void __launch_bounds__(CG_THREADS, 1) k_cg(CgArgs a)
{
    __shared__ Smem sm;
    extern __shared__ __align__(16) unsigned char dyn[];
    const int nf = *a.nfluid;
    const int nchunks = (nf + CHUNK - 1) / CHUNK;
    if (threadIdx.x < 5) {
        sm.dtab[threadIdx.x] = a.dtab[threadIdx.x];
        sm.itab[threadIdx.x] = a.itab[threadIdx.x];
    }
    __syncthreads();
    if (nchunks == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.result->iterations = 0;
            a.result->rr = 0.0;
            a.result->bb = 0.0;
            a.result->status = 0;
        }
        return;
    }
    if (nchunks > a.max_chunks || nchunks > MAX_CHUNKS) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.status, ST_TOO_LARGE);
        return;
    }
    const bool grid = nchunks > SINGLE_CTA_CHUNKS;
    if (!grid && blockIdx.x != 0) return;
    const int per_cta = grid ? (nchunks + gridDim.x - 1) / gridDim.x : nchunks;
    const bool resident = per_cta <= KREG;
    // the CTAs beyond ceil(nchunks / per_cta) would only add arrivals to every barrier
    const int active = grid ? (nchunks + per_cta - 1) / per_cta : 1;
    if (grid && (int)blockIdx.x >= active) return;
    GridSync sync{grid, 0u, active};
    const bool ran = resident && (per_cta <= 4 ? cg_lean<4, R>(a, sm, dyn, nf, nchunks, sync)
                                               : cg_lean<KREG, R>(a, sm, dyn, nf, nchunks, sync));
    if (!ran) cg_stream<R>(a, sm, nf, nchunks, sync);
}

// A batch of independent systems: one thread-block cluster per system (the
// simulation order[cluster]); up to K chunks per CTA in shared memory.  The
// reduction tree, and so every result, is that of k_cg.
template <int K, typename R>
__global__ void __launch_bounds__(CG_THREADS, 1) k_cg_cluster(CgBatchArgs ba)
{
    __shared__ Smem sm;
    extern __shared__ __align__(16) unsigned char dyn[];
    unsigned cluster;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(cluster));
    const int sim = ba.order[cluster];
    const CgSystem& sy = ba.systems[sim];
    CgArgs a;
    a.nfluid = ba.nfluid + sim;
    a.b = ba.b + sy.co;
    a.down = ba.down + sy.co;
    a.up = ba.up + sy.co;
    a.flags = ba.flags + sy.co;
    a.off = sy.off;  // the diagonal tables go straight to shared memory below
    a.tol = sy.tol;
    a.maxit = sy.maxit;
    a.fp64 = ba.fp64;
    a.x = ba.x + sy.co;
    a.r = ba.r + sy.co;
    a.z = ba.z + sy.co;
    a.p = ba.p + sy.co;
    a.q = ba.q + sy.co;
    a.partials = ba.partials + sy.part_off;
    a.max_chunks = sy.max_chunks;
    a.groups = nullptr;
    a.max_groups = 0;
    a.barrier = nullptr;
    a.status = ba.status;
    a.result = ba.result + sim;
    a.missing = 0;
    a.wait_ns = WAIT_LIMIT_NS;
    a.dyn_bytes = (int)cluster_dyn_bytes(K);
    if (threadIdx.x < 5) {
        sm.dtab[threadIdx.x] = sy.dtab[threadIdx.x];
        sm.itab[threadIdx.x] = sy.itab[threadIdx.x];
    }
    __syncthreads();
    ClusterSync sync;
    const int nf = *a.nfluid;
    const int nchunks = (nf + CHUNK - 1) / CHUNK;
    // Every CTA of the cluster takes the same branch: the system is shared.
    if (nchunks == 0) {
        if (sync.rank() == 0 && threadIdx.x == 0) *a.result = CgResult{0, 0, 0.0, 0.0};
        return;
    }
    if (nchunks > a.max_chunks) {
        if (sync.rank() == 0 && threadIdx.x == 0) atomicOr(a.status, ST_TOO_LARGE);
        return;
    }
    // A system that outgrew the cluster's shared memory streams its state
    // from global memory instead (same arithmetic, same results).
    const bool resident = nchunks <= K * sync.size();
    if (!(resident && cg_lean<K, R>(a, sm, dyn, nf, nchunks, sync))) cg_stream<R>(a, sm, nf, nchunks, sync);
}

}  // namespace

int cg_prepare(CgWork& w, int device)
{
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return -1;
    for (const void* f : {(const void*)k_cg<float>, (const void*)k_cg<double>, (const void*)k_cg<DSD>})
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DYN_BYTES) != cudaSuccess)
            return -1;
    for (const void* f : {(const void*)k_cg_large<float>, (const void*)k_cg_large<DSD>})
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LARGE_DYN_BYTES) !=
            cudaSuccess)
            return -1;
    for (const void* f : {(const void*)k_cg<float>, (const void*)k_cg<double>, (const void*)k_cg<DSD>}) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, CG_THREADS, DYN_BYTES) != cudaSuccess)
            return -1;
        if (per_sm < 1) return -1;
    }
    for (const void* f : {(const void*)k_cg_large<float>, (const void*)k_cg_large<DSD>})
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, CG_THREADS, LARGE_DYN_BYTES) != cudaSuccess ||
            per_sm < 1)
            return -1;
    w.grid = sms;  // one CTA per SM: fewer barrier arrivals
    return 0;
}

void cg_solve(const Launch& L, CgWork& w, const int32_t* nfluid, const float* b, const float* diag_tab,
              const int32_t* down, const int32_t* up, const uint8_t* flags, float off, double tol, int maxit,
              int fp64, unsigned* status)
{
    CgArgs a;
    a.nfluid = nfluid;
    a.b = b;
    a.down = down;
    a.up = up;
    a.flags = flags;
    for (int k = 0; k < 5; ++k) {
        a.dtab[k] = diag_tab[k];
        a.itab[k] = diag_tab[k] != 0.0f ? 1.0f / diag_tab[k] : 1.0f;
    }
    a.off = off;
    a.tol = tol;
    a.maxit = maxit;
    a.fp64 = fp64;
    a.x = w.x;
    a.r = w.r;
    a.z = w.z;
    a.p = w.p;
    a.q = w.q;
    a.partials = w.partials;
    a.max_chunks = (int)((w.max_cells + CHUNK - 1) / CHUNK);
    a.groups = w.groups;
    a.max_groups = (a.max_chunks + 31) / 32;
    a.barrier = w.barrier;
    a.status = status;
    a.result = w.result;
    a.missing = w.missing_arrivals;
    a.wait_ns = w.wait_ns;
    a.dyn_bytes = (int)DYN_BYTES;
    cudaMemsetAsync(w.barrier, 0, sizeof(unsigned), L.stream);
    void* args[] = {&a};
    const void* kernel = fp64 == 2 ? (const void*)k_cg<DSD>
                         : fp64  ? (const void*)k_cg<double>
                                 : (const void*)k_cg<float>;
    // Arrays with room for more than KREG chunks per CTA: k_cg_route decides
    // on the device which of k_cg and k_cg_large solves (float and
    // double-single dots; double dots gain nothing from it).
    const bool large = fp64 != 1 && w.route && (a.max_chunks + w.grid - 1) / w.grid > KREG;
    if (large) {
        k_cg_route<<<1, 1, 0, L.stream>>>(nfluid, a.max_chunks, w.grid, w.route);
        L.count();
        a.nfluid = w.route;
    }
    cudaLaunchCooperativeKernel(kernel, dim3(w.grid), dim3(CG_THREADS), args, DYN_BYTES, L.stream);
    L.count();
    if (large) {
        a.nfluid = w.route + 1;
        a.dyn_bytes = (int)LARGE_DYN_BYTES;
        cudaLaunchCooperativeKernel(fp64 == 2 ? (const void*)k_cg_large<DSD> : (const void*)k_cg_large<float>,
                                    dim3(w.grid), dim3(CG_THREADS), args, LARGE_DYN_BYTES, L.stream);
        L.count();
    }
}

namespace {

template <int K>
int prepare_cluster_kernel(int cluster)
{
    const size_t bytes = cluster_dyn_bytes(K);
    if (cudaFuncSetAttribute(k_cg_cluster<K, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_cg_cluster<K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
            cudaSuccess)
        return -1;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = bytes;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0, n64 = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_cg_cluster<K, float>, &cfg) != cudaSuccess) return -1;
    if (cudaOccupancyMaxActiveClusters(&n64, k_cg_cluster<K, double>, &cfg) != cudaSuccess) return -1;
    return n < n64 ? n : n64;
}

template <int K>
cudaError_t launch_cluster(const Launch& L, const CgBatchArgs& ba, int nsys, int cluster)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(nsys * cluster));
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = cluster_dyn_bytes(K);
    cfg.stream = L.stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = ba.fp64 ? cudaLaunchKernelEx(&cfg, k_cg_cluster<K, double>, ba)
                                  : cudaLaunchKernelEx(&cfg, k_cg_cluster<K, float>, ba);
    L.count();
    return e;
}

}  // namespace

int cg_cluster_capacity(int chunks_per_cta, int cluster)
{
    switch (chunks_per_cta) {
        case 4: return prepare_cluster_kernel<4>(cluster);
        case 8: return prepare_cluster_kernel<8>(cluster);
        default: return -1;
    }
}

cudaError_t cg_solve_clusters(const Launch& L, const CgBatchArgs& ba, int nsys, int chunks_per_cta, int cluster)
{
    if (nsys <= 0) return cudaSuccess;
    switch (chunks_per_cta) {
        case 4: return launch_cluster<4>(L, ba, nsys, cluster);
        case 8: return launch_cluster<8>(L, ba, nsys, cluster);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fs
