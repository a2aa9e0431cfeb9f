// Order-preserving bilinear splat: the GPU form of a sequential loop of
// Grid::addToValueInterpolated calls (include/Grid.h:152-184), as used by
// FluidSolver::transferVelocityToGridSpread (src/FluidSolver.cpp:887-897) and
// FluidSolver::advectVelocitySemiLagrangian (src/FluidSolver.cpp:721-771).
//
// Float sums depend on their order, so instead of float atomics the items are
// stably sorted by the base cell of their splat footprint (LSD radix sort,
// 8-bit digits) and every grid node gathers the items of the (up to) four
// base cells that can reach it, merging the four item lists by item index.
// Each node thus adds exactly the same float terms in exactly the same order
// as the reference's sequential loop, and the result is bit-identical.
#include "fs_domain.cuh"

namespace fs {
namespace {

constexpr int RT = 256;            // radix threads per tile
constexpr int RW = RT / 32;        // warps per tile
constexpr int R_PER_WARP = 512;    // items per warp
constexpr int RTILE = RW * R_PER_WARP;  // 4096 items per tile

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Key of each item: the flattened index (co + local cell) of the base cell of
// its footprint, or d.cells for invalid items and for the padding between
// simulations.  Item k of the flattened range belongs to block k / DOMAIN_TPB.
__global__ void __launch_bounds__(DOMAIN_TPB) k_splat_keys(Seg one, const Seg* __restrict__ segs,
                                                           const int2* __restrict__ blk, bool cells, bool pool,
                                                           int64_t n, uint32_t invalid, const float* __restrict__ x,
                                                           const float* __restrict__ y,
                                                           const uint8_t* __restrict__ valid,
                                                           uint32_t* __restrict__ keys, int32_t* __restrict__ vals,
                                                           int32_t* __restrict__ bin_count)
{
    const int64_t k = (int64_t)blockIdx.x * DOMAIN_TPB + threadIdx.x;
    if (k >= n) return;
    Seg s;
    int64_t local;
    if (blk) {
        const int2 m = blk[blockIdx.x];
        s = segs[m.x];
        local = (int64_t)m.y + threadIdx.x;
    } else {
        s = one;
        local = k;
    }
    const int64_t count = cells ? (int64_t)s.g.nx * s.g.ny : s.np;
    uint32_t key = invalid;
    if (local < count && (!valid || valid[k])) {
        const Splat sp = splat(s.g, pool ? s.g.pdx : s.g.dx, pool ? s.g.pdy : s.g.dy, x[k], y[k], 0.0f);
        key = (uint32_t)(s.co + sp.i + (int64_t)sp.j * s.g.nx);
    }
    keys[k] = key;
    vals[k] = (int32_t)k;
    atomicAdd(&bin_count[key], 1);
}

// Per-tile digit histogram, stored digit-major: hist[d * ntiles + tile].
__global__ void __launch_bounds__(RT) k_radix_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                                                  int ntiles, int32_t* __restrict__ hist)
{
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RTILE;
    for (int k = threadIdx.x; k < RTILE; k += RT) {
        const int64_t i = base + k;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: each warp owns 512 consecutive items of the tile and walks
// them 32 at a time; ranks among equal digits come from __match_any_sync.
__global__ void __launch_bounds__(RT) k_radix_scatter(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                                                     uint32_t* __restrict__ kout, int32_t* __restrict__ vout, int64_t n,
                                                     int shift, int ntiles, const int32_t* __restrict__ hist_off)
{
    __shared__ int cnt[RW][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < RW * 256; k += RT) (&cnt[0][0])[k] = 0;
    __syncthreads();
    const int64_t seg = (int64_t)blockIdx.x * RTILE + (int64_t)warp * R_PER_WARP;
    const unsigned lt = lanemask_lt();
    // 1. per-warp digit counts
    for (int r = 0; r < R_PER_WARP; r += 32) {
        const int64_t i = seg + r + lane;
        const bool ok = i < n;
        const unsigned d = ok ? ((kin[i] >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (ok && (peers & lt) == 0) cnt[warp][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // 2. exclusive prefix over warps, offset by the tile's global digit offset
    {
        const int d = threadIdx.x;
        int run = hist_off[(int64_t)d * ntiles + blockIdx.x];
        for (int w = 0; w < RW; ++w) {
            const int c = cnt[w][d];
            cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    // 3. scatter in item order
    for (int r = 0; r < R_PER_WARP; r += 32) {
        const int64_t i = seg + r + lane;
        const bool ok = i < n;
        const uint32_t key = ok ? kin[i] : 0u;
        const unsigned d = ok ? ((key >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        int dest = 0;
        if (ok) dest = cnt[warp][d] + __popc(peers & lt);
        __syncwarp();
        if (ok) {
            kout[dest] = key;
            vout[dest] = vin[i];
            if ((peers & lt) == 0) cnt[warp][d] += __popc(peers);
        }
        __syncwarp();
    }
}

// Each node (a, b) merges the item lists of base cells (a-1..a) x (b-1..b) by
// item index and adds the corners of each item's footprint that land on it.
struct SplatGather
{
    bool pool;
    const float *x, *y;
    int channels;
    const float *val0, *val1;
    const int32_t* bin_start;  // flattened cells + 2
    const int32_t* sorted;
    float *out0, *out1;
    __device__ void operator()(const Seg& s, int64_t c, int a, int b) const
    {
        const Geom& g = s.g;
        const float gdx = pool ? g.pdx : g.dx, gdy = pool ? g.pdy : g.dy;
        int cur[4], end[4];
        int nb = 0;
#pragma unroll
        for (int dj = -1; dj <= 0; ++dj)
#pragma unroll
            for (int di = -1; di <= 0; ++di) {
                const int ii = a + di, jj = b + dj;
                if (ii >= 0 && jj >= 0) {
                    const int64_t cell = s.co + (int64_t)ii + (int64_t)jj * g.nx;
                    cur[nb] = bin_start[cell];
                    end[nb] = bin_start[cell + 1];
                    ++nb;
                }
            }
        float acc0 = 0.0f, acc1 = 0.0f;
        int head[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) head[q] = (q < nb && cur[q] < end[q]) ? sorted[cur[q]] : INT32_MAX;
        for (;;) {
            int best = INT32_MAX, bq = -1;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (head[q] < best) {
                    best = head[q];
                    bq = q;
                }
            if (bq < 0) break;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (q == bq) {
                    ++cur[q];
                    head[q] = cur[q] < end[q] ? sorted[cur[q]] : INT32_MAX;
                }
            const float xi = x[best], yi = y[best];
            const Splat s0 = splat(g, gdx, gdy, xi, yi, val0 ? val0[best] : 1.0f);
            acc0 = splat_accumulate(acc0, s0, a, b);
            if (channels > 1) {
                const Splat s1 = splat(g, gdx, gdy, xi, yi, val1 ? val1[best] : 1.0f);
                acc1 = splat_accumulate(acc1, s1, a, b);
            }
        }
        out0[s.co + c] = acc0;
        if (channels > 1) out1[s.co + c] = acc1;
    }
};

int key_bits(uint32_t max_key)
{
    int b = 1;
    while (b < 32 && (max_key >> b) != 0u) ++b;
    return b;
}

}  // namespace

size_t splat_hist_ints(int64_t n_items)
{
    const int64_t ntiles = (n_items + RTILE - 1) / RTILE;
    return (size_t)(256 * (ntiles > 0 ? ntiles : 1)) + 1;
}

void ordered_splat(const Launch& L, const Domain& d, bool items_are_cells, bool pool_deltas, const float* x,
                   const float* y, const uint8_t* valid, int channels, const float* const* values, float* const* out,
                   SplatWork& w)
{
    const int64_t ncell = d.cells;
    const int64_t n = items_are_cells ? d.cells : d.parts;
    // bin counts over ncell + 1 bins (the last one collects invalid items)
    cudaMemsetAsync(w.hist_scan, 0, sizeof(int32_t) * (size_t)(ncell + 2), L.stream);
    int32_t* bin_count = w.hist_scan;
    if (n > 0) {
        const int2* blk = d.segs ? (items_are_cells ? d.cblk : d.pblk) : nullptr;
        k_splat_keys<<<domain_blocks(n), DOMAIN_TPB, 0, L.stream>>>(d.one, d.segs, blk, items_are_cells, pool_deltas,
                                                                     n, (uint32_t)ncell, x, y, valid, w.keys_a,
                                                                     w.vals_a, bin_count);
        L.count();
    }
    scan_exclusive_i32(L, bin_count, w.bin_start, ncell + 1, w.scan_tmp);
    // stable LSD radix sort of (key, item)
    uint32_t *kin = w.keys_a, *kout = w.keys_b;
    int32_t *vin = w.vals_a, *vout = w.vals_b;
    if (n > 0) {
        const int ntiles = (int)((n + RTILE - 1) / RTILE);
        const int bits = key_bits((uint32_t)ncell);
        for (int shift = 0; shift < bits; shift += 8) {
            k_radix_hist<<<ntiles, RT, 0, L.stream>>>(kin, n, shift, ntiles, w.hist);
            scan_exclusive_i32(L, w.hist, w.hist_scan, (int64_t)256 * ntiles, w.scan_tmp);
            k_radix_scatter<<<ntiles, RT, 0, L.stream>>>(kin, vin, kout, vout, n, shift, ntiles, w.hist_scan);
            L.count(2);
            uint32_t* tk = kin;
            kin = kout;
            kout = tk;
            int32_t* tv = vin;
            vin = vout;
            vout = tv;
        }
    }
    each_cell(L, d,
              SplatGather{pool_deltas, x, y, channels, values[0], channels > 1 ? values[1] : nullptr, w.bin_start, vin,
                          out[0], channels > 1 ? out[1] : nullptr});
}

}  // namespace fs
