// Order-preserving bilinear splat: the GPU form of a sequential loop of
// Grid::addToValueInterpolated calls (include/Grid.h:152-184), as used by
// FluidSolver::transferVelocityToGridSpread (src/FluidSolver.cpp:887-897) and
// FluidSolver::advectVelocitySemiLagrangian (src/FluidSolver.cpp:721-771).
//
// Float sums depend on their order, so instead of float atomics the items are
// binned by the base cell of their splat footprint (a counting sort: bin
// counts, their prefix sum, a scatter with per-bin atomic cursors, then each
// bin sorted by item index, which makes the order the items' own) and every
// grid node gathers the items of the (up to) four base cells that can reach
// it, merging the four item lists by item index.  Each node thus adds exactly
// the same float terms in exactly the same order as the reference's
// sequential loop, and the result is bit-identical.  The key pass keeps each
// item's scaled position (x / dx, y / dy), so that the four nodes of a
// footprint do not repeat its two divisions.
#include "fs_domain.cuh"

namespace fs {
namespace {

// Key of each item: the flattened index (co + local cell) of the base cell of
// its footprint, or d.cells for invalid items and for the padding between
// simulations.  Item k of the flattened range belongs to block k / DOMAIN_TPB.
__global__ void __launch_bounds__(DOMAIN_TPB) k_splat_keys(Seg one, const Seg* __restrict__ segs,
                                                           const int2* __restrict__ blk, bool cells, bool pool,
                                                           int64_t n, uint32_t invalid, const float* __restrict__ x,
                                                           const float* __restrict__ y,
                                                           const uint8_t* __restrict__ valid,
                                                           uint32_t* __restrict__ keys, int32_t* __restrict__ bin_count,
                                                           float* __restrict__ xs, float* __restrict__ ys)
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
        const float sx = fdiv(x[k], pool ? s.g.pdx : s.g.dx), sy = fdiv(y[k], pool ? s.g.pdy : s.g.dy);
        const Splat sp = splat_scaled(s.g, sx, sy, 0.0f);
        key = (uint32_t)(s.co + sp.i + (int64_t)sp.j * s.g.nx);
        xs[k] = sx;
        ys[k] = sy;
    }
    keys[k] = key;
    atomicAdd(&bin_count[key], 1);
}

__global__ void k_bin_count(int64_t n, uint32_t invalid, const uint32_t* __restrict__ keys, int32_t* __restrict__ count)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = keys[k];
    if (key != invalid) atomicAdd(&count[key], 1);
}

// Item k goes to position bin_start[key] + (its rank among the bin's items
// in arrival order, counted down on the bin's count).
__global__ void k_bin_scatter(int64_t n, uint32_t invalid, const uint32_t* __restrict__ keys,
                              const int32_t* __restrict__ bin_start, int32_t* __restrict__ count,
                              int32_t* __restrict__ sorted)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = keys[k];
    if (key == invalid) return;  // the bin of invalid items is never gathered
    const int pos = bin_start[key] + atomicSub(&count[key], 1) - 1;
    sorted[pos] = (int32_t)k;
}

// Each bin's items in increasing item index (insertion sort; bins hold a few
// items).
__global__ void k_bin_sort(int64_t nbins, const int32_t* __restrict__ bin_start, int32_t* __restrict__ sorted)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nbins) return;
    const int b0 = bin_start[c], b1 = bin_start[c + 1];
    if (b1 - b0 < 2) return;
    constexpr int LOCAL = 16;
    if (b1 - b0 <= LOCAL) {
        int v[LOCAL];
        const int m = b1 - b0;
        for (int i = 0; i < m; ++i) v[i] = sorted[b0 + i];
        for (int i = 1; i < m; ++i) {
            const int t = v[i];
            int j = i - 1;
            while (j >= 0 && v[j] > t) {
                v[j + 1] = v[j];
                --j;
            }
            v[j + 1] = t;
        }
        for (int i = 0; i < m; ++i) sorted[b0 + i] = v[i];
    } else {
        for (int i = b0 + 1; i < b1; ++i) {
            const int t = sorted[i];
            int j = i - 1;
            while (j >= b0 && sorted[j] > t) {
                sorted[j + 1] = sorted[j];
                --j;
            }
            sorted[j + 1] = t;
        }
    }
}

// Each node (a, b) merges the item lists of base cells (a-1..a) x (b-1..b) by
// item index and adds the corners of each item's footprint that land on it.
struct SplatGather
{
    const float *xs, *ys;  // scaled positions
    int channels;
    const float *val0, *val1;
    const int32_t* bin_start;  // flattened cells + 2
    const int32_t* sorted;
    float *out0, *out1;
    __device__ void operator()(const Seg& s, int64_t c, int a, int b) const
    {
        const Geom& g = s.g;
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
            const float xi = xs[best], yi = ys[best];
            const Splat s0 = splat_scaled(g, xi, yi, val0 ? val0[best] : 1.0f);
            acc0 = splat_accumulate(acc0, s0, a, b);
            if (channels > 1) {
                const Splat s1 = splat_scaled(g, xi, yi, val1 ? val1[best] : 1.0f);
                acc1 = splat_accumulate(acc1, s1, a, b);
            }
        }
        out0[s.co + c] = acc0;
        if (channels > 1) out1[s.co + c] = acc1;
    }
};

}  // namespace

void group_by_key(const Launch& L, int64_t n, const uint32_t* keys, int64_t nbins, int32_t* bin_count,
                  int32_t* bin_start, int32_t* scan_tmp, int32_t* sorted)
{
    cudaMemsetAsync(bin_count, 0, sizeof(int32_t) * (size_t)(nbins + 1), L.stream);
    if (n > 0) {
        k_bin_count<<<domain_blocks(n), DOMAIN_TPB, 0, L.stream>>>(n, (uint32_t)nbins, keys, bin_count);
        L.count();
    }
    scan_exclusive_i32(L, bin_count, bin_start, nbins, scan_tmp);
    if (n > 0) {
        k_bin_scatter<<<domain_blocks(n), DOMAIN_TPB, 0, L.stream>>>(n, (uint32_t)nbins, keys, bin_start, bin_count,
                                                                      sorted);
        k_bin_sort<<<domain_blocks(nbins), DOMAIN_TPB, 0, L.stream>>>(nbins, bin_start, sorted);
        L.count(2);
    }
}

cudaError_t splat_alloc(SplatWork& w, int64_t items, int64_t cells)
{
    splat_free(w);
    const size_t bins = (size_t)cells + 2;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 4);
    };
    A((void**)&w.keys, 4 * (size_t)items);
    A((void**)&w.sorted, 4 * (size_t)items);
    A((void**)&w.bin_count, 4 * bins);
    A((void**)&w.bin_start, 4 * bins);
    A((void**)&w.xs, 4 * (size_t)items);
    A((void**)&w.ys, 4 * (size_t)items);
    A((void**)&w.scan_tmp, 4 * scan_tmp_ints((int64_t)bins));
    if (e != cudaSuccess) {
        splat_free(w);
        return e;
    }
    w.cap_items = items;
    w.cells = cells;
    return cudaSuccess;
}

void splat_free(SplatWork& w)
{
    for (void* p : {(void*)w.keys, (void*)w.sorted, (void*)w.bin_count, (void*)w.bin_start, (void*)w.scan_tmp,
                    (void*)w.xs, (void*)w.ys})
        cudaFree(p);
    w = SplatWork{};
}

void ordered_splat(const Launch& L, const Domain& d, bool items_are_cells, bool pool_deltas, const float* x,
                   const float* y, const uint8_t* valid, int channels, const float* const* values, float* const* out,
                   SplatWork& w)
{
    const int64_t ncell = d.cells;
    const int64_t n = items_are_cells ? d.cells : d.parts;
    // bin counts over ncell + 1 bins (the last one collects invalid items)
    cudaMemsetAsync(w.bin_count, 0, sizeof(int32_t) * (size_t)(ncell + 2), L.stream);
    if (n > 0) {
        const int2* blk = d.segs ? (items_are_cells ? d.cblk : d.pblk) : nullptr;
        k_splat_keys<<<domain_blocks(n), DOMAIN_TPB, 0, L.stream>>>(d.one, d.segs, blk, items_are_cells, pool_deltas,
                                                                     n, (uint32_t)ncell, x, y, valid, w.keys,
                                                                     w.bin_count, w.xs, w.ys);
        L.count();
    }
    scan_exclusive_i32(L, w.bin_count, w.bin_start, ncell + 1, w.scan_tmp);
    if (n > 0) {
        k_bin_scatter<<<domain_blocks(n), DOMAIN_TPB, 0, L.stream>>>(n, (uint32_t)ncell, w.keys, w.bin_start,
                                                                      w.bin_count, w.sorted);
        k_bin_sort<<<domain_blocks(ncell), DOMAIN_TPB, 0, L.stream>>>(ncell, w.bin_start, w.sorted);
        L.count(2);
    }
    each_cell(L, d,
              SplatGather{w.xs, w.ys, channels, values[0], channels > 1 ? values[1] : nullptr, w.bin_start, w.sorted,
                          out[0], channels > 1 ? out[1] : nullptr});
}

}  // namespace fs
