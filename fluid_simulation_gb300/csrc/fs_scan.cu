// Exclusive prefix sums (three passes: tile reduce, scan of tile sums, apply)
// and the fluid-cell indexing built on them.
#include "fs_internal.h"

namespace fs {
namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
static_assert(SCAN_TILE == SCAN_TILE_ITEMS, "scan_tmp_ints sizes the tiles of this file");

__device__ __forceinline__ int warp_inclusive(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one int per thread over the block; returns the block total in *total.
__device__ __forceinline__ int block_exclusive(int v, int* total)
{
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int inc = warp_inclusive(v);
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        int t = lane < nw ? warp_tot[lane] : 0;
        t = warp_inclusive(t);
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int warp_excl = warp == 0 ? 0 : warp_tot[warp - 1];
    *total = warp_tot[31];
    __syncthreads();
    return warp_excl + inc - v;
}

struct LoadI32
{
    const int32_t* p;
    __device__ int operator()(int64_t i) const { return p[i]; }
};
struct StoreI32
{
    int32_t* out;
    __device__ void operator()(int64_t i, int excl, int) const { out[i] = excl; }
};
struct LoadLiquid
{
    const uint8_t* lab;
    __device__ int operator()(int64_t i) const { return lab[i] == LIQUID ? 1 : 0; }
};
struct StoreFluidIndex
{
    int32_t* fidx;
    int32_t* cell_of;
    __device__ void operator()(int64_t i, int excl, int v) const
    {
        fidx[i] = v ? excl : -1;
        if (v) cell_of[excl] = (int32_t)i;
    }
};

template <class Load>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(Load ld, int64_t n, int32_t* tile_sums)
{
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += ld(base + k);
    int total;
    (void)block_exclusive(s, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block: exclusive scan of nt tile sums in place, SCAN_TILE sums per
// round with a running carry; grand total to *total.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int32_t* tile_sums, int nt, int32_t* total)
{
    int carry = 0;
    for (int round = 0; round < nt; round += SCAN_TILE) {
        const int base = round + threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[k] = base + k < nt ? tile_sums[base + k] : 0;
            s += v[k];
        }
        int tot;
        int run = block_exclusive(s, &tot) + carry;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (base + k < nt) tile_sums[base + k] = run;
            run += v[k];
        }
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <class Load, class Store>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(Load ld, Store st, int64_t n, const int32_t* tile_off)
{
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? ld(base + k) : 0;
        s += v[k];
    }
    int tot;
    int run = block_exclusive(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) st(base + k, run, v[k]);
        run += v[k];
    }
}

template <class Load, class Store>
void scan_generic(const Launch& L, Load ld, Store st, int64_t n, int32_t* tmp, int32_t* total)
{
    const int64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nt == 0) {
        cudaMemsetAsync(total, 0, sizeof(int32_t), L.stream);
        return;
    }
    k_scan_reduce<<<(unsigned)nt, SCAN_THREADS, 0, L.stream>>>(ld, n, tmp);
    k_scan_tiles<<<1, SCAN_THREADS, 0, L.stream>>>(tmp, (int)nt, total);
    k_scan_apply<<<(unsigned)nt, SCAN_THREADS, 0, L.stream>>>(ld, st, n, tmp);
    L.count(3);
}

// Batched fluid indexing, pass 1: LIQUID cells of each cell block.
__global__ void __launch_bounds__(DOMAIN_TPB) k_block_liquid(const Seg* __restrict__ segs, const int2* __restrict__ blk,
                                                             const uint8_t* __restrict__ lab, int32_t* __restrict__ cnt)
{
    const int2 m = blk[blockIdx.x];
    const Seg& s = segs[m.x];
    const int64_t c = (int64_t)m.y + threadIdx.x;
    const int v = (c < (int64_t)s.g.nx * s.g.ny && lab[s.co + c] == LIQUID) ? 1 : 0;
    const int t = __syncthreads_count(v);
    if (threadIdx.x == 0) cnt[blockIdx.x] = t;
}

// Pass 3: local fluid index = (global offset of the block) - (global offset of
// the simulation's first block) + rank within the block.
__global__ void __launch_bounds__(DOMAIN_TPB) k_block_fluid_index(const Seg* __restrict__ segs,
                                                                  const int2* __restrict__ blk,
                                                                  const uint8_t* __restrict__ lab,
                                                                  const int32_t* __restrict__ off,
                                                                  int32_t* __restrict__ fidx,
                                                                  int32_t* __restrict__ cell_of,
                                                                  int32_t* __restrict__ nfluid)
{
    const int2 m = blk[blockIdx.x];
    const Seg& s = segs[m.x];
    const int64_t c = (int64_t)m.y + threadIdx.x;
    const bool in = c < (int64_t)s.g.nx * s.g.ny;
    const int v = (in && lab[s.co + c] == LIQUID) ? 1 : 0;
    int total;
    const int excl = block_exclusive(v, &total);
    const int base = off[blockIdx.x] - off[s.cb0];
    if (in) {
        fidx[s.co + c] = v ? base + excl : -1;
        if (v) cell_of[s.co + base + excl] = (int32_t)c;
    }
    if (threadIdx.x == 0 && (int)blockIdx.x == s.cb0 + s.ncb - 1) nfluid[s.sim] = off[s.cb0 + s.ncb] - off[s.cb0];
}

}  // namespace

void scan_exclusive_i32(const Launch& L, const int32_t* in, int32_t* out, int64_t n, int32_t* tmp)
{
    scan_generic(L, LoadI32{in}, StoreI32{out}, n, tmp, out + n);
}

void fluid_index(const Launch& L, const uint8_t* labels, int64_t n, int32_t* fidx, int32_t* cell_of,
                 int32_t* nfluid, int32_t* tmp)
{
    scan_generic(L, LoadLiquid{labels}, StoreFluidIndex{fidx, cell_of}, n, tmp, nfluid);
}

}  // namespace fs

namespace fs {

size_t fluid_index_batch_tmp_ints(const Domain& d) { return 2 * ((size_t)d.ncblk + 1) + scan_tmp_ints((int64_t)d.ncblk + 1); }

void fluid_index_batch(const Launch& L, const Domain& d, const uint8_t* labels, int32_t* fidx, int32_t* cell_of,
                       int32_t* nfluid, int32_t* tmp)
{
    if (!d.segs) {
        fluid_index(L, labels, d.cells, fidx, cell_of, nfluid, tmp);
        return;
    }
    if (d.ncblk == 0) return;
    int32_t* cnt = tmp;
    int32_t* off = tmp + d.ncblk + 1;
    int32_t* stmp = off + d.ncblk + 1;
    k_block_liquid<<<d.ncblk, DOMAIN_TPB, 0, L.stream>>>(d.segs, d.cblk, labels, cnt);
    L.count();
    scan_exclusive_i32(L, cnt, off, d.ncblk, stmp);
    k_block_fluid_index<<<d.ncblk, DOMAIN_TPB, 0, L.stream>>>(d.segs, d.cblk, labels, off, fidx, cell_of, nfluid);
    L.count();
}

}  // namespace fs
