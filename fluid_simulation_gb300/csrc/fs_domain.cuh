// Launch domains: the cells or the particles of one simulation, or of every
// simulation of a batch, walked by generic kernels that apply a per-item
// functor.  The single-simulation path is a batch of one with zero offsets,
// so both paths run exactly the same per-item arithmetic.
//
// Batch layout: each simulation's cells occupy [co, co + nx*ny) of the
// flattened cell arrays and its particles [po, po + np) of the flattened
// particle arrays; co and po are multiples of DOMAIN_TPB, so every block of
// DOMAIN_TPB items belongs to one simulation and blk[b] = {simulation, first
// local item of block b} describes the whole flattened range.
#pragma once

#include "fs_internal.h"

namespace fs {

template <class Op>
__global__ void __launch_bounds__(DOMAIN_TPB) k_each_cell(Seg one, const Seg* __restrict__ segs,
                                                          const int2* __restrict__ blk, Op op)
{
    Seg s;
    int64_t c;
    if (blk) {
        const int2 m = blk[blockIdx.x];
        s = segs[m.x];
        c = (int64_t)m.y + threadIdx.x;
    } else {
        s = one;
        c = (int64_t)blockIdx.x * DOMAIN_TPB + threadIdx.x;
    }
    if (c >= (int64_t)s.g.nx * s.g.ny) return;
    op(s, c, (int)(c % s.g.nx), (int)(c / s.g.nx));
}

template <class Op>
__global__ void __launch_bounds__(DOMAIN_TPB) k_each_particle(Seg one, const Seg* __restrict__ segs,
                                                              const int2* __restrict__ blk, Op op)
{
    Seg s;
    int64_t k;
    if (blk) {
        const int2 m = blk[blockIdx.x];
        s = segs[m.x];
        k = (int64_t)m.y + threadIdx.x;
    } else {
        s = one;
        k = (int64_t)blockIdx.x * DOMAIN_TPB + threadIdx.x;
    }
    if (k >= s.np) return;
    op(s, k);
}

inline unsigned domain_blocks(int64_t n) { return (unsigned)((n + DOMAIN_TPB - 1) / DOMAIN_TPB); }

// op(seg, local cell c, i, j) for every cell of the domain.
template <class Op>
void each_cell(const Launch& L, const Domain& d, const Op& op)
{
    const unsigned nb = d.segs ? d.ncblk : domain_blocks((int64_t)d.one.g.nx * d.one.g.ny);
    if (nb == 0) return;
    k_each_cell<Op><<<nb, DOMAIN_TPB, 0, L.stream>>>(d.one, d.segs, d.segs ? d.cblk : nullptr, op);
    L.count();
}

// op(seg, local particle k) for every particle of the domain.
template <class Op>
void each_particle(const Launch& L, const Domain& d, const Op& op)
{
    const unsigned nb = d.segs ? d.npblk : domain_blocks(d.one.np);
    if (nb == 0) return;
    k_each_particle<Op><<<nb, DOMAIN_TPB, 0, L.stream>>>(d.one, d.segs, d.segs ? d.pblk : nullptr, op);
    L.count();
}

}  // namespace fs
