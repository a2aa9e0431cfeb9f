// Shared device helpers for the fsgpu kernels.
//
// Bit-exactness with the reference rests on three rules applied everywhere:
//   1. every float product, quotient and sum is rounded on its own, in the
//      reference's evaluation order (explicit __f*_rn intrinsics, and the
//      whole library is built with -fmad=false);
//   2. expressions the reference writes with double literals on float
//      operands (`y - _DELTA_Y * 0.5`, `(j + 0.5) * dy`, `dx / 2.5`) are single
//      operations on float operands, whose double-then-float rounding equals
//      the float rounding (53 >= 2*24+2), so they are evaluated in float;
//   3. float -> int conversions truncate toward zero like the C++ casts, and
//      CLAMP goes through float (include/MathDefinitions.h:16-19).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fsgpu.h"

namespace fs {

constexpr uint8_t LIQUID = FS_LIQUID;
constexpr uint8_t AIR = FS_AIR;
constexpr uint8_t SOLID = FS_SOLID;

// Device status word bits (fs_handle::d_status).
constexpr unsigned ST_TIMEOUT = 1u;
constexpr unsigned ST_INTERNAL = 2u;
constexpr unsigned ST_TOO_LARGE = 4u;

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Double-single pairs: a float*float product exactly as an unevaluated sum
// hi + lo (fmul, then fmaf for its rounding error), and pairs added with a
// TwoSum of the high parts, the error and both low parts then added in float
// (not renormalised).  About 48 bits in float arithmetic alone.
struct ds
{
    float hi, lo;
};
__device__ __forceinline__ ds ds_prod(float a, float b)
{
    const float p = fmul(a, b);
    return ds{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ds ds_add(ds a, ds b)
{
    const float s = fadd(a.hi, b.hi);
    const float v = fsub(s, a.hi);
    float e = fadd(fsub(a.hi, fsub(s, v)), fsub(b.hi, v));
    e = fadd(e, a.lo);
    e = fadd(e, b.lo);
    return ds{s, e};
}

// C++ (int)x for float x: truncation toward zero.
__device__ __forceinline__ int trunc_i(float x) { return __float2int_rz(x); }

// CLAMP(MyFloat d, MyFloat min, MyFloat max) applied to ints, then back to int.
__device__ __forceinline__ int clampi(int d, int lo, int hi)
{
    const float fd = (float)d, flo = (float)lo, fhi = (float)hi;
    const float t = fd < flo ? flo : fd;
    return (int)(t > fhi ? fhi : t);
}
__device__ __forceinline__ float clampf(float d, float lo, float hi)
{
    const float t = d < lo ? lo : d;
    return t > hi ? hi : t;
}

// Geometry and constants of one simulation, passed by value to kernels.
struct Geom
{
    int nx, ny;
    float dx, dy;      // MacGrid deltas (length / size)
    float lx, ly;      // GridInterface::lengthX/Y: size * delta
    float pdx, pdy;    // the solver pool's deltas (pdy == dx in the reference)
};

__device__ __forceinline__ uint8_t cell_type(const uint8_t* __restrict__ lab, const Geom& g, int i, int j)
{
    i = clampi(i, 0, g.nx - 1);
    j = clampi(j, 0, g.ny - 1);
    return lab[i + j * g.nx];
}

// Row of the pressure matrix for fluid cell c = (i, j) (src/FluidSolver.cpp:369-410):
// flags bit 0 / bit 1 = liquid left / right neighbour (fluid indices k-1 / k+1
// in the j-major order), bits 2-4 = number of non-solid neighbours n (the
// diagonal is -n / dx^2); down / up = fluid indices of the liquid cells below /
// above, or -1.  A LIQUID cell on the grid border (impossible after
// classification) would make the reference read outside the grid; such
// neighbours are skipped.
__device__ __forceinline__ void matrix_row(const uint8_t* __restrict__ lab, const Geom& g,
                                           const int32_t* __restrict__ fidx, int64_t c, int i, int j, uint8_t& flags,
                                           int32_t& down, int32_t& up)
{
    int nns = 0;
    uint8_t fl = 0;
    down = up = -1;
    uint8_t ct = cell_type(lab, g, i - 1, j);
    if (ct != SOLID) {
        if (ct == LIQUID && i > 0) fl |= 1;
        ++nns;
    }
    ct = cell_type(lab, g, i + 1, j);
    if (ct != SOLID) {
        if (ct == LIQUID && i < g.nx - 1) fl |= 2;
        ++nns;
    }
    ct = cell_type(lab, g, i, j - 1);
    if (ct != SOLID) {
        if (ct == LIQUID && j > 0) down = fidx[c - g.nx];
        ++nns;
    }
    ct = cell_type(lab, g, i, j + 1);
    if (ct != SOLID) {
        if (ct == LIQUID && j < g.ny - 1) up = fidx[c + g.nx];
        ++nns;
    }
    flags = (uint8_t)(fl | (nns << 2));
}

// Grid::valueInterpolated (include/Grid.h:117-144); +1 neighbour formed after clamping.
__device__ __forceinline__ float value_interp(const float* __restrict__ grid, const Geom& g, float gdx, float gdy,
                                              float x, float y)
{
    const float xs = fdiv(x, gdx);
    const float ys = fdiv(y, gdy);
    int i = trunc_i(xs);
    int j = trunc_i(ys);
    const float i_frac = fsub(xs, (float)i);
    const float j_frac = fsub(ys, (float)j);
    i = clampi(i, 0, g.nx - 1);
    j = clampi(j, 0, g.ny - 1);
    const int i1 = clampi(i + 1, 0, g.nx - 1);
    const int j1 = clampi(j + 1, 0, g.ny - 1);
    const float v00 = grid[i + j * g.nx];
    const float v10 = grid[i1 + j * g.nx];
    const float v01 = grid[i + j1 * g.nx];
    const float v11 = grid[i1 + j1 * g.nx];
    const float omi = fsub(1.0f, i_frac);
    const float value_0 = fadd(fmul(omi, v00), fmul(i_frac, v10));
    const float value_1 = fadd(fmul(omi, v01), fmul(i_frac, v11));
    return fadd(fmul(fsub(1.0f, j_frac), value_0), fmul(j_frac, value_1));
}

// MacGrid::velXInterpolated / velYInterpolated (include/MacGrid.h:66-79).
__device__ __forceinline__ float vel_x_interp(const float* __restrict__ u, const Geom& g, float x, float y)
{
    return value_interp(u, g, g.dx, g.dy, x, fsub(y, fmul(g.dy, 0.5f)));
}
__device__ __forceinline__ float vel_y_interp(const float* __restrict__ v, const Geom& g, float x, float y)
{
    return value_interp(v, g, g.dx, g.dy, fsub(x, fmul(g.dx, 0.5f)), y);
}

// Footprint of Grid::addToValueInterpolated (include/Grid.h:152-184): the
// clamped corners (i, j), (i1, j), (i, j1), (i1, j1) and their weights
// w00..w11 applied to `value`.  The +1 neighbour is formed before clamping.
struct Splat
{
    int i, j, i1, j1;
    float v00, v10, v01, v11;
};

// The footprint from the scaled position (xs, ys) = (x / gdx, y / gdy).
__device__ __forceinline__ Splat splat_scaled(const Geom& g, float xs, float ys, float value)
{
    Splat s;
    int i = trunc_i(xs);
    int j = trunc_i(ys);
    const int i1 = i + 1;
    const int j1 = j + 1;
    const float i_frac = fsub(xs, (float)i);
    const float j_frac = fsub(ys, (float)j);
    s.i = clampi(i, 0, g.nx - 1);
    s.j = clampi(j, 0, g.ny - 1);
    s.i1 = clampi(i1, 0, g.nx - 1);
    s.j1 = clampi(j1, 0, g.ny - 1);
    const float value_0 = fmul(fsub(1.0f, j_frac), value);
    const float value_1 = fmul(j_frac, value);
    const float omi = fsub(1.0f, i_frac);
    s.v00 = fmul(omi, value_0);
    s.v10 = fmul(i_frac, value_0);
    s.v01 = fmul(omi, value_1);
    s.v11 = fmul(i_frac, value_1);
    return s;
}

__device__ __forceinline__ Splat splat(const Geom& g, float gdx, float gdy, float x, float y, float value)
{
    return splat_scaled(g, fdiv(x, gdx), fdiv(y, gdy), value);
}

// Adds, in the reference's corner order 00, 10, 01, 11, the corners of s that
// land on node (a, b) to acc.
__device__ __forceinline__ float splat_accumulate(float acc, const Splat& s, int a, int b)
{
    if (s.i == a && s.j == b) acc = fadd(acc, s.v00);
    if (s.i1 == a && s.j == b) acc = fadd(acc, s.v10);
    if (s.i == a && s.j1 == b) acc = fadd(acc, s.v01);
    if (s.i1 == a && s.j1 == b) acc = fadd(acc, s.v11);
    return acc;
}

// RK3::step (include/OdeSolver.h:102-113) on FluidSolver's Vec2
// (include/FluidSolver.h:120-141) through the front velocity grids, as used by
// FluidSolver::getAdvectedPosition (src/FluidSolver.cpp:793-814).
__device__ __forceinline__ void advected_position(const float* __restrict__ u, const float* __restrict__ v,
                                                  const Geom& g, float x, float y, float h, float* ox, float* oy)
{
    const float k1x = vel_x_interp(u, g, x, y);
    const float k1y = vel_y_interp(v, g, x, y);
    float ax = fadd(x, fdiv(fmul(fmul(k1x, h), 1.0f), 2.0f));
    float ay = fadd(y, fdiv(fmul(fmul(k1y, h), 1.0f), 2.0f));
    const float k2x = vel_x_interp(u, g, ax, ay);
    const float k2y = vel_y_interp(v, g, ax, ay);
    ax = fadd(x, fdiv(fmul(fmul(k2x, h), 3.0f), 4.0f));
    ay = fadd(y, fdiv(fmul(fmul(k2y, h), 3.0f), 4.0f));
    const float k3x = vel_x_interp(u, g, ax, ay);
    const float k3y = vel_y_interp(v, g, ax, ay);
    float sx = fadd(fadd(fmul(k1x, 2.0f), fmul(k2x, 3.0f)), fmul(k3x, 4.0f));
    float sy = fadd(fadd(fmul(k1y, 2.0f), fmul(k2y, 3.0f)), fmul(k3y, 4.0f));
    sx = fdiv(fmul(fmul(sx, h), 1.0f), 9.0f);
    sy = fdiv(fmul(fmul(sy, h), 1.0f), 9.0f);
    *ox = fadd(x, sx);
    *oy = fadd(y, sy);
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Whether an arrival counter has reached target.  Both advance by the grid's
// arrivals per barrier and wrap modulo 2^32 together (after about 14 million
// CG iterations of a 152-CTA grid), and a waiting CTA's counter is never more
// than a few hundred arrivals from its target, so their signed difference
// decides.
__device__ __forceinline__ bool count_reached(unsigned count, unsigned target) { return (int)(count - target) >= 0; }

}  // namespace fs
