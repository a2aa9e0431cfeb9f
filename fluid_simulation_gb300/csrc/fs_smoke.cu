// Differentiable smoke (include/fsgpu.h, fs_smoke_*): semi-Lagrangian
// advection of a passive density and of the velocity by gathering (each grid
// sample traces back through the velocity field and samples the old field
// there), solid-wall conditions and the pressure projection, for a number of
// steps; the loss is the L2 distance of the final density to a target; the
// gradient of the loss with respect to the initial state comes from a
// hand-written adjoint with checkpoint-and-recompute.  Not in the reference,
// whose semi-Lagrangian step scatters (src/FluidSolver.cpp:709-772); the
// pieces it shares with the reference follow it:
//   * bilinear sampling: Grid::valueInterpolated (include/Grid.h:117-144) --
//     the fraction taken before the corner indices are clamped; u faces at
//     (i h, (j + 1/2) h), v faces at ((i + 1/2) h, j h) (MacGrid::vel{X,Y}
//     Interpolated, include/MacGrid.h:66-79); density at cell centres;
//   * back-trace: explicit Euler, the midpoint rule (RK2) or Ralston's RK3 as
//     in RK3::step (include/OdeSolver.h:102-113), with step -dt;
//   * projection: FluidSolver::pressureSolve's matrix (src/FluidSolver.cpp:
//     363-416) on the non-solid cells, divergence as MacGrid::divVel{X,Y}
//     (include/MacGrid.h:98-111), u -= grad p on faces between two fluid
//     cells; faces touching a solid cell carry zero velocity.
//
// The projection composed with the wall condition is symmetric (B - B D^T
// A^-1 D B with the wall mask B and the divergence D), so its adjoint is the
// same operation on the adjoint velocity.  The adjoint of advection sends
// each sample's adjoint through the transposed bilinear weights and carries
// the adjoint of the traced position back through the integrator stages.
// The transpose is a gather, so that gradients repeat to the bit: every
// contribution becomes an item keyed by the node it adds to, the counting
// sort of the ordered splat (group_by_key) groups the items by node in item
// order, and each node adds its items in that order.  Fields and advection
// run in the handle's precision (float or double); adjoints are double.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fs_internal.h"

using namespace fs;

namespace {

constexpr int TPB = 256;

template <typename T> __device__ __forceinline__ int trunc_t(T x);
template <> __device__ __forceinline__ int trunc_t<float>(float x) { return __float2int_rz(x); }
template <> __device__ __forceinline__ int trunc_t<double>(double x) { return __double2int_rz(x); }

// Corner nodes and fractions of a bilinear sample at (x, y) of a field whose
// node (i, j) sits at (i h, j h) (include/Grid.h:117-144).
template <typename T>
struct Foot
{
    int i, j, i1, j1;
    T fi, fj;
};

template <typename T>
__device__ __forceinline__ Foot<T> footprint(int nx, int ny, T h, T x, T y)
{
    const T xs = x / h, ys = y / h;
    int i = trunc_t(xs), j = trunc_t(ys);
    Foot<T> F;
    F.fi = xs - (T)i;
    F.fj = ys - (T)j;
    i = min(max(i, 0), nx - 1);
    j = min(max(j, 0), ny - 1);
    F.i = i;
    F.j = j;
    F.i1 = min(i + 1, nx - 1);
    F.j1 = min(j + 1, ny - 1);
    return F;
}

// Field values stored as S, sampled in the arithmetic A of the footprint.
template <typename S, typename A>
__device__ __forceinline__ A interp(const S* __restrict__ f, int nx, const Foot<A>& F)
{
    const A v00 = (A)f[F.i + F.j * nx], v10 = (A)f[F.i1 + F.j * nx];
    const A v01 = (A)f[F.i + F.j1 * nx], v11 = (A)f[F.i1 + F.j1 * nx];
    const A a = (A(1) - F.fi) * v00 + F.fi * v10;
    const A b = (A(1) - F.fi) * v01 + F.fi * v11;
    return (A(1) - F.fj) * a + F.fj * b;
}

// d interp / d(x, y), in double.
template <typename S, typename A>
__device__ __forceinline__ void interp_grad(const S* __restrict__ f, int nx, const Foot<A>& F, double h, double& gx,
                                            double& gy)
{
    const double v00 = f[F.i + F.j * nx], v10 = f[F.i1 + F.j * nx];
    const double v01 = f[F.i + F.j1 * nx], v11 = f[F.i1 + F.j1 * nx];
    const double fi = F.fi, fj = F.fj;
    gx = ((1.0 - fj) * (v10 - v00) + fj * (v11 - v01)) / h;
    gy = ((1.0 - fi) * (v01 - v00) + fi * (v11 - v10)) / h;
}

// Contribution items of one adjoint step: item q * n + c is contribution
// slot q of cell c; key = field * n + node (field 0 u, 1 v, 2 density), or
// 3 n for an empty slot; val = the value added there.
struct Items
{
    uint32_t* key;
    double* val;
    int64_t n;
};

// Slots of a sample's contributions: its final footprint (4 corners), then 8
// per integrator stage (4 u corners, 4 v corners).
__host__ __device__ constexpr int stage_count(int integrator)
{
    return integrator == FS_INTEGRATOR_EULER ? 1 : integrator == FS_INTEGRATOR_RK2 ? 2 : 3;
}
__host__ __device__ constexpr int sample_slots(int integrator) { return 4 + 8 * stage_count(integrator); }

// w * (the bilinear weights of F) into field `field`: the transpose of
// interp, as four items from slot q of cell c.
template <typename T>
__device__ __forceinline__ void scatter(const Items& it, int64_t c, int q, int field, int nx, const Foot<T>& F,
                                        double w)
{
    const uint32_t none = (uint32_t)(3 * it.n);
    const int64_t base = (int64_t)field * it.n;
    const double fi = F.fi, fj = F.fj;
    const int64_t node[4] = {F.i + (int64_t)F.j * nx, F.i1 + (int64_t)F.j * nx, F.i + (int64_t)F.j1 * nx,
                             F.i1 + (int64_t)F.j1 * nx};
    const double wt[4] = {(1.0 - fi) * (1.0 - fj) * w, fi * (1.0 - fj) * w, (1.0 - fi) * fj * w, fi * fj * w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int64_t item = (int64_t)(q + k) * it.n + c;
        it.key[item] = w == 0.0 ? none : (uint32_t)(base + node[k]);
        it.val[item] = wt[k];
    }
}

// Fields stored as S; back-trace positions, footprints and samples in the
// arithmetic A (S, or double for float fields traced in double).
template <typename S, typename A = S>
struct Fields
{
    const S *u, *v, *d;
    int nx, ny;
    A h;
    __device__ Foot<A> foot_u(A x, A y) const { return footprint<A>(nx, ny, h, x, y - h / A(2)); }
    __device__ Foot<A> foot_v(A x, A y) const { return footprint<A>(nx, ny, h, x - h / A(2), y); }
    __device__ Foot<A> foot_d(A x, A y) const { return footprint<A>(nx, ny, h, x - h / A(2), y - h / A(2)); }
    __device__ void vel(A x, A y, A& vx, A& vy) const
    {
        vx = interp<S, A>(u, nx, foot_u(x, y));
        vy = interp<S, A>(v, nx, foot_v(x, y));
    }
};

// Stage positions of the back-trace from (x, y) with step ht = -dt.
template <typename T>
struct Trace
{
    T x[3], y[3];  // stage positions (x[0] = the sample point)
    T kx[3], ky[3];
    T ox, oy;      // the traced position
};

template <typename S, typename T>
__device__ __forceinline__ void trace(const Fields<S, T>& F, int integrator, T ht, T x, T y, Trace<T>& tr)
{
    tr.x[0] = x;
    tr.y[0] = y;
    F.vel(x, y, tr.kx[0], tr.ky[0]);
    if (integrator == FS_INTEGRATOR_EULER) {
        tr.ox = x + ht * tr.kx[0];
        tr.oy = y + ht * tr.ky[0];
    } else if (integrator == FS_INTEGRATOR_RK2) {
        tr.x[1] = x + ht / T(2) * tr.kx[0];
        tr.y[1] = y + ht / T(2) * tr.ky[0];
        F.vel(tr.x[1], tr.y[1], tr.kx[1], tr.ky[1]);
        tr.ox = x + ht * tr.kx[1];
        tr.oy = y + ht * tr.ky[1];
    } else {
        // RK3::step (include/OdeSolver.h:102-113)
        tr.x[1] = x + tr.kx[0] * ht * T(1) / T(2);
        tr.y[1] = y + tr.ky[0] * ht * T(1) / T(2);
        F.vel(tr.x[1], tr.y[1], tr.kx[1], tr.ky[1]);
        tr.x[2] = x + tr.kx[1] * ht * T(3) / T(4);
        tr.y[2] = y + tr.ky[1] * ht * T(3) / T(4);
        F.vel(tr.x[2], tr.y[2], tr.kx[2], tr.ky[2]);
        tr.ox = x + (tr.kx[0] * T(2) + tr.kx[1] * T(3) + tr.kx[2] * T(4)) * ht * T(1) / T(9);
        tr.oy = y + (tr.ky[0] * T(2) + tr.ky[1] * T(3) + tr.ky[2] * T(4)) * ht * T(1) / T(9);
    }
}

__device__ __forceinline__ bool solid_at(const uint8_t* lab, int nx, int i, int j) { return lab[i + j * nx] == FS_SOLID; }

// Faces that touch a solid cell or the grid edge carry no velocity.
__device__ __forceinline__ bool u_open(const uint8_t* lab, int nx, int i, int j)
{
    return i > 0 && !solid_at(lab, nx, i - 1, j) && !solid_at(lab, nx, i, j);
}
__device__ __forceinline__ bool v_open(const uint8_t* lab, int nx, int i, int j)
{
    return j > 0 && !solid_at(lab, nx, i, j - 1) && !solid_at(lab, nx, i, j);
}

// One advection: every u face, v face and cell centre gathers from the old
// fields at its traced position; closed faces get 0.
template <typename S, typename T>
__global__ void k_advect(Fields<S, T> F, const uint8_t* __restrict__ lab, int integrator, T dt, S* __restrict__ un,
                         S* __restrict__ vn, S* __restrict__ dn)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)F.nx * F.ny) return;
    const int i = (int)(c % F.nx), j = (int)(c / F.nx);
    const T h = F.h, ht = -dt;
    Trace<T> tr;
    if (u_open(lab, F.nx, i, j)) {
        trace(F, integrator, ht, T(i) * h, (T(j) + T(0.5)) * h, tr);
        un[c] = (S)interp<S, T>(F.u, F.nx, F.foot_u(tr.ox, tr.oy));
    } else {
        un[c] = S(0);
    }
    if (v_open(lab, F.nx, i, j)) {
        trace(F, integrator, ht, (T(i) + T(0.5)) * h, T(j) * h, tr);
        vn[c] = (S)interp<S, T>(F.v, F.nx, F.foot_v(tr.ox, tr.oy));
    } else {
        vn[c] = S(0);
    }
    trace(F, integrator, ht, (T(i) + T(0.5)) * h, (T(j) + T(0.5)) * h, tr);
    dn[c] = (S)interp<S, T>(F.d, F.nx, F.foot_d(tr.ox, tr.oy));
}

// rhs = divergence on fluid cells (double), 0 elsewhere.
template <typename T>
__global__ void k_divergence(int nx, int ny, double h, const uint8_t* __restrict__ lab, const T* __restrict__ u,
                             const T* __restrict__ v, double* __restrict__ rhs)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)nx * ny) return;
    const int i = (int)(c % nx), j = (int)(c / nx);
    if (lab[c] != FS_LIQUID || i >= nx - 1 || j >= ny - 1) {
        rhs[c] = 0.0;
        return;
    }
    rhs[c] = ((double)u[c + 1] - (double)u[c]) / h + ((double)v[c + nx] - (double)v[c]) / h;
}

// u -= grad p on faces between two fluid cells.
template <typename T>
__global__ void k_subtract_gradient(int nx, int ny, double h, const uint8_t* __restrict__ lab,
                                    const double* __restrict__ p, T* __restrict__ u, T* __restrict__ v)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)nx * ny) return;
    const int i = (int)(c % nx), j = (int)(c / nx);
    const bool here = lab[c] == FS_LIQUID;
    if (here && i > 0 && lab[c - 1] == FS_LIQUID) u[c] = (T)((double)u[c] - (p[c] - p[c - 1]) / h);
    if (here && j > 0 && lab[c - nx] == FS_LIQUID) v[c] = (T)((double)v[c] - (p[c] - p[c - nx]) / h);
}

// The adjoint of one advection as contribution items (Items).  lu, lv, ld:
// adjoints of the advected fields (already through the projection's
// adjoint); the items add up to the adjoints of the old fields.
template <typename S, typename T>
__global__ void k_advect_adjoint(Fields<S, T> F, const uint8_t* __restrict__ lab, int integrator, T dt,
                                 const double* __restrict__ lu, const double* __restrict__ lv,
                                 const double* __restrict__ ld, Items items)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)F.nx * F.ny) return;
    const int i = (int)(c % F.nx), j = (int)(c / F.nx);
    const T h = F.h, ht = -dt;
    const double hd = (double)h, htd = (double)ht;
    const int per = sample_slots(integrator);
    for (int s = 0; s < 3; ++s) {
        const int q0 = s * per;
        double lam;
        T x0, y0;
        if (s == 0) {
            lam = u_open(lab, F.nx, i, j) ? lu[c] : 0.0;
            x0 = T(i) * h;
            y0 = (T(j) + T(0.5)) * h;
        } else if (s == 1) {
            lam = v_open(lab, F.nx, i, j) ? lv[c] : 0.0;
            x0 = (T(i) + T(0.5)) * h;
            y0 = T(j) * h;
        } else {
            lam = ld[c];
            x0 = (T(i) + T(0.5)) * h;
            y0 = (T(j) + T(0.5)) * h;
        }
        if (lam == 0.0) {
            for (int q = 0; q < per; ++q) items.key[(int64_t)(q0 + q) * items.n + c] = (uint32_t)(3 * items.n);
            continue;
        }
        Trace<T> tr;
        trace(F, integrator, ht, x0, y0, tr);
        // the sampled field at the traced position
        double gx, gy;
        if (s == 0) {
            const Foot<T> fo = F.foot_u(tr.ox, tr.oy);
            scatter(items, c, q0, 0, F.nx, fo, lam);
            interp_grad(F.u, F.nx, fo, hd, gx, gy);
        } else if (s == 1) {
            const Foot<T> fo = F.foot_v(tr.ox, tr.oy);
            scatter(items, c, q0, 1, F.nx, fo, lam);
            interp_grad(F.v, F.nx, fo, hd, gx, gy);
        } else {
            const Foot<T> fo = F.foot_d(tr.ox, tr.oy);
            scatter(items, c, q0, 2, F.nx, fo, lam);
            interp_grad(F.d, F.nx, fo, hd, gx, gy);
        }
        const double lx = lam * gx, ly = lam * gy;  // adjoint of the traced position
        // back through the stages: adjoint of the velocity sample k at stage
        // position q adds to the fields there and to q's adjoint (the t-th
        // stage visited fills slots 4 + 8 t .. 11 + 8 t of the sample)
        int t = 0;
        auto stage = [&](int q, double kxa, double kya, double& pxa, double& pya) {
            const Foot<T> fu = F.foot_u(tr.x[q], tr.y[q]);
            const Foot<T> fv = F.foot_v(tr.x[q], tr.y[q]);
            scatter(items, c, q0 + 4 + 8 * t, 0, F.nx, fu, kxa);
            scatter(items, c, q0 + 8 + 8 * t, 1, F.nx, fv, kya);
            ++t;
            double ux, uy, vx, vy;
            interp_grad(F.u, F.nx, fu, hd, ux, uy);
            interp_grad(F.v, F.nx, fv, hd, vx, vy);
            pxa = ux * kxa + vx * kya;
            pya = uy * kxa + vy * kya;
        };
        double px, py;
        if (integrator == FS_INTEGRATOR_EULER) {
            stage(0, htd * lx, htd * ly, px, py);
        } else if (integrator == FS_INTEGRATOR_RK2) {
            stage(1, htd * lx, htd * ly, px, py);              // k2 at the midpoint
            stage(0, htd / 2.0 * px, htd / 2.0 * py, px, py);  // k1
        } else {
            double k1x = 2.0 * htd / 9.0 * lx, k1y = 2.0 * htd / 9.0 * ly;
            double k2x = 3.0 * htd / 9.0 * lx, k2y = 3.0 * htd / 9.0 * ly;
            const double k3x = 4.0 * htd / 9.0 * lx, k3y = 4.0 * htd / 9.0 * ly;
            stage(2, k3x, k3y, px, py);
            k2x += 3.0 * htd / 4.0 * px;
            k2y += 3.0 * htd / 4.0 * py;
            stage(1, k2x, k2y, px, py);
            k1x += htd / 2.0 * px;
            k1y += htd / 2.0 * py;
            stage(0, k1x, k1y, px, py);
        }
    }
}

// acc[field][node] = the sum of the items grouped at bin field * n + node, in
// item order (bin_start / sorted from group_by_key).
__global__ void k_adjoint_gather(int64_t n, const int32_t* __restrict__ bin_start, const int32_t* __restrict__ sorted,
                                 const double* __restrict__ val, double* __restrict__ au, double* __restrict__ av,
                                 double* __restrict__ ad)
{
    const int64_t b = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (b >= 3 * n) return;
    double acc = 0.0;
    for (int k = bin_start[b]; k < bin_start[b + 1]; ++k) acc += val[sorted[k]];
    double* out = b < n ? au : b < 2 * n ? av : ad;
    out[b % n] = acc;
}

// Adjoint of the wall condition: closed faces pass nothing back.
__global__ void k_close_faces(int nx, int ny, const uint8_t* __restrict__ lab, double* __restrict__ u,
                              double* __restrict__ v)
{
    const int64_t c = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (c >= (int64_t)nx * ny) return;
    const int i = (int)(c % nx), j = (int)(c / nx);
    if (!u_open(lab, nx, i, j)) u[c] = 0.0;
    if (!v_open(lab, nx, i, j)) v[c] = 0.0;
}

template <typename T>
__global__ void k_to_double(int64_t n, const T* __restrict__ a, double* __restrict__ out)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k < n) out[k] = (double)a[k];
}

template <typename T>
__global__ void k_from_double(int64_t n, const double* __restrict__ a, T* __restrict__ out)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k < n) out[k] = (T)a[k];
}

// Per-block partial sums of (d - target)^2 in double, then one block adds the
// partials: a fixed order, so the loss is reproducible.
template <typename T>
__global__ void k_loss_partials(int64_t n, const T* __restrict__ d, const double* __restrict__ target,
                                double* __restrict__ part)
{
    __shared__ double s[TPB];
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    double e = 0.0;
    if (k < n) {
        e = (double)d[k] - target[k];
        e = e * e;
    }
    s[threadIdx.x] = e;
    __syncthreads();
    for (int w = TPB / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_loss_final(int nb, const double* __restrict__ part, double* __restrict__ out)
{
    __shared__ double s[TPB];
    double acc = 0.0;
    for (int k = threadIdx.x; k < nb; k += TPB) acc += part[k];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = TPB / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = s[0];
}

// dL/dd for L = ||d - target||: (d - target) / L.
template <typename T>
__global__ void k_loss_grad(int64_t n, const T* __restrict__ d, const double* __restrict__ target, double inv_l,
                            double* __restrict__ out)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k < n) out[k] = ((double)d[k] - target[k]) * inv_l;
}

unsigned nblocks(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

thread_local std::string g_smoke_error;

}  // namespace

struct fs_smoke
{
    fs_smoke_config cfg{};
    int nx = 0, ny = 0;
    int64_t n = 0;
    double h = 1.0;
    bool fp64 = false;
    bool trace64 = false;  // float fields, back-traces in double
    size_t esize = 4;  // bytes per field value
    fs_poisson* poisson = nullptr;
    cudaStream_t stream = nullptr;
    uint8_t* labels = nullptr;
    // fields in the handle's precision: the initial state, the running state,
    // the checkpoints and the states of one recomputed segment
    void* init[3] = {};
    void* cur[3] = {};
    void* nxt[3] = {};
    std::vector<void*> ckpt;  // 3 per checkpoint
    std::vector<void*> seg;   // 3 per step of a segment
    int steps_done = -1;      // steps of the last forward
    double* target = nullptr;
    double* rhs = nullptr;
    double* pres = nullptr;
    double* lam[3] = {};  // adjoint of the current state (u, v, d)
    double* acc[3] = {};  // adjoint of the previous state
    double* part = nullptr;
    double* scal = nullptr;
    // contribution items of the adjoint's advection step and their grouping
    // by node (allocated by the first backward pass)
    int64_t n_items = 0;
    uint32_t* item_key = nullptr;
    double* item_val = nullptr;
    int32_t* item_sorted = nullptr;
    int32_t* bin_count = nullptr;
    int32_t* bin_start = nullptr;
    int32_t* scan_tmp = nullptr;
    double loss = 0.0;
    int64_t launches = 0;
    std::string err;
};

namespace {

int sfail(fs_smoke* s, int code, const std::string& msg)
{
    if (s) s->err = msg;
    else g_smoke_error = msg;
    return code;
}

int scuda(fs_smoke* s, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return FS_OK;
    return sfail(s, e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename S, typename A = S>
Fields<S, A> fields(const fs_smoke* s, void* const* st)
{
    Fields<S, A> F;
    F.u = static_cast<const S*>(st[0]);
    F.v = static_cast<const S*>(st[1]);
    F.d = static_cast<const S*>(st[2]);
    F.nx = s->nx;
    F.ny = s->ny;
    F.h = (A)s->h;
    return F;
}

void copy_state(fs_smoke* s, void* const* src, void* const* dst)
{
    for (int k = 0; k < 3; ++k) cudaMemcpyAsync(dst[k], src[k], s->esize * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream);
}

// The projection of (u, v) in the handle's precision (fields[0..1]).
int project_fields(fs_smoke* s, void* u, void* v)
{
    const unsigned nb = nblocks(s->n);
    if (s->fp64) k_divergence<double><<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->h, s->labels, (double*)u, (double*)v, s->rhs);
    else k_divergence<float><<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->h, s->labels, (float*)u, (float*)v, s->rhs);
    s->launches += 1;
    fs_poisson_stats st{};
    const int rc = poisson_solve_device(s->poisson, s->rhs, s->pres, s->cfg.projection_method, s->cfg.cg_tolerance,
                                        s->cfg.cg_max_iterations, s->cfg.inner_tolerance, FS_CG_FLOAT, &st);
    if (rc) return sfail(s, rc, std::string("projection: ") + fs_last_error(nullptr));
    if (s->fp64)
        k_subtract_gradient<double><<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->h, s->labels, s->pres, (double*)u, (double*)v);
    else
        k_subtract_gradient<float><<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->h, s->labels, s->pres, (float*)u, (float*)v);
    s->launches += 1;
    return scuda(s, cudaGetLastError(), "projection");
}

// state out = step(state in)
int step_state(fs_smoke* s, void* const* in, void* const* out)
{
    const unsigned nb = nblocks(s->n);
    const double dt = s->cfg.dt;
    if (s->fp64)
        k_advect<double, double><<<nb, TPB, 0, s->stream>>>(fields<double>(s, in), s->labels, s->cfg.integrator, dt,
                                                            (double*)out[0], (double*)out[1], (double*)out[2]);
    else if (s->trace64)
        k_advect<float, double><<<nb, TPB, 0, s->stream>>>(fields<float, double>(s, in), s->labels,
                                                           s->cfg.integrator, dt, (float*)out[0], (float*)out[1],
                                                           (float*)out[2]);
    else
        k_advect<float, float><<<nb, TPB, 0, s->stream>>>(fields<float>(s, in), s->labels, s->cfg.integrator,
                                                          (float)dt, (float*)out[0], (float*)out[1], (float*)out[2]);
    s->launches += 1;
    return project_fields(s, out[0], out[1]);
}

// lam (adjoint of state n+1) -> acc (adjoint of state n), given state n.
int adjoint_step(fs_smoke* s, void* const* state_n)
{
    const unsigned nb = nblocks(s->n);
    // projection (symmetric with the wall condition): lam_uv <- M lam_uv
    k_close_faces<<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->labels, s->lam[0], s->lam[1]);
    k_divergence<double><<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->h, s->labels, s->lam[0], s->lam[1], s->rhs);
    s->launches += 2;
    fs_poisson_stats st{};
    int rc = poisson_solve_device(s->poisson, s->rhs, s->pres, s->cfg.projection_method, s->cfg.cg_tolerance,
                                  s->cfg.cg_max_iterations, s->cfg.inner_tolerance, FS_CG_FLOAT, &st);
    if (rc) return sfail(s, rc, std::string("adjoint projection: ") + fs_last_error(nullptr));
    k_subtract_gradient<double><<<nb, TPB, 0, s->stream>>>(s->nx, s->ny, s->h, s->labels, s->pres, s->lam[0], s->lam[1]);
    s->launches += 1;
    // advection: contribution items, grouped by node, summed in item order
    const Items items{s->item_key, s->item_val, s->n};
    if (s->fp64)
        k_advect_adjoint<double, double><<<nb, TPB, 0, s->stream>>>(fields<double>(s, state_n), s->labels,
                                                                    s->cfg.integrator, s->cfg.dt, s->lam[0],
                                                                    s->lam[1], s->lam[2], items);
    else if (s->trace64)
        k_advect_adjoint<float, double><<<nb, TPB, 0, s->stream>>>(fields<float, double>(s, state_n), s->labels,
                                                                   s->cfg.integrator, s->cfg.dt, s->lam[0],
                                                                   s->lam[1], s->lam[2], items);
    else
        k_advect_adjoint<float, float><<<nb, TPB, 0, s->stream>>>(fields<float>(s, state_n), s->labels,
                                                                  s->cfg.integrator, (float)s->cfg.dt, s->lam[0],
                                                                  s->lam[1], s->lam[2], items);
    s->launches += 1;
    const Launch L{s->stream, &s->launches, 0};
    group_by_key(L, s->n_items, s->item_key, 3 * s->n, s->bin_count, s->bin_start, s->scan_tmp, s->item_sorted);
    k_adjoint_gather<<<nblocks(3 * s->n), TPB, 0, s->stream>>>(s->n, s->bin_start, s->item_sorted, s->item_val,
                                                               s->acc[0], s->acc[1], s->acc[2]);
    s->launches += 1;
    for (int k = 0; k < 3; ++k) std::swap(s->lam[k], s->acc[k]);
    return scuda(s, cudaGetLastError(), "adjoint step");
}

void free_smoke(fs_smoke* s)
{
    if (!s) return;
    cudaSetDevice(s->cfg.device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    std::vector<void*> ptrs = {s->labels, s->target, s->rhs, s->pres, s->part, s->scal, s->item_key, s->item_val,
                               s->item_sorted, s->bin_count, s->bin_start, s->scan_tmp};
    for (int k = 0; k < 3; ++k) {
        ptrs.push_back(s->init[k]);
        ptrs.push_back(s->cur[k]);
        ptrs.push_back(s->nxt[k]);
        ptrs.push_back(s->lam[k]);
        ptrs.push_back(s->acc[k]);
    }
    ptrs.insert(ptrs.end(), s->ckpt.begin(), s->ckpt.end());
    ptrs.insert(ptrs.end(), s->seg.begin(), s->seg.end());
    for (void* p : ptrs) cudaFree(p);
    if (s->poisson) fs_poisson_destroy(s->poisson);
    delete s;
}

int upload_field(fs_smoke* s, const double* host, void* dev)
{
    cudaError_t e = cudaMemcpyAsync(s->rhs, host, 8 * (size_t)s->n, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return scuda(s, e, "upload");
    if (s->fp64) k_from_double<double><<<nblocks(s->n), TPB, 0, s->stream>>>(s->n, s->rhs, (double*)dev);
    else k_from_double<float><<<nblocks(s->n), TPB, 0, s->stream>>>(s->n, s->rhs, (float*)dev);
    s->launches += 1;
    return scuda(s, cudaStreamSynchronize(s->stream), "upload");
}

int download_field(fs_smoke* s, const void* dev, double* host)
{
    if (s->fp64) k_to_double<double><<<nblocks(s->n), TPB, 0, s->stream>>>(s->n, (const double*)dev, s->rhs);
    else k_to_double<float><<<nblocks(s->n), TPB, 0, s->stream>>>(s->n, (const float*)dev, s->rhs);
    s->launches += 1;
    cudaMemcpyAsync(host, s->rhs, 8 * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream);
    return scuda(s, cudaStreamSynchronize(s->stream), "download");
}

}  // namespace

extern "C" {

void fs_smoke_config_init(fs_smoke_config* c, int size_x, int size_y)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->size_x = size_x;
    c->size_y = size_y;
    c->length_x = (float)size_x;
    c->length_y = (float)size_y;
    c->dt = 0.01f;
    c->integrator = FS_INTEGRATOR_RK2;
    c->precision = FS_SMOKE_FP32;
    c->projection_method = FS_POISSON_MIXED;
    c->cg_tolerance = 1e-10;
    c->cg_max_iterations = 100000;
    c->inner_tolerance = 1e-3;
    c->checkpoint_every = 8;
    c->device = 0;
}

const char* fs_smoke_last_error(const fs_smoke* s) { return s ? s->err.c_str() : g_smoke_error.c_str(); }

int fs_smoke_create(const fs_smoke_config* cfg, fs_smoke** out)
{
    g_smoke_error.clear();
    if (!cfg || !out) return sfail(nullptr, FS_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    const fs_smoke_config& c = *cfg;
    if (c.size_x < 3 || c.size_y < 3 || !(c.length_x > 0) || !(c.length_y > 0) || !(c.dt >= 0) ||
        c.integrator < FS_INTEGRATOR_EULER || c.integrator > FS_INTEGRATOR_RK3 ||
        (c.precision != FS_SMOKE_FP32 && c.precision != FS_SMOKE_FP64 && c.precision != FS_SMOKE_FP32_TRACE64) ||
        c.checkpoint_every < 1 ||
        c.projection_method < FS_POISSON_FP32 || c.projection_method > FS_POISSON_MIXED_MG)
        return sfail(nullptr, FS_ERR_INVALID_ARGUMENT, "invalid smoke configuration");
    const double hx = (double)c.length_x / c.size_x, hy = (double)c.length_y / c.size_y;
    if (std::fabs(hx - hy) > 1e-12 * hx) return sfail(nullptr, FS_ERR_INVALID_ARGUMENT, "cells must be square");
    if ((int64_t)c.size_x * c.size_y > (int64_t)4096 * 4096)
        return sfail(nullptr, FS_ERR_TOO_LARGE, "grid larger than 16777216 cells");
    fs_smoke* s = new fs_smoke();
    s->cfg = c;
    s->nx = c.size_x;
    s->ny = c.size_y;
    s->n = (int64_t)c.size_x * c.size_y;
    s->h = hx;
    s->fp64 = c.precision == FS_SMOKE_FP64;
    s->trace64 = c.precision == FS_SMOKE_FP32_TRACE64;
    s->esize = s->fp64 ? 8 : 4;
    cudaError_t e = cudaSetDevice(c.device);
    if (e != cudaSuccess) {
        delete s;
        return scuda(nullptr, e, "cudaSetDevice");
    }
    int rc = fs_poisson_create(c.size_x, c.size_y, c.length_x, c.length_y, c.device, &s->poisson);
    if (rc) {
        g_smoke_error = std::string("projection solver: ") + fs_last_error(nullptr);
        delete s;
        return rc;
    }
    s->stream = poisson_stream(s->poisson);
    const size_t N = (size_t)s->n, F = s->esize * N;
    auto A = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    A((void**)&s->labels, N);
    for (int k = 0; k < 3; ++k) {
        A(&s->init[k], F);
        A(&s->cur[k], F);
        A(&s->nxt[k], F);
        A((void**)&s->lam[k], 8 * N);
        A((void**)&s->acc[k], 8 * N);
    }
    for (double** d : {&s->target, &s->rhs, &s->pres}) A((void**)d, 8 * N);
    A((void**)&s->part, 8 * (size_t)nblocks(s->n));
    A((void**)&s->scal, 8);
    if (e == cudaSuccess) {
        // solid border, fluid inside
        std::vector<uint8_t> lab(N, FS_LIQUID);
        for (int j = 0; j < s->ny; ++j)
            for (int i = 0; i < s->nx; ++i)
                if (i == 0 || j == 0 || i == s->nx - 1 || j == s->ny - 1) lab[i + (size_t)j * s->nx] = FS_SOLID;
        e = cudaMemcpyAsync(s->labels, lab.data(), N, cudaMemcpyHostToDevice, s->stream);
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMemsetAsync(s->init[k], 0, F, s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->target, 0, 8 * N, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
    if (e == cudaSuccess) {
        rc = poisson_set_labels_device(s->poisson, s->labels);
        if (rc) e = cudaErrorUnknown;
    }
    if (e != cudaSuccess) {
        rc = scuda(nullptr, e, "fs_smoke_create");
        free_smoke(s);
        return rc;
    }
    *out = s;
    return FS_OK;
}

int fs_smoke_destroy(fs_smoke* s)
{
    free_smoke(s);
    return FS_OK;
}

int fs_smoke_set_solid_mask(fs_smoke* s, const uint8_t* mask)
{
    if (!s) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->cfg.device);
    std::vector<uint8_t> lab((size_t)s->n, FS_LIQUID);
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
            const size_t c = i + (size_t)j * s->nx;
            if (i == 0 || j == 0 || i == s->nx - 1 || j == s->ny - 1 || (mask && mask[c])) lab[c] = FS_SOLID;
        }
    cudaError_t e = cudaMemcpyAsync(s->labels, lab.data(), (size_t)s->n, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return scuda(s, e, "solid mask");
    const int rc = poisson_set_labels_device(s->poisson, s->labels);
    if (rc) return sfail(s, rc, fs_last_error(nullptr));
    s->steps_done = -1;
    return FS_OK;
}

int fs_smoke_set_state(fs_smoke* s, const double* u, const double* v, const double* density)
{
    if (!s || !u || !v || !density) return s ? sfail(s, FS_ERR_INVALID_ARGUMENT, "null field") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->cfg.device);
    const double* src[3] = {u, v, density};
    for (int k = 0; k < 3; ++k) {
        const int rc = upload_field(s, src[k], s->init[k]);
        if (rc) return rc;
    }
    s->steps_done = -1;
    return FS_OK;
}

int fs_smoke_set_target(fs_smoke* s, const double* target)
{
    if (!s || !target) return s ? sfail(s, FS_ERR_INVALID_ARGUMENT, "null target") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->cfg.device);
    cudaError_t e = cudaMemcpyAsync(s->target, target, 8 * (size_t)s->n, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return scuda(s, e, "target");
}

int fs_smoke_forward(fs_smoke* s, int steps, double* loss)
{
    if (!s || steps < 0) return s ? sfail(s, FS_ERR_INVALID_ARGUMENT, "negative steps") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->cfg.device);
    const int C = s->cfg.checkpoint_every;
    const int nck = (steps + C - 1) / C;
    const size_t F = s->esize * (size_t)s->n;
    cudaError_t e = cudaSuccess;
    while ((int)s->ckpt.size() < 3 * nck && e == cudaSuccess) {
        void* p = nullptr;
        e = cudaMalloc(&p, F);
        if (e == cudaSuccess) s->ckpt.push_back(p);
    }
    while ((int)s->seg.size() < 3 * C && e == cudaSuccess) {
        void* p = nullptr;
        e = cudaMalloc(&p, F);
        if (e == cudaSuccess) s->seg.push_back(p);
    }
    if (e != cudaSuccess) return scuda(s, e, "checkpoint storage");
    copy_state(s, s->init, s->cur);
    for (int n = 0; n < steps; ++n) {
        if (n % C == 0) copy_state(s, s->cur, &s->ckpt[3 * (n / C)]);
        const int rc = step_state(s, s->cur, s->nxt);
        if (rc) return rc;
        for (int k = 0; k < 3; ++k) std::swap(s->cur[k], s->nxt[k]);
    }
    const unsigned nb = nblocks(s->n);
    if (s->fp64) k_loss_partials<double><<<nb, TPB, 0, s->stream>>>(s->n, (const double*)s->cur[2], s->target, s->part);
    else k_loss_partials<float><<<nb, TPB, 0, s->stream>>>(s->n, (const float*)s->cur[2], s->target, s->part);
    k_loss_final<<<1, TPB, 0, s->stream>>>((int)nb, s->part, s->scal);
    s->launches += 2;
    double l2 = 0.0;
    e = cudaMemcpyAsync(&l2, s->scal, 8, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return scuda(s, e, "loss");
    s->loss = std::sqrt(l2);
    s->steps_done = steps;
    if (loss) *loss = s->loss;
    return FS_OK;
}

int fs_smoke_get_state(fs_smoke* s, double* u, double* v, double* density)
{
    if (!s || !u || !v || !density || s->steps_done < 0)
        return s ? sfail(s, FS_ERR_INVALID_ARGUMENT, "no forward run") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->cfg.device);
    double* dst[3] = {u, v, density};
    for (int k = 0; k < 3; ++k) {
        const int rc = download_field(s, s->cur[k], dst[k]);
        if (rc) return rc;
    }
    return FS_OK;
}

int fs_smoke_backward(fs_smoke* s, double* grad_u, double* grad_v, double* grad_density)
{
    if (!s || s->steps_done < 0) return s ? sfail(s, FS_ERR_INVALID_ARGUMENT, "no forward run") : FS_ERR_INVALID_ARGUMENT;
    if (!grad_u || !grad_v || !grad_density) return sfail(s, FS_ERR_INVALID_ARGUMENT, "null gradient");
    cudaSetDevice(s->cfg.device);
    const unsigned nb = nblocks(s->n);
    const size_t bytes = 8 * (size_t)s->n;
    const int steps = s->steps_done, C = s->cfg.checkpoint_every;
    if (!s->item_key) {
        // 3 samples per cell, sample_slots items each; 3 n bins (one per node of u, v, density)
        const int64_t items = (int64_t)s->n * 3 * sample_slots(s->cfg.integrator);
        if (items > INT32_MAX || 3 * s->n >= (int64_t)UINT32_MAX)
            return sfail(s, FS_ERR_TOO_LARGE, "grid too large for the adjoint's contribution items");
        const size_t bins = (size_t)(3 * s->n) + 2;
        cudaError_t e = cudaSuccess;
        auto A = [&](void** p, size_t nbytes) {
            if (e == cudaSuccess) e = cudaMalloc(p, nbytes);
        };
        A((void**)&s->item_key, 4 * (size_t)items);
        A((void**)&s->item_val, 8 * (size_t)items);
        A((void**)&s->item_sorted, 4 * (size_t)items);
        A((void**)&s->bin_count, 4 * bins);
        A((void**)&s->bin_start, 4 * bins);
        A((void**)&s->scan_tmp, 4 * scan_tmp_ints((int64_t)bins));
        if (e != cudaSuccess) {
            for (void** p : {(void**)&s->item_key, (void**)&s->item_val, (void**)&s->item_sorted,
                             (void**)&s->bin_count, (void**)&s->bin_start, (void**)&s->scan_tmp}) {
                cudaFree(*p);
                *p = nullptr;
            }
            return scuda(s, e, "adjoint item buffers");
        }
        s->n_items = items;
    }
    cudaMemsetAsync(s->lam[0], 0, bytes, s->stream);
    cudaMemsetAsync(s->lam[1], 0, bytes, s->stream);
    const double inv_l = s->loss > 0 ? 1.0 / s->loss : 0.0;
    if (s->fp64) k_loss_grad<double><<<nb, TPB, 0, s->stream>>>(s->n, (const double*)s->cur[2], s->target, inv_l, s->lam[2]);
    else k_loss_grad<float><<<nb, TPB, 0, s->stream>>>(s->n, (const float*)s->cur[2], s->target, inv_l, s->lam[2]);
    s->launches += 1;
    for (int first = ((steps - 1) / C) * C; steps > 0 && first >= 0; first -= C) {
        const int last = std::min(first + C, steps);
        // recompute the segment's states from its checkpoint
        copy_state(s, &s->ckpt[3 * (first / C)], &s->seg[0]);
        for (int n = first + 1; n < last; ++n) {
            const int rc = step_state(s, &s->seg[3 * (n - 1 - first)], &s->seg[3 * (n - first)]);
            if (rc) return rc;
        }
        for (int n = last - 1; n >= first; --n) {
            const int rc = adjoint_step(s, &s->seg[3 * (n - first)]);
            if (rc) return rc;
        }
    }
    double* dst[3] = {grad_u, grad_v, grad_density};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpyAsync(dst[k], s->lam[k], bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return scuda(s, e, "gradient download");
}

int64_t fs_smoke_kernel_launches(const fs_smoke* s) { return s ? s->launches + poisson_launches(s->poisson) : 0; }

}  // extern "C"
