// Per-particle kernels: grid-to-particle transfers, particle advection, the
// semi-Lagrangian back-trace of faces, and layout conversion.  Particles are
// stored as four SoA float arrays (x, y, vx, vy) in the caller's order.
#include "fs_domain.cuh"

namespace fs {
namespace {

constexpr int TPB = 256;

// transferVelocityToParticles{PICFLIP,PIC,FLIP} (src/FluidSolver.cpp:921-963)
// followed by MarkerParticleSet::advectAndEnsureOutsideObstacles
// (src/MarkerParticleSet.cpp:48-62), ::advect (:40-46) or
// FluidSolver::advectParticlesWithGrid (src/FluidSolver.cpp:774-791).
struct G2PAdvect
{
    int g2p, adv;
    float *px, *py, *pvx, *pvy;
    const float *uf, *vf, *ud, *vd;
    const uint8_t* lab;
    float dt;
    __device__ void operator()(const Seg& s, int64_t kl) const
    {
        const Geom& g = s.g;
        const int64_t k = s.po + kl;
        const float* U = uf + s.co;
        const float* V = vf + s.co;
        const float r = s.pic;
        float x = px[k], y = py[k], vx = pvx[k], vy = pvy[k];
        if (g2p == G2P_PICFLIP) {
            const float pic_x = vel_x_interp(U, g, x, y);
            const float pic_y = vel_y_interp(V, g, x, y);
            const float flip_x = fadd(vx, vel_x_interp(ud + s.co, g, x, y));
            const float flip_y = fadd(vy, vel_y_interp(vd + s.co, g, x, y));
            const float omr = fsub(1.0f, r);
            vx = fadd(fmul(pic_x, r), fmul(flip_x, omr));
            vy = fadd(fmul(pic_y, r), fmul(flip_y, omr));
        } else if (g2p == G2P_PIC) {
            vx = vel_x_interp(U, g, x, y);
            vy = vel_y_interp(V, g, x, y);
        } else if (g2p == G2P_FLIP) {
            const float a = vel_x_interp(ud + s.co, g, x, y);
            const float b = vel_y_interp(vd + s.co, g, x, y);
            vx = fadd(vx, a);
            vy = fadd(vy, b);
        }
        if (adv == ADV_SAFE || adv == ADV_PLAIN) {
            x = fadd(x, fmul(vx, dt));
            y = fadd(y, fmul(vy, dt));
            if (adv == ADV_SAFE) {
                const int ci = trunc_i(fdiv(x, g.dx));
                const int cj = trunc_i(fdiv(y, g.dy));
                if (cell_type(lab + s.co, g, ci, cj) == SOLID) {
                    const float mdt = -dt;
                    x = fadd(x, fmul(vx, mdt));
                    y = fadd(y, fmul(vy, mdt));
                }
            }
        } else if (adv == ADV_RK3) {
            float ox, oy;
            advected_position(U, V, g, x, y, dt, &ox, &oy);
            x = ox;
            y = oy;
        }
        px[k] = x;
        py[k] = y;
        pvx[k] = vx;
        pvy[k] = vy;
    }
};

// Splat positions of transferVelocityToGridSpread (src/FluidSolver.cpp:889-896):
// u at (px, py - 0.5 dy), v at (px - 0.5 dx, py).
struct P2GPositions
{
    const float *px, *py;
    float *yu, *xv;
    __device__ void operator()(const Seg& s, int64_t kl) const
    {
        const int64_t k = s.po + kl;
        yu[k] = fsub(py[k], fmul(s.g.dy, 0.5f));
        xv[k] = fsub(px[k], fmul(s.g.dx, 0.5f));
    }
};

// advectVelocitySemiLagrangian's per-face work (src/FluidSolver.cpp:725-769):
// for faces with a liquid neighbour, the RK3 back-traced splat position and
// the velocity sampled at the face.
struct SLFaces
{
    const uint8_t* lab;
    const float *uf, *vf;
    float dt;
    float *ux, *uy, *uval;
    uint8_t* uok;
    float *vx, *vy, *vval;
    uint8_t* vok;
    __device__ void operator()(const Seg& s, int64_t cl, int i, int j) const
    {
        const Geom& g = s.g;
        const uint8_t* L = lab + s.co;
        const float* U = uf + s.co;
        const float* V = vf + s.co;
        const int64_t c = s.co + cl;
        const bool liq = L[cl] == LIQUID;
        const float mdt = -dt;
        if (liq || cell_type(L, g, i - 1, j) == LIQUID) {
            const float x = fmul((float)i, g.dx);
            const float y = fmul(fadd((float)j, 0.5f), g.dy);
            float xp, yp;
            advected_position(U, V, g, x, y, mdt, &xp, &yp);
            uval[c] = vel_x_interp(U, g, x, y);
            ux[c] = xp;
            uy[c] = fsub(yp, fmul(g.dy, 0.5f));
            uok[c] = 1;
        } else {
            uok[c] = 0;
        }
        if (liq || cell_type(L, g, i, j - 1) == LIQUID) {
            const float x = fmul(fadd((float)i, 0.5f), g.dx);
            const float y = fmul((float)j, g.dy);
            float xp, yp;
            advected_position(U, V, g, x, y, mdt, &xp, &yp);
            vval[c] = vel_y_interp(V, g, x, y);
            vx[c] = fsub(xp, fmul(g.dx, 0.5f));
            vy[c] = yp;
            vok[c] = 1;
        } else {
            vok[c] = 0;
        }
    }
};

// MarkerParticle(x, y, vx, vy) for y over ys (outer) and x over xs (inner),
// the loop order of FluidSource::update (src/FluidDomain.cpp:39-47).
__global__ void k_spawn_lattice(const float* __restrict__ xs, int nx, const float* __restrict__ ys, int64_t n,
                                float vx, float vy, float* __restrict__ px, float* __restrict__ py,
                                float* __restrict__ pvx, float* __restrict__ pvy)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    px[t] = xs[t % nx];
    py[t] = ys[t / nx];
    pvx[t] = vx;
    pvy[t] = vy;
}

__global__ void k_aos_to_soa(const float4* __restrict__ in, int64_t n, float* __restrict__ px,
                             float* __restrict__ py, float* __restrict__ pvx, float* __restrict__ pvy)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 p = in[k];
    px[k] = p.x;
    py[k] = p.y;
    pvx[k] = p.z;
    pvy[k] = p.w;
}

__global__ void k_soa_to_aos(const float* __restrict__ px, const float* __restrict__ py,
                             const float* __restrict__ pvx, const float* __restrict__ pvy, int64_t n,
                             float4* __restrict__ out)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    out[k] = make_float4(px[k], py[k], pvx[k], pvy[k]);
}

unsigned blocks_for(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

}  // namespace

void g2p_advect(const Launch& L, const Domain& d, int g2p_mode, int adv_mode, float* px, float* py, float* pvx,
                float* pvy, const float* uf, const float* vf, const float* ud, const float* vd, const uint8_t* lab,
                float dt)
{
    each_particle(L, d, G2PAdvect{g2p_mode, adv_mode, px, py, pvx, pvy, uf, vf, ud, vd, lab, dt});
}

void p2g_positions(const Launch& L, const Domain& d, const float* px, const float* py, float* yu, float* xv)
{
    each_particle(L, d, P2GPositions{px, py, yu, xv});
}

void sl_faces(const Launch& L, const Domain& d, const uint8_t* lab, const float* uf, const float* vf, float dt, float* ux,
              float* uy, float* uval, uint8_t* uok, float* vx, float* vy, float* vval, uint8_t* vok)
{
    each_cell(L, d, SLFaces{lab, uf, vf, dt, ux, uy, uval, uok, vx, vy, vval, vok});
}

void spawn_lattice(const Launch& L, const float* xs, int nx, const float* ys, int ny, float vx, float vy, float* px,
                   float* py, float* pvx, float* pvy)
{
    const int64_t n = (int64_t)nx * ny;
    if (n <= 0) return;
    k_spawn_lattice<<<blocks_for(n), TPB, 0, L.stream>>>(xs, nx, ys, n, vx, vy, px, py, pvx, pvy);
    L.count();
}

void aos_to_soa(const Launch& L, const float* xyuv, int64_t n, float* px, float* py, float* pvx, float* pvy)
{
    if (n <= 0) return;
    k_aos_to_soa<<<blocks_for(n), TPB, 0, L.stream>>>(reinterpret_cast<const float4*>(xyuv), n, px, py, pvx, pvy);
    L.count();
}

void soa_to_aos(const Launch& L, const float* px, const float* py, const float* pvx, const float* pvy, int64_t n,
                float* xyuv)
{
    if (n <= 0) return;
    k_soa_to_aos<<<blocks_for(n), TPB, 0, L.stream>>>(px, py, pvx, pvy, n, reinterpret_cast<float4*>(xyuv));
    L.count();
}

}  // namespace fs
