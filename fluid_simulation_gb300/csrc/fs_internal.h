// Host-side launch wrappers of the fsgpu kernels (one declaration per kernel
// family).  Every wrapper queues work on L.stream and counts its launches.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fs_common.cuh"

namespace fs {

// Sets the message fs_last_error(NULL) returns on this thread.
void set_thread_error(const char* msg);

struct Launch
{
    cudaStream_t stream;
    int64_t* counter;  // kernels queued (for the launch count the API reports)
    int num_sms;
    void count(int n = 1) const
    {
        if (counter) *counter += n;
    }
};

// ---- scan (fs_scan.cu) ----------------------------------------------------
// Exclusive prefix sum of n int32 values into out[0..n]; out[n] = total.
// tmp must hold scan_tmp_ints(n) ints.
size_t scan_tmp_ints(int64_t n);
void scan_exclusive_i32(const Launch& L, const int32_t* in, int32_t* out, int64_t n, int32_t* tmp);
// Fluid indexing (FluidSolver.cpp:329-346): fidx[c] = running index of LIQUID
// cells in j-major order or -1; cell_of[k] = c; *nfluid = count.
void fluid_index(const Launch& L, const uint8_t* labels, int64_t n, int32_t* fidx, int32_t* cell_of,
                 int32_t* nfluid, int32_t* tmp);

// ---- stable radix sort + ordered splat (fs_splat.cu) ---------------------
struct SplatWork
{
    // Sort buffers sized for the largest item count.
    uint32_t *keys_a, *keys_b;
    int32_t *vals_a, *vals_b;
    int32_t* hist;       // 256 * blocks(n) + 1
    int32_t* hist_scan;  // same
    int32_t* scan_tmp;
    int32_t* bin_start;  // cells + 1
    int64_t cap_items;
};
size_t splat_hist_ints(int64_t n_items);
// Accumulates, for each node of a size nx*ny grid, sum over items k in
// increasing k of the bilinear splat (Grid::addToValueInterpolated,
// include/Grid.h:152-184) of value[c][k] at (x[k], y[k]) for channel c, exactly
// as a sequential loop over k would (float adds in item order, corner order
// 00, 10, 01, 11).  Items with valid[k] == 0 (or valid == nullptr: all valid)
// contribute nothing.  out[c] are overwritten (start from +0).
void ordered_splat(const Launch& L, const Geom& g, float gdx, float gdy, int64_t n_items, const float* x,
                   const float* y, const uint8_t* valid, int channels, const float* const* values,
                   float* const* out, SplatWork& w);

// ---- grid kernels (fs_grid.cu) -------------------------------------------
void labels_clear(const Launch& L, const Geom& g, uint8_t* lab);
void labels_from_particles(const Launch& L, const Geom& g, const float* px, const float* py, int64_t n,
                           uint8_t* lab);
void labels_finalize(const Launch& L, const Geom& g, uint8_t* lab, const uint8_t* solid);
void count_particles(const Launch& L, const Geom& g, const float* px, const float* py, int64_t n,
                     int32_t* counts32, unsigned* warn);
void p2g_finish(const Launch& L, const Geom& g, const float* sum_u, const float* w_u, const float* sum_v,
                const float* w_v, float* ub, float* vb);
void grid_copy2(const Launch& L, const Geom& g, const float* a0, const float* a1, float* b0, float* b1);
void grid_diff(const Launch& L, const Geom& g, const float* uf, const float* vf, const float* up,
               const float* vp, float* ud, float* vd);
void gravity(const Launch& L, const Geom& g, const uint8_t* lab, float* uf, float* vf, float ax_dt,
             float ay_dt);
void dirichlet(const Launch& L, const Geom& g, const uint8_t* lab, float* uf, float* vf);
void extend_init(const Launch& L, const Geom& g, const uint8_t* lab, float* uf, float* vf, float* ub, float* vb,
                 uint8_t* mxf, uint8_t* mxb, uint8_t* myf, uint8_t* myb);
void extend_sweep(const Launch& L, const Geom& g, const uint8_t* lab, float* ub, float* vb, const uint8_t* mxf,
                  uint8_t* mxb, const uint8_t* myf, uint8_t* myb);
void assemble(const Launch& L, const Geom& g, const uint8_t* lab, const int32_t* fidx, const int32_t* cell_of,
              const int32_t* nfluid, const float* uf, const float* vf, float* b, int32_t* down, int32_t* up,
              uint8_t* flags, const int32_t* counts32, uint8_t* counts8);
void project(const Launch& L, const Geom& g, const int32_t* fidx, const int32_t* nfluid, const float* x,
             float* uf, float* vf, float* ub, float* vb, float dt_over_rho);
void pressure_to_grid(const Launch& L, const Geom& g, const int32_t* fidx, const int32_t* nfluid,
                      const float* x, float* out);

// ---- particle kernels (fs_particles.cu) ----------------------------------
enum G2PMode
{
    G2P_NONE = 0,
    G2P_PICFLIP = 1,
    G2P_PIC = 2,
    G2P_FLIP = 3
};
enum AdvectMode
{
    ADV_NONE = 0,
    ADV_SAFE = 1,
    ADV_PLAIN = 2,
    ADV_RK3 = 3
};
void g2p_advect(const Launch& L, const Geom& g, int g2p_mode, int adv_mode, float* px, float* py, float* pvx,
                float* pvy, int64_t n, const float* uf, const float* vf, const float* ud, const float* vd,
                const uint8_t* lab, float pic_ratio, float dt);
void p2g_positions(const Launch& L, const Geom& g, const float* px, const float* py, int64_t n, float* yu,
                   float* xv);
void sl_faces(const Launch& L, const Geom& g, const uint8_t* lab, const float* uf, const float* vf, float dt,
              float* ux, float* uy, float* uval, uint8_t* uok, float* vx, float* vy, float* vval, uint8_t* vok);
void aos_to_soa(const Launch& L, const float* xyuv, int64_t n, float* px, float* py, float* pvx, float* pvy);
void soa_to_aos(const Launch& L, const float* px, const float* py, const float* pvx, const float* pvy, int64_t n,
                float* xyuv);

// ---- conjugate gradient (fs_cg.cu) ---------------------------------------
struct CgResult
{
    int iterations;
    int status;  // ST_* bits
    double rr;   // final ||r||^2
    double bb;   // ||b||^2
};
struct CgWork
{
    float *x, *r, *z, *p, *q;
    double* partials;   // tagged partial words, 8 per chunk (zeroed once at allocation)
    unsigned* barrier;  // reduction sequence number; persists across launches (zeroed at allocation)
    CgResult* result;
    int64_t max_cells;
    int grid;           // co-resident CTAs of the cooperative launch
};
int cg_prepare(CgWork& w, int device);  // picks the cooperative grid size
// fp64: 0 = float dot products (the reference's precision), 1 = double.
void cg_solve(const Launch& L, CgWork& w, const int32_t* nfluid, const float* b, const float* diag_tab,
              const int32_t* down, const int32_t* up, const uint8_t* flags, float off, double tol, int maxit,
              int fp64, unsigned* status);

}  // namespace fs
