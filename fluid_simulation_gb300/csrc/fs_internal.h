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

// ---- launch domains (fs_domain.cuh) ---------------------------------------
constexpr int DOMAIN_TPB = 256;

// One simulation's slice of the flattened arrays (offsets 0 for a lone simulation).
struct Seg
{
    Geom g;
    int64_t co;   // first cell in the flattened cell arrays (a multiple of DOMAIN_TPB)
    int64_t po;   // first particle in the flattened particle arrays (a multiple of DOMAIN_TPB)
    int64_t np;   // particles
    float pic;    // FluidDomain::picRatio
    float rho;    // FluidDomain::density
    float gx, gy; // gravitational acceleration
    int sim;      // index of the simulation (0 for a lone one)
    int cb0;      // first cell block of the simulation (batch only)
    int ncb;      // its cell blocks (batch only)
};

// The simulations a kernel runs over: `one` when segs == nullptr, else every
// simulation of a batch through its block tables (blk[b] = {simulation, first
// local item of block b}, DOMAIN_TPB items per block).
struct Domain
{
    Seg one{};
    const Seg* segs = nullptr;
    const int2* cblk = nullptr;
    unsigned ncblk = 0;
    const int2* pblk = nullptr;
    unsigned npblk = 0;
    int nsim = 1;
    int64_t cells = 0;  // flattened cells
    int64_t parts = 0;  // flattened particles

    static Domain single(const Seg& s)
    {
        Domain d;
        d.one = s;
        d.cells = (int64_t)s.g.nx * s.g.ny;
        d.parts = s.np;
        return d;
    }
};

// ---- scan (fs_scan.cu) ----------------------------------------------------
// Exclusive prefix sum of n int32 values into out[0..n]; out[n] = total.
// tmp must hold scan_tmp_ints(n) ints: one partial sum per tile of
// SCAN_TILE_ITEMS items, plus one.
constexpr int64_t SCAN_TILE_ITEMS = 4096;
constexpr size_t scan_tmp_ints(int64_t n) { return (size_t)((n + SCAN_TILE_ITEMS - 1) / SCAN_TILE_ITEMS) + 1; }
void scan_exclusive_i32(const Launch& L, const int32_t* in, int32_t* out, int64_t n, int32_t* tmp);
// Fluid indexing (FluidSolver.cpp:329-346): fidx[c] = running index of LIQUID
// cells in j-major order or -1; cell_of[k] = c; *nfluid = count.
void fluid_index(const Launch& L, const uint8_t* labels, int64_t n, int32_t* fidx, int32_t* cell_of,
                 int32_t* nfluid, int32_t* tmp);
// The same per simulation of a batch: local fluid indices, cell_of[co + k] =
// local cell, nfluid[sim].  tmp must hold 2 * (d.ncblk + 1) + scan_tmp_ints(d.ncblk + 1) ints.
size_t fluid_index_batch_tmp_ints(const Domain& d);
void fluid_index_batch(const Launch& L, const Domain& d, const uint8_t* labels, int32_t* fidx, int32_t* cell_of,
                       int32_t* nfluid, int32_t* tmp);

// ---- counting-sort binning + ordered splat (fs_splat.cu) -----------------
struct SplatWork
{
    uint32_t* keys = nullptr;      // bin of each item
    int32_t* sorted = nullptr;     // items grouped by bin, each bin in item order
    int32_t* bin_count = nullptr;  // cells + 2
    int32_t* bin_start = nullptr;  // cells + 2
    int32_t* scan_tmp = nullptr;
    float *xs = nullptr, *ys = nullptr;  // scaled positions x / dx, y / dy of the valid items
    int64_t cap_items = 0;
    int64_t cells = 0;
};
// Groups items 0..n-1 by key (keys[k] < nbins; keys[k] == nbins: left out):
// bin_start[0..nbins] (nbins + 1 entries) and sorted[], each bin's items in
// increasing k.  bin_count holds nbins + 1 ints, scan_tmp scan_tmp_ints(nbins).
void group_by_key(const Launch& L, int64_t n, const uint32_t* keys, int64_t nbins, int32_t* bin_count,
                  int32_t* bin_start, int32_t* scan_tmp, int32_t* sorted);
// Buffers for up to `items` items over `cells` cells (frees what w held).
cudaError_t splat_alloc(SplatWork& w, int64_t items, int64_t cells);
void splat_free(SplatWork& w);
// Accumulates, for each node of every simulation of d, sum over that
// simulation's items k in increasing k of the bilinear splat
// (Grid::addToValueInterpolated, include/Grid.h:152-184) of value[c][k] at
// (x[k], y[k]) for channel c, exactly as a sequential loop over k would (float
// adds in item order, corner order 00, 10, 01, 11).  Items are the particles
// (items_are_cells false) or the cells of d, in the flattened layout; items
// with valid[k] == 0 (or valid == nullptr: all valid) contribute nothing.
// pool_deltas selects the solver pool's deltas (pdx, pdy) instead of (dx, dy).
// out[c] are overwritten (start from +0).
void ordered_splat(const Launch& L, const Domain& d, bool items_are_cells, bool pool_deltas, const float* x,
                   const float* y, const uint8_t* valid, int channels, const float* const* values,
                   float* const* out, SplatWork& w);

// ---- grid kernels (fs_grid.cu) -------------------------------------------
// Cell arrays are flattened (simulation s at d's cell offset co); particle
// arrays likewise at po.  Per-simulation scalars come from the Seg.
void labels_clear(const Launch& L, const Domain& d, uint8_t* lab);
void labels_from_particles(const Launch& L, const Domain& d, const float* px, const float* py, uint8_t* lab);
void labels_finalize(const Launch& L, const Domain& d, uint8_t* lab, const uint8_t* solid);
void count_particles(const Launch& L, const Domain& d, const float* px, const float* py, int32_t* counts32,
                     unsigned* warn);
// labels_from_particles and count_particles in one pass over the particles.
void labels_and_counts(const Launch& L, const Domain& d, const float* px, const float* py, uint8_t* lab,
                       int32_t* counts32, unsigned* warn);
// gravity, dirichlet and extend_init in one pass over the faces.
void forces_extend_init(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf, float dt,
                        float* ub, float* vb, uint8_t* mxf, uint8_t* mxb, uint8_t* myf, uint8_t* myb);
void p2g_finish(const Launch& L, const Domain& d, const float* sum_u, const float* w_u, const float* sum_v,
                const float* w_v, float* ub, float* vb);
void grid_copy2(const Launch& L, const Domain& d, const float* a0, const float* a1, float* b0, float* b1);
void grid_diff(const Launch& L, const Domain& d, const float* uf, const float* vf, const float* up,
               const float* vp, float* ud, float* vd);
void gravity(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf, float dt);
void dirichlet(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf);
void extend_init(const Launch& L, const Domain& d, const uint8_t* lab, float* uf, float* vf, float* ub, float* vb,
                 uint8_t* mxf, uint8_t* mxb, uint8_t* myf, uint8_t* myb);
void extend_sweep(const Launch& L, const Domain& d, const uint8_t* lab, float* ub, float* vb, const uint8_t* mxf,
                  uint8_t* mxb, const uint8_t* myf, uint8_t* myb);
// nfluid[sim]; fluid-index vectors of simulation s start at its cell offset co.
void assemble(const Launch& L, const Domain& d, const uint8_t* lab, const int32_t* fidx, const int32_t* cell_of,
              const int32_t* nfluid, const float* uf, const float* vf, float* b, int32_t* down, int32_t* up,
              uint8_t* flags, const int32_t* counts32, uint8_t* counts8);
void project(const Launch& L, const Domain& d, const int32_t* fidx, const int32_t* nfluid, const float* x,
             float* uf, float* vf, float* ub, float* vb, float dt);
void pressure_to_grid(const Launch& L, const Domain& d, const int32_t* fidx, const int32_t* nfluid,
                      const float* x, float* out);
// The level set (one simulation): FluidDomain::advectLevelSet into out, and
// FluidDomain::classifyCells(LevelSet&).
void advect_level_set(const Launch& L, const Domain& d, const float* ls, const float* uf, const float* vf, float dt,
                      float* out);
void classify_level_set(const Launch& L, const Domain& d, const float* ls, uint8_t* lab, const uint8_t* solid);

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
void g2p_advect(const Launch& L, const Domain& d, int g2p_mode, int adv_mode, float* px, float* py, float* pvx,
                float* pvy, const float* uf, const float* vf, const float* ud, const float* vd, const uint8_t* lab,
                float dt);
void p2g_positions(const Launch& L, const Domain& d, const float* px, const float* py, float* yu, float* xv);
void sl_faces(const Launch& L, const Domain& d, const uint8_t* lab, const float* uf, const float* vf, float dt,
              float* ux, float* uy, float* uval, uint8_t* uok, float* vx, float* vy, float* vval, uint8_t* vok);
// Appends nx * ny particles (xs[i], ys[j], vx, vy), j outer, i inner.
void spawn_lattice(const Launch& L, const float* xs, int nx, const float* ys, int ny, float vx, float vy, float* px,
                   float* py, float* pvx, float* pvy);
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
    double* partials;   // chunk partials of the reductions, [2 buffers][2 values][max chunks]
    double* groups = nullptr;  // group partials, [2 buffers][2 values][ceil(max chunks / 32)], or null
    unsigned* barrier;  // arrival counter of the grid barrier, cleared before every solve
    CgResult* result;
    int32_t* route = nullptr;  // 2 ints: the fluid cells k_cg and the pipelined kernel take (large systems)
    int64_t max_cells;
    int grid;           // co-resident CTAs of the cooperative launch
    unsigned missing_arrivals = 0;       // test hook: barrier waits for CTAs that do not exist
    uint64_t wait_ns = 2000000000ull;    // bound of every device-side wait
};
int cg_prepare(CgWork& w, int device);  // picks the cooperative grid size
// fp64: 0 = float dot products (the reference's precision), 1 = double,
// 2 = double-single (FS_CG_DS: compensated float pairs within each warp,
// double above).
void cg_solve(const Launch& L, CgWork& w, const int32_t* nfluid, const float* b, const float* diag_tab,
              const int32_t* down, const int32_t* up, const uint8_t* flags, float off, double tol, int maxit,
              int fp64, unsigned* status);

// One system of a batch of independent pressure solves (a simulation of a batch).
struct CgSystem
{
    int64_t co;        // its fluid-index vectors start at this offset (the simulation's cell offset)
    int64_t part_off;  // its chunk partials start here (doubles)
    int max_chunks;    // chunk capacity of its partial buffers
    float dtab[5];     // diagonal by non-solid count
    float itab[5];     // 1 / diagonal, or 1 where the diagonal is 0
    float off;         // off-diagonal coefficient
    double tol;
    int maxit;
};
struct CgBatchArgs
{
    const CgSystem* systems;  // [simulation]
    const int32_t* order;     // simulation of each cluster of the launch
    const int32_t* nfluid;    // [simulation]
    const float* b;
    const int32_t* down;
    const int32_t* up;
    const uint8_t* flags;
    float *x, *r, *z, *p, *q;
    double* partials;
    unsigned* status;
    CgResult* result;  // [simulation]
    int fp64;
};
// Co-resident clusters of `cluster` CTAs with chunks_per_cta (4 or 8)
// chunks of shared-memory state each (also sets the kernel's shared-memory
// attribute); < 1 if that shape cannot run.
int cg_cluster_capacity(int chunks_per_cta, int cluster);
// Solves systems order[0..nsys) of ba, one cluster each; a system of more than
// chunks_per_cta * cluster chunks of 1024 fluid cells streams its state from
// global memory instead of holding it in shared memory.
cudaError_t cg_solve_clusters(const Launch& L, const CgBatchArgs& ba, int nsys, int chunks_per_cta, int cluster);

// ---- the Poisson solver of fs_poisson.cu, from device pointers --------------
// Labels (device, FS_* cell types) define the system; d_rhs and d_x hold one
// double per cell (the solution is 0 outside fluid).  Work runs on the
// solver's own stream; the call returns after the solve.
cudaStream_t poisson_stream(const fs_poisson* p);
int poisson_set_labels_device(fs_poisson* p, const uint8_t* d_labels);
int poisson_solve_device(fs_poisson* p, const double* d_rhs, double* d_x, int method, double tol, int max_iterations,
                         double inner_tolerance, int inner_precision, fs_poisson_stats* stats);
int64_t poisson_launches(const fs_poisson* p);

}  // namespace fs
