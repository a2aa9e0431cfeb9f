// C ABI (include/fsgpu.h): one handle = one FluidDomain + FluidSolver pair
// resident in device memory, stepped by the kernels of this library on the
// handle's CUDA stream.  A whole step is recorded once into a CUDA graph (per
// method, dt, buffer parity and particle count) and replayed afterwards.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fs_mg.h"
#include "fs_render.h"
#include "fs_step.h"

using namespace fs;

namespace {

thread_local std::string g_create_error;

}  // namespace

void fs::set_thread_error(const char* msg) { g_create_error = msg ? msg : ""; }

namespace {

struct GraphEntry
{
    int method;
    uint32_t dt_bits;
    int front_in, vfront_in;
    int front_out, vfront_out;
    int64_t n_part;
    bool timing;
    int64_t kernels;
    cudaGraphExec_t exec;
};

uint32_t float_bits(float f)
{
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

// FluidSource (src/FluidDomain.cpp:3-52): the timing state on the host, the
// spawn lattice's coordinates -- the reference's float-accumulated loop
// variables, expanded once -- on the device.
struct DevSource
{
    float vx, vy, time_step, time_since_last;
    int max_spawns, n_spawns;
    int nx, ny;
    float* d_xs;
    float* d_ys;
};

}  // namespace

struct fs_handle
{
    fs_config cfg{};
    Geom g{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t ncell = 0;

    int front = 0, vfront = 0;
    float* u[2] = {nullptr, nullptr};
    float* v[2] = {nullptr, nullptr};
    float *u_prev = nullptr, *v_prev = nullptr, *u_diff = nullptr, *v_diff = nullptr;
    uint8_t* labels = nullptr;
    uint8_t* solid = nullptr;
    float* level_set = nullptr;      // FluidDomain::_level_set
    float* level_set_tmp = nullptr;  // the new LevelSet of an advection
    uint8_t* vmx[2] = {nullptr, nullptr};
    uint8_t* vmy[2] = {nullptr, nullptr};
    int32_t *fidx = nullptr, *cell_of = nullptr, *counts32 = nullptr;
    uint8_t* counts8 = nullptr;
    float* acc[4] = {nullptr, nullptr, nullptr, nullptr};
    float* grid_tmp = nullptr;

    // semi-Lagrangian face scratch (allocated on first use)
    float* sl[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint8_t* sl_ok[2] = {nullptr, nullptr};

    // particles (SoA)
    float *px = nullptr, *py = nullptr, *pvx = nullptr, *pvy = nullptr;
    float *yu = nullptr, *xv = nullptr;
    float* staging = nullptr;  // AoS staging, 4 * cap floats
    int64_t n_part = 0, cap_part = 0;

    SplatWork sw{};
    SplatWork sw2{};              // the v splats' scratch, beside the u splats on aux
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;

    // pressure solve
    CgWork cg{};
    float* cg_b = nullptr;
    int32_t *cg_down = nullptr, *cg_up = nullptr;
    uint8_t* cg_flags = nullptr;
    int32_t* d_nfluid = nullptr;
    unsigned* d_status = nullptr;
    unsigned* d_warn = nullptr;
    int32_t* scan_tmp = nullptr;
    float diag_tab[5]{};
    float off = 0.0f;

    float pic = 0.0f;
    float gx = 0.0f, gy = -9.82f;
    double cg_tol = 0.0;
    int cg_maxit = 100;
    int cg_fp64 = 0;
    int n_ext = 2;
    int solver = FS_SOLVER_JACOBI_PCG;
    MgSolver* mg = nullptr;  // FS_SOLVER_MGPCG, made on first use
    float* mg_b = nullptr;
    cudaError_t mg_error = cudaSuccess;

    bool timing = false;
    bool graphs = true;
    bool timed_valid = false;
    cudaEvent_t ev[FS_NUM_TIMED + 1] = {};
    int64_t launches = 0;
    std::vector<GraphEntry> graph_cache;
    std::vector<DevSource> sources;
    std::string err;

    Launch L() { return Launch{stream, &launches, 0}; }
};

// A device copy of a handle's simulation state (fs_snapshot / fs_restore).
struct fs_saved_state
{
    const fs_handle* owner = nullptr;
    int64_t ncell = 0, n_part = 0;
    int front = 0, vfront = 0;
    unsigned char* cells = nullptr;  // cell arrays, one after another
    float* parts = nullptr;          // x, y, vx, vy
    unsigned char* misc = nullptr;   // nfluid, CG result, warnings
    std::vector<float> src_time;
    std::vector<int> src_spawns;
};

namespace {

int fail(fs_handle* h, int code, const std::string& msg)
{
    if (h) h->err = msg;
    return code;
}

int cuda_fail(fs_handle* h, cudaError_t e, const char* what)
{
    return fail(h, e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
cudaError_t dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

void clear_graphs(fs_handle* h)
{
    for (auto& e : h->graph_cache) cudaGraphExecDestroy(e.exec);
    h->graph_cache.clear();
}

cudaError_t ensure_splat_capacity(fs_handle* h, int64_t items)
{
    if (items <= h->sw.cap_items) return cudaSuccess;
    cudaError_t e = splat_alloc(h->sw, items, h->ncell);
    if (e == cudaSuccess) e = splat_alloc(h->sw2, items, h->ncell);
    clear_graphs(h);
    return e;
}

cudaError_t ensure_particle_capacity(fs_handle* h, int64_t n)
{
    if (n <= h->cap_part) return cudaSuccess;
    int64_t cap = h->cap_part ? h->cap_part : 4096;
    while (cap < n) cap *= 2;
    float* np[7] = {};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = dalloc(&np[k], (size_t)cap);
    if (e == cudaSuccess) e = dalloc(&np[6], (size_t)cap * 4);
    if (e != cudaSuccess) {
        for (float* p : np) cudaFree(p);
        return e;
    }
    if (h->n_part > 0) {
        const size_t bytes = sizeof(float) * (size_t)h->n_part;
        cudaMemcpyAsync(np[0], h->px, bytes, cudaMemcpyDeviceToDevice, h->stream);
        cudaMemcpyAsync(np[1], h->py, bytes, cudaMemcpyDeviceToDevice, h->stream);
        cudaMemcpyAsync(np[2], h->pvx, bytes, cudaMemcpyDeviceToDevice, h->stream);
        cudaMemcpyAsync(np[3], h->pvy, bytes, cudaMemcpyDeviceToDevice, h->stream);
    }
    cudaStreamSynchronize(h->stream);
    cudaFree(h->px);
    cudaFree(h->py);
    cudaFree(h->pvx);
    cudaFree(h->pvy);
    cudaFree(h->yu);
    cudaFree(h->xv);
    cudaFree(h->staging);
    h->px = np[0];
    h->py = np[1];
    h->pvx = np[2];
    h->pvy = np[3];
    h->yu = np[4];
    h->xv = np[5];
    h->staging = np[6];
    h->cap_part = cap;
    clear_graphs(h);
    return ensure_splat_capacity(h, std::max<int64_t>(cap, h->ncell));
}

cudaError_t ensure_sl_scratch(fs_handle* h)
{
    if (h->sl[0]) return cudaSuccess;
    cudaError_t e;
    for (int k = 0; k < 6; ++k)
        if ((e = dalloc(&h->sl[k], (size_t)h->ncell)) != cudaSuccess) return e;
    for (int k = 0; k < 2; ++k)
        if ((e = dalloc(&h->sl_ok[k], (size_t)h->ncell)) != cudaSuccess) return e;
    return ensure_splat_capacity(h, std::max<int64_t>(h->cap_part, h->ncell));
}

float* UF(fs_handle* h) { return h->u[h->front]; }
float* VF(fs_handle* h) { return h->v[h->front]; }
float* UB(fs_handle* h) { return h->u[1 - h->front]; }
float* VB(fs_handle* h) { return h->v[1 - h->front]; }

Seg seg(const fs_handle* h)
{
    Seg s{};
    s.g = h->g;
    s.np = h->n_part;
    s.pic = h->pic;
    s.rho = h->cfg.density;
    s.gx = h->gx;
    s.gy = h->gy;
    return s;
}

Domain domain(const fs_handle* h) { return Domain::single(seg(h)); }

void solve_hook(void* owner, const Launch& L)
{
    fs_handle* h = static_cast<fs_handle*>(owner);
    if (h->solver == FS_SOLVER_MGPCG) {
        // the system on the cell grid, its solution back in fluid-index order
        mg_set_labels(h->mg, L.stream, h->labels, L.counter);
        mg_fluid_to_cells<float>(L, h->ncell, h->fidx, h->d_nfluid, h->cg_b, h->mg_b);
        int iters = 0;
        double rr = 0, bb = 0;
        float* xc = nullptr;
        cudaError_t e = mg_solve(h->mg, L.stream, h->mg_b, h->cg_tol, h->cg_maxit, L.counter, &iters, &rr, &bb, &xc);
        if (e == cudaSuccess) {
            mg_cells_to_fluid<float>(L, h->ncell, h->d_nfluid, h->cell_of, xc, h->cg.x);
            const CgResult r{iters, 0, rr, bb};
            e = cudaMemcpy(h->cg.result, &r, sizeof(r), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess && h->mg_error == cudaSuccess) h->mg_error = e;
        return;
    }
    cg_solve(L, h->cg, h->d_nfluid, h->cg_b, h->diag_tab, h->cg_down, h->cg_up, h->cg_flags, h->off, h->cg_tol,
             h->cg_maxit, h->cg_fp64, h->d_status);
}

void mark_hook(void* owner, int k)
{
    fs_handle* h = static_cast<fs_handle*>(owner);
    if (h->timing) cudaEventRecord(h->ev[k], h->stream);
}

// The handle's device arrays as the shared step code sees them.
StepState state(fs_handle* h)
{
    StepState st{};
    st.d = domain(h);
    st.front = &h->front;
    st.vfront = &h->vfront;
    for (int b = 0; b < 2; ++b) {
        st.u[b] = h->u[b];
        st.v[b] = h->v[b];
        st.vmx[b] = h->vmx[b];
        st.vmy[b] = h->vmy[b];
        st.sl_ok[b] = h->sl_ok[b];
    }
    st.u_prev = h->u_prev;
    st.v_prev = h->v_prev;
    st.u_diff = h->u_diff;
    st.v_diff = h->v_diff;
    st.labels = h->labels;
    st.solid = h->solid;
    st.fidx = h->fidx;
    st.cell_of = h->cell_of;
    st.counts32 = h->counts32;
    st.counts8 = h->counts8;
    for (int k = 0; k < 4; ++k) st.acc[k] = h->acc[k];
    for (int k = 0; k < 6; ++k) st.sl[k] = h->sl[k];
    st.px = h->px;
    st.py = h->py;
    st.pvx = h->pvx;
    st.pvy = h->pvy;
    st.yu = h->yu;
    st.xv = h->xv;
    st.sw = &h->sw;
    st.sw2 = &h->sw2;
    st.aux = h->aux;
    st.fork = h->fork;
    st.join = h->join;
    st.cg_b = h->cg_b;
    st.cg_down = h->cg_down;
    st.cg_up = h->cg_up;
    st.cg_flags = h->cg_flags;
    st.cg_x = h->cg.x;
    st.nfluid = h->d_nfluid;
    st.warn = h->d_warn;
    st.index_tmp = h->scan_tmp;
    st.n_ext = h->n_ext;
    st.solve = solve_hook;
    st.mark = mark_hook;
    st.owner = h;
    return st;
}

int run_step(fs_handle* h, int method, float dt)
{
    StepState st = state(h);
    enqueue_step(h->L(), st, method, dt);
    if (h->mg_error != cudaSuccess) {
        cudaGetLastError();
        const cudaError_t e = h->mg_error;
        h->mg_error = cudaSuccess;
        return cuda_fail(h, e, "multigrid pressure solve");
    }
    return FS_OK;
}

int check_launch(fs_handle* h, const char* what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, what);
    return FS_OK;
}

// FluidSolver::validate (src/FluidSolver.cpp:89-97) against the solver's pool,
// whose copy constructor keeps delta_x for delta_y (src/FluidSolver.cpp:56-62).
bool validate(const fs_handle* h) { return std::fabs(h->g.dy - h->g.pdy) < 0.0000001; }

const char* kValidateMessage =
    "Memory pool and fluid domain does not match. Initialize the fluid solver with a memory pool corresponding "
    "to the right fluid domain!";

void destroy_all(fs_handle* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    clear_graphs(h);
    void* ptrs[] = {h->level_set, h->level_set_tmp, h->u[0], h->u[1], h->v[0], h->v[1], h->u_prev, h->v_prev, h->u_diff, h->v_diff, h->labels,
                    h->solid, h->vmx[0], h->vmx[1], h->vmy[0], h->vmy[1], h->fidx, h->cell_of, h->counts32,
                    h->counts8, h->acc[0], h->acc[1], h->acc[2], h->acc[3], h->grid_tmp, h->sl[0], h->sl[1],
                    h->sl[2], h->sl[3], h->sl[4], h->sl[5], h->sl_ok[0], h->sl_ok[1], h->px, h->py, h->pvx,
                    h->pvy, h->yu, h->xv, h->staging, h->cg.x, h->cg.r, h->cg.z,
                    h->cg.p, h->cg.q, h->cg.partials, h->cg.barrier, h->cg.result, h->cg.route, h->cg_b, h->cg_down, h->cg_up,
                    h->cg_flags, h->d_nfluid, h->d_status, h->d_warn, h->scan_tmp};
    for (void* p : ptrs) cudaFree(p);
    splat_free(h->sw);
    splat_free(h->sw2);
    if (h->aux) {
        cudaStreamSynchronize(h->aux);
        cudaStreamDestroy(h->aux);
    }
    for (cudaEvent_t e : {h->fork, h->join})
        if (e) cudaEventDestroy(e);
    mg_destroy(h->mg);
    cudaFree(h->mg_b);
    for (DevSource& src : h->sources) {
        cudaFree(src.d_xs);
        cudaFree(src.d_ys);
    }
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int device_status(fs_handle* h)
{
    unsigned st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, h->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
    if (st & ST_TIMEOUT) {
        // Every solve clears the barrier counter before it starts and writes
        // its partials before reading them, so only the status word is reset.
        cudaMemsetAsync(h->d_status, 0, sizeof(unsigned), h->stream);
        cudaStreamSynchronize(h->stream);
        return fail(h, FS_ERR_TIMEOUT, "a device-side wait of the CG kernel timed out");
    }
    if (st & ST_TOO_LARGE) return fail(h, FS_ERR_TOO_LARGE, "too many fluid cells for the CG kernel");
    if (st & ST_INTERNAL) return fail(h, FS_ERR_INTERNAL, "internal consistency check failed on the device");
    return FS_OK;
}

template <class T>
int copy_out(fs_handle* h, T* host, const T* dev, size_t count)
{
    if (!host) return fail(h, FS_ERR_INVALID_ARGUMENT, "null output pointer");
    cudaError_t e = cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "copy to host");
    return FS_OK;
}

template <class T>
int copy_in(fs_handle* h, T* dev, const T* host, size_t count)
{
    if (!host) return fail(h, FS_ERR_INVALID_ARGUMENT, "null input pointer");
    cudaError_t e = cudaMemcpyAsync(dev, host, count * sizeof(T), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "copy to device");
    clear_graphs(h);  // a step graph never depends on data, but keep capture state simple
    return FS_OK;
}

float* grid_ptr(fs_handle* h, int which)
{
    switch (which) {
        case FS_U_FRONT: return UF(h);
        case FS_V_FRONT: return VF(h);
        case FS_U_BACK: return UB(h);
        case FS_V_BACK: return VB(h);
        case FS_U_PREV: return h->u_prev;
        case FS_V_PREV: return h->v_prev;
        case FS_U_DIFF: return h->u_diff;
        case FS_V_DIFF: return h->v_diff;
        default: return nullptr;
    }
}

}  // namespace

extern "C" {

void fs_config_init(fs_config* c, int size_x, int size_y)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->size_x = size_x;
    c->size_y = size_y;
    c->length_x = (float)size_x;
    c->length_y = (float)size_y;
    c->density = 1.0f;
    c->pic_ratio = 0.0f;
    c->gravity_x = 0.0f;
    c->gravity_y = (float)-9.82;
    c->cg_max_iterations = 100;
    c->cg_tolerance = 1.1920928955078125e-07;  // FLT_EPSILON
    c->extension_iterations = 2;
    c->device = 0;
}

const char* fs_last_error(const fs_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int fs_create(const fs_config* cfg, fs_handle** out)
{
    g_create_error.clear();
    if (!cfg || !out) {
        g_create_error = "null argument";
        return FS_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (cfg->size_x < 1 || cfg->size_y < 1 || !(cfg->length_x > 0) || !(cfg->length_y > 0) ||
        !std::isfinite(cfg->length_x) || !std::isfinite(cfg->length_y)) {
        g_create_error = "invalid grid size or length";
        return FS_ERR_INVALID_ARGUMENT;
    }
    const int64_t ncell = (int64_t)cfg->size_x * cfg->size_y;
    if (ncell > (int64_t)4096 * 4096 || cfg->size_x > (1 << 20) || cfg->size_y > (1 << 20)) {
        g_create_error = "grid larger than 16777216 cells";
        return FS_ERR_TOO_LARGE;
    }
    fs_handle* h = new fs_handle();
    h->cfg = *cfg;
    h->device = cfg->device;
    h->ncell = ncell;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        delete h;
        return FS_ERR_CUDA;
    }
    // GridInterface(size, size, length / size, ...) (src/FluidDomain.cpp:62, src/MacGrid.cpp:9)
    Geom& g = h->g;
    g.nx = cfg->size_x;
    g.ny = cfg->size_y;
    g.dx = cfg->length_x / (float)cfg->size_x;
    g.dy = cfg->length_y / (float)cfg->size_y;
    g.lx = (float)g.nx * g.dx;
    g.ly = (float)g.ny * g.dy;
    g.pdx = g.dx;
    g.pdy = g.dx;  // FluidSolverMemoryPool copy keeps delta_x for delta_y (src/FluidSolver.cpp:56-62)
    h->pic = cfg->pic_ratio;  // stored as given (src/FluidDomain.cpp:64)
    h->gx = cfg->gravity_x;
    h->gy = cfg->gravity_y;
    h->cg_tol = cfg->cg_tolerance;
    h->cg_maxit = cfg->cg_max_iterations;
    h->cg_fp64 = cfg->cg_precision == FS_CG_DOUBLE ? 1 : cfg->cg_precision == FS_CG_DS ? 2 : 0;
    h->n_ext = cfg->extension_iterations;
    // Matrix coefficients through double pow() as in src/FluidSolver.cpp:381-410.
    const double dx2 = std::pow((double)g.dx, 2);
    h->off = (float)(1 / dx2);
    for (int n = 0; n < 5; ++n) h->diag_tab[n] = (float)(-n / dx2);

    const size_t N = (size_t)ncell;
    const int64_t max_chunks = (ncell + 1023) / 1024;
    bool ok = true;
    auto A = [&](cudaError_t r) {
        if (r != cudaSuccess && ok) {
            ok = false;
            e = r;
        }
    };
    A(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
    A(cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking));
    A(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
    A(cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming));
    for (int b = 0; b < 2; ++b) {
        A(dalloc(&h->u[b], N));
        A(dalloc(&h->v[b], N));
        A(dalloc(&h->vmx[b], N));
        A(dalloc(&h->vmy[b], N));
    }
    A(dalloc(&h->u_prev, N));
    A(dalloc(&h->v_prev, N));
    A(dalloc(&h->u_diff, N));
    A(dalloc(&h->v_diff, N));
    A(dalloc(&h->labels, N));
    A(dalloc(&h->level_set, N));
    A(dalloc(&h->level_set_tmp, N));
    A(dalloc(&h->fidx, N));
    A(dalloc(&h->cell_of, N));
    A(dalloc(&h->counts32, N));
    A(dalloc(&h->counts8, N));
    for (int k = 0; k < 4; ++k) A(dalloc(&h->acc[k], N));
    A(dalloc(&h->grid_tmp, N));
    // The CG kernel copies whole 1024-element chunks of its system arrays, so
    // they are allocated to the last chunk's end.
    const size_t NP = (size_t)max_chunks * 1024;
    A(dalloc(&h->cg.x, NP));
    A(dalloc(&h->cg.r, NP));
    A(dalloc(&h->cg.z, NP));
    A(dalloc(&h->cg.p, NP));
    A(dalloc(&h->cg.q, NP));
    A(dalloc(&h->cg.partials, (size_t)8 * max_chunks));
    A(dalloc(&h->cg.barrier, 1));
    A(dalloc(&h->cg.result, 1));
    A(dalloc(&h->cg.route, 2));
    A(dalloc(&h->cg_b, N));
    A(dalloc(&h->cg_down, NP));
    A(dalloc(&h->cg_up, NP));
    A(dalloc(&h->cg_flags, NP));
    A(dalloc(&h->d_nfluid, 1));
    A(dalloc(&h->d_status, 1));
    A(dalloc(&h->d_warn, 1));
    A(dalloc(&h->scan_tmp, scan_tmp_ints(ncell + 2)));
    for (auto& ev : h->ev) A(cudaEventCreate(&ev));
    h->cg.max_cells = ncell;
    if (h->cg.partials) h->cg.groups = h->cg.partials + 4 * max_chunks;  // the second half of partials
    if (ok && cg_prepare(h->cg, h->device) != 0) {
        ok = false;
        e = cudaErrorInvalidConfiguration;
    }
    if (ok) A(ensure_splat_capacity(h, ncell));
    if (ok) {
        // Zero-initialised state, as the reference's Grid<T> ctor (include/Grid.h:129-139).
        for (int b = 0; b < 2; ++b) {
            A(cudaMemsetAsync(h->u[b], 0, N * 4, h->stream));
            A(cudaMemsetAsync(h->v[b], 0, N * 4, h->stream));
            A(cudaMemsetAsync(h->vmx[b], 0, N, h->stream));
            A(cudaMemsetAsync(h->vmy[b], 0, N, h->stream));
        }
        for (float* p : {h->u_prev, h->v_prev, h->u_diff, h->v_diff, h->cg.x, h->level_set})
            A(cudaMemsetAsync(p, 0, N * 4, h->stream));
        A(cudaMemsetAsync(h->fidx, 0, N * 4, h->stream));
        A(cudaMemsetAsync(h->counts8, 0, N, h->stream));
        A(cudaMemsetAsync(h->d_nfluid, 0, 4, h->stream));
        A(cudaMemsetAsync(h->d_status, 0, 4, h->stream));
        A(cudaMemsetAsync(h->d_warn, 0, 4, h->stream));
        A(cudaMemsetAsync(h->cg.result, 0, sizeof(CgResult), h->stream));
        A(cudaMemsetAsync(h->cg.partials, 0, sizeof(double) * 8 * (size_t)max_chunks, h->stream));
        A(cudaMemsetAsync(h->cg.barrier, 0, sizeof(unsigned), h->stream));
        labels_clear(h->L(), domain(h), h->labels);  // MacGrid ctor -> clearCellTypeBuffer (src/MacGrid.cpp:24)
        A(cudaGetLastError());
        A(cudaStreamSynchronize(h->stream));
    }
    if (!ok) {
        g_create_error = std::string("fs_create: ") + cudaGetErrorString(e);
        const int code = e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA;
        destroy_all(h);
        return code;
    }
    *out = h;
    return FS_OK;
}

int fs_destroy(fs_handle* h)
{
    destroy_all(h);
    return FS_OK;
}

int fs_set_pic_ratio(fs_handle* h, float r)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    // FluidDomain::setPicRatio (src/FluidDomain.cpp:99-102): CLAMP(pic_ratio, 0, 1)
    const float t = r < 0.0f ? 0.0f : r;
    const float v = t > 1.0f ? 1.0f : t;
    if (float_bits(v) != float_bits(h->pic)) clear_graphs(h);
    h->pic = v;
    return FS_OK;
}

int fs_set_gravity(fs_handle* h, float gx, float gy)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    if (float_bits(gx) != float_bits(h->gx) || float_bits(gy) != float_bits(h->gy)) clear_graphs(h);
    h->gx = gx;
    h->gy = gy;
    return FS_OK;
}

int fs_set_cg(fs_handle* h, double tol, int maxit)
{
    if (!h || !(tol >= 0) || maxit < 0) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "invalid CG settings") : 1;
    if (tol != h->cg_tol || maxit != h->cg_maxit) clear_graphs(h);
    h->cg_tol = tol;
    h->cg_maxit = maxit;
    return FS_OK;
}

int fs_set_cg_precision(fs_handle* h, int precision)
{
    if (!h || (precision != FS_CG_FLOAT && precision != FS_CG_DOUBLE && precision != FS_CG_DS))
        return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "unknown CG precision") : FS_ERR_INVALID_ARGUMENT;
    const int fp64 = precision == FS_CG_DOUBLE ? 1 : precision == FS_CG_DS ? 2 : 0;
    if (fp64 != h->cg_fp64) clear_graphs(h);
    h->cg_fp64 = fp64;
    return FS_OK;
}

int fs_set_pressure_solver(fs_handle* h, int solver)
{
    if (!h || (solver != FS_SOLVER_JACOBI_PCG && solver != FS_SOLVER_MGPCG))
        return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "unknown pressure solver") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    if (solver == FS_SOLVER_MGPCG && !h->mg) {
        if (mg_create(&h->mg, h->g.nx, h->g.ny, h->g.dx, h->device) != 0)
            return fail(h, FS_ERR_OUT_OF_MEMORY, "multigrid levels");
        const cudaError_t e = dalloc(&h->mg_b, (size_t)h->ncell);
        if (e != cudaSuccess) return cuda_fail(h, e, "multigrid right-hand side");
    }
    if (solver != h->solver) clear_graphs(h);
    h->solver = solver;
    return FS_OK;
}

int fs_set_extension_iterations(fs_handle* h, int n)
{
    if (!h || n < 0) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "negative extension iterations") : 1;
    if (n != h->n_ext) clear_graphs(h);
    h->n_ext = n;
    return FS_OK;
}

int fs_set_solid_mask(fs_handle* h, const uint8_t* mask)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    clear_graphs(h);
    if (!mask) {
        cudaStreamSynchronize(h->stream);
        cudaFree(h->solid);
        h->solid = nullptr;
        return FS_OK;
    }
    if (!h->solid) {
        cudaError_t e = dalloc(&h->solid, (size_t)h->ncell);
        if (e != cudaSuccess) return cuda_fail(h, e, "solid mask");
    }
    return copy_in(h, h->solid, mask, (size_t)h->ncell);
}

int fs_set_particles(fs_handle* h, const float* xyuv, int64_t n)
{
    if (!h || n < 0 || (n > 0 && !xyuv)) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "invalid particles") : 1;
    if (n > (int64_t)INT32_MAX) return fail(h, FS_ERR_TOO_LARGE, "more than 2^31-1 particles");
    cudaSetDevice(h->device);
    cudaError_t e = ensure_particle_capacity(h, n);
    if (e != cudaSuccess) return cuda_fail(h, e, "particle storage");
    if (n > 0) {
        e = cudaMemcpyAsync(h->staging, xyuv, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "particle upload");
        aos_to_soa(h->L(), h->staging, n, h->px, h->py, h->pvx, h->pvy);
    }
    if (n != h->n_part) clear_graphs(h);
    h->n_part = n;
    return check_launch(h, "particle upload");
}

int fs_set_particles_device(fs_handle* h, const float* d_xyuv, int64_t n)
{
    if (!h || n < 0 || (n > 0 && !d_xyuv)) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "invalid particles") : 1;
    if (((uintptr_t)d_xyuv & 15u) != 0) return fail(h, FS_ERR_INVALID_ARGUMENT, "device particle array not 16-byte aligned");
    if (n > (int64_t)INT32_MAX) return fail(h, FS_ERR_TOO_LARGE, "more than 2^31-1 particles");
    cudaSetDevice(h->device);
    cudaError_t e = ensure_particle_capacity(h, n);
    if (e != cudaSuccess) return cuda_fail(h, e, "particle storage");
    if (n > 0) aos_to_soa(h->L(), d_xyuv, n, h->px, h->py, h->pvx, h->pvy);
    if (n != h->n_part) clear_graphs(h);
    h->n_part = n;
    return check_launch(h, "particle upload");
}

int fs_add_particles(fs_handle* h, const float* xyuv, int64_t n)
{
    if (!h || n < 0 || (n > 0 && !xyuv)) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "invalid particles") : 1;
    if (n == 0) return FS_OK;
    const int64_t total = h->n_part + n;
    if (total > (int64_t)INT32_MAX) return fail(h, FS_ERR_TOO_LARGE, "more than 2^31-1 particles");
    cudaSetDevice(h->device);
    cudaError_t e = ensure_particle_capacity(h, total);
    if (e != cudaSuccess) return cuda_fail(h, e, "particle storage");
    e = cudaMemcpyAsync(h->staging, xyuv, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "particle upload");
    const int64_t o = h->n_part;
    aos_to_soa(h->L(), h->staging, n, h->px + o, h->py + o, h->pvx + o, h->pvy + o);
    h->n_part = total;
    clear_graphs(h);
    return check_launch(h, "particle upload");
}

int fs_num_particles(fs_handle* h, int64_t* n)
{
    if (!h || !n) return FS_ERR_INVALID_ARGUMENT;
    *n = h->n_part;
    return FS_OK;
}

int fs_get_particles(fs_handle* h, float* xyuv, int64_t n)
{
    if (!h || n != h->n_part) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "particle count mismatch") : 1;
    if (n == 0) return FS_OK;
    cudaSetDevice(h->device);
    soa_to_aos(h->L(), h->px, h->py, h->pvx, h->pvy, n, h->staging);
    const int rc = check_launch(h, "particle download");
    if (rc) return rc;
    return copy_out(h, xyuv, h->staging, (size_t)n * 4);
}

int fs_get_particles_device(fs_handle* h, float* d_xyuv, int64_t n)
{
    if (!h || n != h->n_part || (n > 0 && !d_xyuv)) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "particle count mismatch") : 1;
    if (((uintptr_t)d_xyuv & 15u) != 0) return fail(h, FS_ERR_INVALID_ARGUMENT, "device particle array not 16-byte aligned");
    if (n == 0) return FS_OK;
    cudaSetDevice(h->device);
    soa_to_aos(h->L(), h->px, h->py, h->pvx, h->pvy, n, d_xyuv);
    return check_launch(h, "particle download");
}

int fs_get_grid(fs_handle* h, int which, float* out)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    float* p = grid_ptr(h, which);
    if (!p) return fail(h, FS_ERR_INVALID_ARGUMENT, "unknown grid");
    cudaSetDevice(h->device);
    return copy_out(h, out, p, (size_t)h->ncell);
}

int fs_set_grid(fs_handle* h, int which, const float* in)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    float* p = grid_ptr(h, which);
    if (!p) return fail(h, FS_ERR_INVALID_ARGUMENT, "unknown grid");
    cudaSetDevice(h->device);
    return copy_in(h, p, in, (size_t)h->ncell);
}

int fs_get_labels(fs_handle* h, uint8_t* out)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return copy_out(h, out, h->labels, (size_t)h->ncell);
}

int fs_set_labels(fs_handle* h, const uint8_t* in)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return copy_in(h, h->labels, in, (size_t)h->ncell);
}

int fs_get_fluid_indices(fs_handle* h, int32_t* out)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return copy_out(h, out, h->fidx, (size_t)h->ncell);
}

int fs_get_particle_counts(fs_handle* h, uint8_t* out)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return copy_out(h, out, h->counts8, (size_t)h->ncell);
}

int fs_get_pressure(fs_handle* h, float* out)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    pressure_to_grid(h->L(), domain(h), h->fidx, h->d_nfluid, h->cg.x, h->grid_tmp);
    const int rc = check_launch(h, "pressure");
    if (rc) return rc;
    return copy_out(h, out, h->grid_tmp, (size_t)h->ncell);
}

int fs_phase(fs_handle* h, int ph, float dt)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    if (ph < FS_PH_CLASSIFY || ph > FS_PH_SWAP) return fail(h, FS_ERR_INVALID_ARGUMENT, "unknown phase");
    cudaSetDevice(h->device);
    if (ph == FS_PH_SL_VELOCITY) {
        cudaError_t e = ensure_sl_scratch(h);
        if (e != cudaSuccess) return cuda_fail(h, e, "semi-Lagrangian scratch");
    }
    StepState st = state(h);
    st.mark = nullptr;
    enqueue_phase(h->L(), st, ph, dt);
    return check_launch(h, "phase");
}

int fs_step(fs_handle* h, int method, float dt)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    if (method < FS_STEP_SEMI_LAGRANGIAN || method > FS_STEP_PICFLIP)
        return fail(h, FS_ERR_INVALID_ARGUMENT, "unknown step method");
    if (!validate(h)) return fail(h, FS_ERR_VALIDATE, kValidateMessage);
    cudaSetDevice(h->device);
    if (method == FS_STEP_SEMI_LAGRANGIAN) {
        cudaError_t e = ensure_sl_scratch(h);
        if (e != cudaSuccess) return cuda_fail(h, e, "semi-Lagrangian scratch");
    }
    h->timed_valid = h->timing;
    // per-phase events are recorded by direct launches; the multigrid solve polls its flag from the host
    if (!h->graphs || h->timing || h->solver == FS_SOLVER_MGPCG) {
        const int rc = run_step(h, method, dt);
        return rc ? rc : check_launch(h, "step");
    }
    const uint32_t db = float_bits(dt);
    for (auto& ge : h->graph_cache) {
        if (ge.method == method && ge.dt_bits == db && ge.front_in == h->front && ge.vfront_in == h->vfront &&
            ge.n_part == h->n_part && ge.timing == h->timing) {
            cudaError_t e = cudaGraphLaunch(ge.exec, h->stream);
            if (e != cudaSuccess) return cuda_fail(h, e, "graph launch");
            h->front = ge.front_out;
            h->vfront = ge.vfront_out;
            h->launches += ge.kernels;
            return FS_OK;
        }
    }
    GraphEntry ge{};
    ge.method = method;
    ge.dt_bits = db;
    ge.front_in = h->front;
    ge.vfront_in = h->vfront;
    ge.n_part = h->n_part;
    ge.timing = h->timing;  // event-record nodes of the per-phase timers are part of the graph
    const int64_t l0 = h->launches;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(h, e, "begin capture");
    run_step(h, method, dt);
    cudaError_t e_launch = cudaGetLastError();
    e = cudaStreamEndCapture(h->stream, &graph);
    ge.front_out = h->front;
    ge.vfront_out = h->vfront;
    ge.kernels = h->launches - l0;
    h->launches = l0;
    if (e != cudaSuccess || e_launch != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        // Fall back to direct launches for this handle.
        h->graphs = false;
        h->front = ge.front_in;
        h->vfront = ge.vfront_in;
        const int rc = run_step(h, method, dt);
        return rc ? rc : check_launch(h, "step");
    }
    e = cudaGraphInstantiate(&ge.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        h->graphs = false;
        h->front = ge.front_in;
        h->vfront = ge.vfront_in;
        const int rc = run_step(h, method, dt);
        return rc ? rc : check_launch(h, "step");
    }
    if (h->graph_cache.size() >= 8) {  // particle counts that changed (fluid sources) leave unused graphs
        cudaGraphExecDestroy(h->graph_cache.front().exec);
        h->graph_cache.erase(h->graph_cache.begin());
    }
    h->graph_cache.push_back(ge);
    e = cudaGraphLaunch(ge.exec, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "graph launch");
    h->launches += ge.kernels;
    return FS_OK;
}

int fs_add_fluid_source(fs_handle* h, float x_min, float x_max, float y_min, float y_max, float delta_x,
                        float delta_y, float x_velocity, float y_velocity, float time_step, int max_spawns)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    // the spawn lattice of FluidSource::update (src/FluidDomain.cpp:37-48):
    // increments delta / 2.5 rounded to float, loop variables accumulated in float
    const float x_incr = (float)(delta_x / 2.5);
    const float y_incr = (float)(delta_y / 2.5);
    constexpr size_t kMaxLattice = (size_t)1 << 26;
    std::vector<float> xs, ys;
    for (float x = x_min; x < x_max; x += x_incr) {
        xs.push_back(x);
        if (xs.size() > kMaxLattice)  // the reference would not stop (an increment too small to advance x)
            return fail(h, FS_ERR_INVALID_ARGUMENT, "fluid source lattice does not end in x");
    }
    for (float y = y_min; y < y_max; y += y_incr) {
        ys.push_back(y);
        if (ys.size() > kMaxLattice) return fail(h, FS_ERR_INVALID_ARGUMENT, "fluid source lattice does not end in y");
    }
    if (!xs.empty() && !ys.empty() && xs.size() * ys.size() > (size_t)INT32_MAX)
        return fail(h, FS_ERR_TOO_LARGE, "fluid source spawns more than 2^31-1 particles");
    cudaSetDevice(h->device);
    DevSource src{};
    src.vx = x_velocity;
    src.vy = y_velocity;
    src.time_step = time_step;
    src.time_since_last = 0.0f;
    src.max_spawns = max_spawns;
    src.n_spawns = 0;
    src.nx = (int)xs.size();
    src.ny = (int)ys.size();
    cudaError_t e = dalloc(&src.d_xs, xs.size());
    if (e == cudaSuccess) e = dalloc(&src.d_ys, ys.size());
    if (e == cudaSuccess && !xs.empty())
        e = cudaMemcpyAsync(src.d_xs, xs.data(), 4 * xs.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && !ys.empty())
        e = cudaMemcpyAsync(src.d_ys, ys.data(), 4 * ys.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        cudaFree(src.d_xs);
        cudaFree(src.d_ys);
        return cuda_fail(h, e, "fluid source");
    }
    h->sources.push_back(src);
    return FS_OK;
}

int fs_update(fs_handle* h, float dt)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    for (DevSource& src : h->sources) {
        // FluidSource::update (src/FluidDomain.cpp:29-52)
        if (src.max_spawns != -1 && src.n_spawns >= src.max_spawns) continue;
        if (src.time_since_last >= src.time_step) {
            const int64_t k = (int64_t)src.nx * src.ny;
            if (k > 0) {
                const int64_t total = h->n_part + k;
                if (total > (int64_t)INT32_MAX) return fail(h, FS_ERR_TOO_LARGE, "more than 2^31-1 particles");
                const cudaError_t e = ensure_particle_capacity(h, total);
                if (e != cudaSuccess) return cuda_fail(h, e, "particle storage");
                spawn_lattice(h->L(), src.d_xs, src.nx, src.d_ys, src.ny, src.vx, src.vy, h->px + h->n_part,
                              h->py + h->n_part, h->pvx + h->n_part, h->pvy + h->n_part);
                h->n_part = total;
                const int rc = check_launch(h, "fluid source");
                if (rc) return rc;
            }
            src.time_since_last = 0;
            src.n_spawns++;
        }
        src.time_since_last += dt;
    }
    return FS_OK;
}

int fs_clear_fluid_sources(fs_handle* h)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    for (DevSource& src : h->sources) {
        cudaFree(src.d_xs);
        cudaFree(src.d_ys);
    }
    h->sources.clear();
    return FS_OK;
}

int fs_set_fluid_source_state(fs_handle* h, int index, float time_since_last, int n_spawns)
{
    if (!h || index < 0 || index >= (int)h->sources.size())
        return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "no such fluid source") : FS_ERR_INVALID_ARGUMENT;
    h->sources[index].time_since_last = time_since_last;
    h->sources[index].n_spawns = n_spawns;
    return FS_OK;
}

int fs_num_fluid_sources(fs_handle* h, int* n)
{
    if (!h || !n) return FS_ERR_INVALID_ARGUMENT;
    *n = (int)h->sources.size();
    return FS_OK;
}

int fs_reset_particles(fs_handle* h)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    h->n_part = 0;  // FluidDomain::resetParticleSet (src/FluidDomain.cpp:94-97)
    return FS_OK;
}

}  // extern "C"

namespace {

// The cell arrays a snapshot holds: {pointer, bytes per cell}.
std::vector<std::pair<void*, size_t>> snapshot_cells(fs_handle* h)
{
    return {{h->u[0], 4}, {h->u[1], 4}, {h->v[0], 4},   {h->v[1], 4},   {h->u_prev, 4},  {h->v_prev, 4},
            {h->u_diff, 4}, {h->v_diff, 4}, {h->labels, 1}, {h->vmx[0], 1}, {h->vmx[1], 1}, {h->vmy[0], 1},
            {h->vmy[1], 1}, {h->fidx, 4},  {h->counts8, 1}, {h->cg.x, 4},   {h->level_set, 4}};
}

cudaError_t copy_snapshot(fs_handle* h, fs_saved_state* sn, bool save)
{
    cudaError_t e = cudaSuccess;
    size_t off = 0;
    for (auto& a : snapshot_cells(h)) {
        const size_t bytes = a.second * (size_t)h->ncell;
        if (e == cudaSuccess)
            e = save ? cudaMemcpyAsync(sn->cells + off, a.first, bytes, cudaMemcpyDeviceToDevice, h->stream)
                     : cudaMemcpyAsync(a.first, sn->cells + off, bytes, cudaMemcpyDeviceToDevice, h->stream);
        off += (bytes + 255) / 256 * 256;
    }
    float* P[4] = {h->px, h->py, h->pvx, h->pvy};
    const size_t pb = 4 * (size_t)sn->n_part;
    for (int k = 0; k < 4 && e == cudaSuccess && pb; ++k)
        e = save ? cudaMemcpyAsync(sn->parts + k * sn->n_part, P[k], pb, cudaMemcpyDeviceToDevice, h->stream)
                 : cudaMemcpyAsync(P[k], sn->parts + k * sn->n_part, pb, cudaMemcpyDeviceToDevice, h->stream);
    struct M
    {
        void* p;
        size_t bytes;
    } misc[3] = {{h->d_nfluid, 4}, {h->cg.result, sizeof(CgResult)}, {h->d_warn, 4}};
    off = 0;
    for (const M& m : misc) {
        if (e == cudaSuccess)
            e = save ? cudaMemcpyAsync(sn->misc + off, m.p, m.bytes, cudaMemcpyDeviceToDevice, h->stream)
                     : cudaMemcpyAsync(m.p, sn->misc + off, m.bytes, cudaMemcpyDeviceToDevice, h->stream);
        off += 64;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e;
}

}  // namespace

extern "C" {

int fs_snapshot(fs_handle* h, fs_saved_state** out)
{
    if (!h || !out) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "null snapshot") : FS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cudaSetDevice(h->device);
    fs_saved_state* sn = new fs_saved_state();
    sn->owner = h;
    sn->ncell = h->ncell;
    sn->n_part = h->n_part;
    sn->front = h->front;
    sn->vfront = h->vfront;
    size_t cbytes = 0;
    for (auto& a : snapshot_cells(h)) cbytes += (a.second * (size_t)h->ncell + 255) / 256 * 256;
    cudaError_t e = cudaMalloc(&sn->cells, cbytes);
    if (e == cudaSuccess) e = cudaMalloc(&sn->parts, 16 * (size_t)std::max<int64_t>(sn->n_part, 1));
    if (e == cudaSuccess) e = cudaMalloc(&sn->misc, 3 * 64);
    if (e == cudaSuccess) e = copy_snapshot(h, sn, true);
    if (e != cudaSuccess) {
        fs_snapshot_destroy(sn);
        return cuda_fail(h, e, "snapshot");
    }
    for (const DevSource& src : h->sources) {
        sn->src_time.push_back(src.time_since_last);
        sn->src_spawns.push_back(src.n_spawns);
    }
    *out = sn;
    return FS_OK;
}

int fs_restore(fs_handle* h, const fs_saved_state* sn)
{
    if (!h || !sn) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "null snapshot") : FS_ERR_INVALID_ARGUMENT;
    if (sn->owner != h) return fail(h, FS_ERR_INVALID_ARGUMENT, "snapshot of another handle");
    if (sn->src_time.size() != h->sources.size())
        return fail(h, FS_ERR_INVALID_ARGUMENT, "fluid sources were added or cleared since the snapshot");
    cudaSetDevice(h->device);
    cudaError_t e = ensure_particle_capacity(h, sn->n_part);
    if (e != cudaSuccess) return cuda_fail(h, e, "particle storage");
    if (sn->n_part != h->n_part) clear_graphs(h);
    h->n_part = sn->n_part;
    h->front = sn->front;
    h->vfront = sn->vfront;
    e = copy_snapshot(h, const_cast<fs_saved_state*>(sn), false);
    if (e != cudaSuccess) return cuda_fail(h, e, "restore");
    for (size_t k = 0; k < h->sources.size(); ++k) {
        h->sources[k].time_since_last = sn->src_time[k];
        h->sources[k].n_spawns = sn->src_spawns[k];
    }
    return FS_OK;
}

int fs_snapshot_destroy(fs_saved_state* sn)
{
    if (!sn) return FS_OK;
    cudaFree(sn->cells);
    cudaFree(sn->parts);
    cudaFree(sn->misc);
    delete sn;
    return FS_OK;
}

int fs_get_level_set(fs_handle* h, float* out)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return copy_out(h, out, h->level_set, (size_t)h->ncell);
}

int fs_set_level_set(fs_handle* h, const float* in)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return copy_in(h, h->level_set, in, (size_t)h->ncell);
}

int fs_advect_level_set(fs_handle* h, float dt)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    advect_level_set(h->L(), domain(h), h->level_set, UF(h), VF(h), dt, h->level_set_tmp);
    std::swap(h->level_set, h->level_set_tmp);  // _level_set = std::move(new_level_set)
    clear_graphs(h);                             // no step graph reads the level set, but keep pointers current
    return check_launch(h, "level set advection");
}

int fs_classify_level_set(fs_handle* h)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    classify_level_set(h->L(), domain(h), h->level_set, h->labels, h->solid);
    return check_launch(h, "level set classification");
}

int fs_render(fs_handle* h, fs_canvas* c, int what, const float* area)
{
    if (!h || !c || !area) return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "null render argument") : FS_ERR_INVALID_ARGUMENT;
    if (c->device != h->device) return fail(h, FS_ERR_INVALID_ARGUMENT, "canvas on another device");
    cudaSetDevice(h->device);
    const Launch L = h->L();
    const View v = render_view(area, c->width, c->height);
    cudaError_t e = cudaSuccess;
    switch (what) {
        case FS_RENDER_CLEAR: render_clear(L, c); break;
        case FS_RENDER_CELLS: render_cells(L, c, v, h->g, h->labels, nullptr); break;
        case FS_RENDER_LEVEL_SET: render_cells(L, c, v, h->g, h->labels, h->level_set); break;
        case FS_RENDER_VELOCITIES: render_velocities(L, c, v, h->g, UF(h), VF(h)); break;
        case FS_RENDER_PARTICLES: render_particles(L, c, v, h->px, h->py, h->n_part); break;
        case FS_RENDER_METABALLS: e = render_metaballs(L, c, v, h->px, h->py, h->n_part); break;
        default: return fail(h, FS_ERR_INVALID_ARGUMENT, "unknown render pass");
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);  // the canvas is read from any stream
    if (e != cudaSuccess) return cuda_fail(h, e, "render");
    return FS_OK;
}

int fs_debug_set_cg_barrier_fault(fs_handle* h, int missing_arrivals, double wait_limit_seconds)
{
    if (!h || missing_arrivals < 0 || !(wait_limit_seconds > 0) || wait_limit_seconds > 10.0)
        return h ? fail(h, FS_ERR_INVALID_ARGUMENT, "invalid barrier fault settings") : FS_ERR_INVALID_ARGUMENT;
    h->cg.missing_arrivals = (unsigned)missing_arrivals;
    h->cg.wait_ns = (uint64_t)(wait_limit_seconds * 1e9);
    clear_graphs(h);  // both are arguments of the recorded CG launch
    return FS_OK;
}

int fs_synchronize(fs_handle* h)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    return device_status(h);
}

int fs_get_stats(fs_handle* h, fs_step_stats* out)
{
    if (!h || !out) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    const int rc = device_status(h);
    std::memset(out, 0, sizeof(*out));
    CgResult r{};
    int32_t nf = 0;
    unsigned warn = 0;
    cudaMemcpy(&r, h->cg.result, sizeof(r), cudaMemcpyDeviceToHost);
    cudaMemcpy(&nf, h->d_nfluid, sizeof(nf), cudaMemcpyDeviceToHost);
    cudaMemcpy(&warn, h->d_warn, sizeof(warn), cudaMemcpyDeviceToHost);
    cudaMemsetAsync(h->d_warn, 0, sizeof(unsigned), h->stream);
    out->cg_iterations = r.iterations;
    out->n_fluid = nf;
    out->cg_residual = r.bb > 0 ? std::sqrt(r.rr / r.bb) : 0.0;
    if (nf > 0 && r.bb > 0 && r.iterations >= h->cg_maxit && std::sqrt(r.rr / r.bb) >= h->cg_tol)
        warn |= FS_WARN_CG_NOT_CONVERGED;
    out->warnings = warn;
    if (h->timed_valid) {
        float total = 0.0f;
        for (int k = 0; k < FS_NUM_TIMED; ++k) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, h->ev[k], h->ev[k + 1]) == cudaSuccess) out->ms_phase[k] = ms;
            total += out->ms_phase[k];
        }
        out->ms_total = total;
    }
    cudaGetLastError();
    return rc;
}

int fs_set_timing(fs_handle* h, int enable)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    h->timing = enable != 0;
    return FS_OK;
}

int fs_set_graphs(fs_handle* h, int enable)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    h->graphs = enable != 0;
    if (!h->graphs) clear_graphs(h);
    return FS_OK;
}

void* fs_get_stream(fs_handle* h) { return h ? (void*)h->stream : nullptr; }

int fs_set_stream(fs_handle* h, void* stream)
{
    if (!h) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    clear_graphs(h);
    return FS_OK;
}

int64_t fs_kernel_launches(fs_handle* h) { return h ? h->launches : 0; }

}  // extern "C"
