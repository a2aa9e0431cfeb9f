// fs_pressure_solve_noalloc: the pressure solve of FluidSolver::pressureSolve
// (fluid indexing, divergence and matrix rows, Jacobi-PCG) for callers that
// cannot allocate device memory.
//
// Who needs it: applications that own every device byte themselves and
// forbid allocation once they are running -- a real-time frame loop where a
// cudaMalloc / cudaFree can block on device-wide synchronisation and miss a
// frame, or a plugin that lives inside a host application's fixed memory
// budget and is handed only its input and output buffers.  fs_create cannot
// serve them because every handle allocates its grids and scratch.
//
// How: all scratch (fluid indices, matrix rows, CG vectors, reduction
// partials, counters) lives in one file-scope static __device__ array,
// sized for NOALLOC_MAX_CELLS cells, that every GPU loading this library
// holds until the process exits.  Host code cannot use the array's name as
// a device address, so the first call on each device looks the address up
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call before any stream capture.  The cached address belongs to
// the device's context at that time: after cudaDeviceReset the process must
// not call this entry point on that device again.  Every call shares the
// array and finds the previous call's contents in it: the parts that must
// start at zero are cleared by each call, and calls whose work overlaps on
// the GPU (different streams, different threads) race on the array.
//
// Every call synchronises its stream and reads the device status word before
// it returns, so a device-side failure is reported by the call that met it
// and never left for a later call to clear.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "fs_internal.h"

namespace {

using namespace fs;

constexpr int64_t NOALLOC_MAX_CELLS = 16384;  // e.g. 128 x 128
constexpr int64_t NOALLOC_MAX_CHUNKS = (NOALLOC_MAX_CELLS + 1023) / 1024;
constexpr size_t ALIGN = 256;
constexpr size_t up_to(size_t n) { return (n + ALIGN - 1) / ALIGN * ALIGN; }

// Byte offsets of the scratch arrays.
constexpr size_t N = (size_t)NOALLOC_MAX_CELLS;
constexpr size_t OFF_FIDX = 0;
constexpr size_t OFF_CELL_OF = OFF_FIDX + up_to(4 * N);
constexpr size_t OFF_COUNTS32 = OFF_CELL_OF + up_to(4 * N);
constexpr size_t OFF_COUNTS8 = OFF_COUNTS32 + up_to(4 * N);
constexpr size_t OFF_B = OFF_COUNTS8 + up_to(N);
constexpr size_t OFF_DOWN = OFF_B + up_to(4 * N);
constexpr size_t OFF_UP = OFF_DOWN + up_to(4 * N);
constexpr size_t OFF_FLAGS = OFF_UP + up_to(4 * N);
constexpr size_t OFF_X = OFF_FLAGS + up_to(N);
constexpr size_t OFF_R = OFF_X + up_to(4 * N);
constexpr size_t OFF_Z = OFF_R + up_to(4 * N);
constexpr size_t OFF_P = OFF_Z + up_to(4 * N);
constexpr size_t OFF_Q = OFF_P + up_to(4 * N);
constexpr size_t OFF_PARTIALS = OFF_Q + up_to(4 * N);
constexpr size_t OFF_SCAN = OFF_PARTIALS + up_to(8 * 8 * (size_t)NOALLOC_MAX_CHUNKS);
constexpr size_t SCAN_INTS = 64;
static_assert(scan_tmp_ints(NOALLOC_MAX_CELLS + 2) <= SCAN_INTS, "the scan's tile sums fit their scratch");
constexpr size_t OFF_NFLUID = OFF_SCAN + up_to(4 * SCAN_INTS);
constexpr size_t OFF_STATUS = OFF_NFLUID + ALIGN;
constexpr size_t OFF_WARN = OFF_STATUS + ALIGN;
constexpr size_t OFF_BARRIER = OFF_WARN + ALIGN;
constexpr size_t OFF_RESULT = OFF_BARRIER + ALIGN;
constexpr size_t SCRATCH_BYTES = OFF_RESULT + up_to(sizeof(CgResult));

__device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
unsigned char* g_scratch[MAX_DEVICES] = {};
int g_cg_grid[MAX_DEVICES] = {};
int fail(int code, const std::string& msg)
{
    set_thread_error(msg.c_str());  // reported by fs_last_error(NULL)
    return code;
}

// Once per device, with that device current: the array's device address and
// the cooperative grid size of the CG kernel.
int setup(int dev, unsigned char** base, int* grid)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(FS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        CgWork w{};
        if (cg_prepare(w, dev) != 0) return fail(FS_ERR_CUDA, "CG kernel configuration failed");
        g_cg_grid[dev] = w.grid;
        g_scratch[dev] = static_cast<unsigned char*>(p);
    }
    *base = g_scratch[dev];
    *grid = g_cg_grid[dev];
    return FS_OK;
}

}  // namespace

extern "C" FS_API int fs_pressure_solve_noalloc(int size_x, int size_y, float length_x, float length_y,
                                                const uint8_t* labels, const float* u, const float* v,
                                                double cg_tolerance, int cg_max_iterations, int cg_precision,
                                                float* pressure, int* cg_iterations, double* cg_residual,
                                                void* stream)
{
    set_thread_error("");
    if (size_x < 1 || size_y < 1 || !(length_x > 0) || !(length_y > 0) || !labels || !u || !v || !pressure ||
        !(cg_tolerance >= 0) || cg_max_iterations < 0 || (cg_precision != FS_CG_FLOAT && cg_precision != FS_CG_DOUBLE))
        return fail(FS_ERR_INVALID_ARGUMENT, "invalid argument");
    const int64_t ncell = (int64_t)size_x * size_y;
    if (ncell > NOALLOC_MAX_CELLS) {
        char msg[160];
        std::snprintf(msg, sizeof(msg),
                      "grid of %lld cells exceeds the %lld-cell limit of the allocation-free pressure solve",
                      (long long)ncell, (long long)NOALLOC_MAX_CELLS);
        return fail(FS_ERR_TOO_LARGE, msg);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return fail(FS_ERR_CUDA, "no current CUDA device");
    unsigned char* base = nullptr;
    int grid = 0;
    int rc = setup(dev, &base, &grid);
    if (rc != FS_OK) return rc;

    int32_t* fidx = reinterpret_cast<int32_t*>(base + OFF_FIDX);
    int32_t* cell_of = reinterpret_cast<int32_t*>(base + OFF_CELL_OF);
    int32_t* counts32 = reinterpret_cast<int32_t*>(base + OFF_COUNTS32);
    uint8_t* counts8 = base + OFF_COUNTS8;
    float* b = reinterpret_cast<float*>(base + OFF_B);
    int32_t* down = reinterpret_cast<int32_t*>(base + OFF_DOWN);
    int32_t* up = reinterpret_cast<int32_t*>(base + OFF_UP);
    uint8_t* flags = base + OFF_FLAGS;
    int32_t* scan_tmp = reinterpret_cast<int32_t*>(base + OFF_SCAN);
    int32_t* nfluid = reinterpret_cast<int32_t*>(base + OFF_NFLUID);
    unsigned* status = reinterpret_cast<unsigned*>(base + OFF_STATUS);
    CgWork w{};
    w.x = reinterpret_cast<float*>(base + OFF_X);
    w.r = reinterpret_cast<float*>(base + OFF_R);
    w.z = reinterpret_cast<float*>(base + OFF_Z);
    w.p = reinterpret_cast<float*>(base + OFF_P);
    w.q = reinterpret_cast<float*>(base + OFF_Q);
    w.partials = reinterpret_cast<double*>(base + OFF_PARTIALS);
    w.barrier = reinterpret_cast<unsigned*>(base + OFF_BARRIER);
    w.result = reinterpret_cast<CgResult*>(base + OFF_RESULT);
    w.max_cells = NOALLOC_MAX_CELLS;
    w.grid = grid;

    // Same geometry and coefficients as fs_create (src/FluidDomain.cpp:62, src/FluidSolver.cpp:381-410).
    Geom g{};
    g.nx = size_x;
    g.ny = size_y;
    g.dx = length_x / (float)size_x;
    g.dy = length_y / (float)size_y;
    g.lx = (float)g.nx * g.dx;
    g.ly = (float)g.ny * g.dy;
    g.pdx = g.dx;
    g.pdy = g.dx;
    const double dx2 = std::pow((double)g.dx, 2);
    const float off = (float)(1 / dx2);
    float diag_tab[5];
    for (int n = 0; n < 5; ++n) diag_tab[n] = (float)(-n / dx2);

    const Launch L{static_cast<cudaStream_t>(stream), nullptr, 0};
    // State the previous call left behind: clear what is accumulated into.
    cudaMemsetAsync(counts32, 0, sizeof(int32_t) * (size_t)ncell, L.stream);
    cudaMemsetAsync(status, 0, sizeof(unsigned), L.stream);
    fluid_index(L, labels, ncell, fidx, cell_of, nfluid, scan_tmp);
    Seg sg{};
    sg.g = g;
    const Domain d = Domain::single(sg);
    assemble(L, d, labels, fidx, cell_of, nfluid, u, v, b, down, up, flags, counts32, counts8);
    cg_solve(L, w, nfluid, b, diag_tab, down, up, flags, off, cg_tolerance, cg_max_iterations,
             cg_precision == FS_CG_DOUBLE ? 1 : 0, status);
    pressure_to_grid(L, d, fidx, nfluid, w.x, pressure);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    // The status is read on every call: the next call clears it.
    CgResult res{};
    unsigned st = 0;
    cudaMemcpyAsync(&res, w.result, sizeof(res), cudaMemcpyDeviceToHost, L.stream);
    cudaMemcpyAsync(&st, status, sizeof(st), cudaMemcpyDeviceToHost, L.stream);
    e = cudaStreamSynchronize(L.stream);
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
    if (st & ST_TIMEOUT) return fail(FS_ERR_TIMEOUT, "a device-side wait of the CG kernel timed out");
    if (st & ST_TOO_LARGE) return fail(FS_ERR_TOO_LARGE, "too many fluid cells");
    if (st) return fail(FS_ERR_INTERNAL, "internal consistency check failed on the device");
    if (cg_iterations) *cg_iterations = res.iterations;
    if (cg_residual) *cg_residual = res.bb > 0 ? std::sqrt(res.rr / res.bb) : 0.0;
    return FS_OK;
}
