// C ABI of a batch of independent simulations (include/fsgpu.h, fs_batch_*):
// many FluidDomain + FluidSolver pairs of uneven grid sizes stepped together.
// Each phase of the step is one launch over the cells or particles of every
// simulation (fs_domain.cuh), and the pressure solves run as one thread-block
// cluster per simulation (k_cg_cluster), grouped into launch classes by
// cluster size and shared-memory footprint; the classes run concurrently on
// forked streams.  A whole step is captured once into a CUDA graph and
// replayed.  Every simulation's results are bit-identical to stepping it
// alone: the per-item arithmetic and the CG reduction tree are the same.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fs_step.h"

using namespace fs;

namespace {

thread_local std::string g_batch_error;

constexpr int MAX_CLASSES = 8;
constexpr int64_t BATCH_MAX_CELLS = (int64_t)16 * 1024 * 1024 - 4096;
constexpr int64_t BATCH_MAX_INTERIOR = 8 * 8 * 1024;  // 8 CTAs x 8 chunks of 1024 fluid cells

struct ClassPlan
{
    int K;      // chunks per CTA held in shared memory
    int C;      // CTAs per cluster
    int first;  // first entry of the class in the order table
    int count;  // simulations
};

struct BatchGraph
{
    int method;
    uint32_t dt_bits;
    int front_in, vfront_in, front_out, vfront_out;
    int plan;
    int64_t layout;
    int64_t kernels;
    cudaGraphExec_t exec;
};

int64_t round_up(int64_t n, int64_t m) { return (n + m - 1) / m * m; }

uint32_t float_bits(float f)
{
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

template <class T>
cudaError_t dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

}  // namespace

struct fs_batch
{
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux[MAX_CLASSES - 1] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[MAX_CLASSES - 1] = {};
    int n = 0;
    std::vector<fs_config> cfg;
    std::vector<Seg> seg;                     // host copy of the segment table
    std::vector<int64_t> cap;                 // particle capacity of each simulation (multiple of DOMAIN_TPB)
    std::vector<std::vector<float>> pending;  // particles set since the last layout (AoS)
    std::vector<char> has_pending;
    bool layout_dirty = false;
    int64_t layout_version = 0;
    int64_t cells = 0, parts = 0;

    Seg* d_seg = nullptr;
    int2* d_cblk = nullptr;
    int2* d_pblk = nullptr;
    unsigned ncblk = 0, npblk = 0;

    float* u[2] = {};
    float* v[2] = {};
    float *u_prev = nullptr, *v_prev = nullptr, *u_diff = nullptr, *v_diff = nullptr;
    uint8_t* labels = nullptr;
    uint8_t* solid = nullptr;
    uint8_t* vmx[2] = {};
    uint8_t* vmy[2] = {};
    int32_t *fidx = nullptr, *cell_of = nullptr, *counts32 = nullptr;
    uint8_t* counts8 = nullptr;
    float* acc[4] = {};
    float* grid_tmp = nullptr;
    float* sl[6] = {};
    uint8_t* sl_ok[2] = {};
    float* cg_b = nullptr;
    int32_t *cg_down = nullptr, *cg_up = nullptr;
    uint8_t* cg_flags = nullptr;
    float *cx = nullptr, *cr = nullptr, *cz = nullptr, *cp = nullptr, *cq = nullptr;

    float *px = nullptr, *py = nullptr, *pvx = nullptr, *pvy = nullptr, *yu = nullptr, *xv = nullptr;
    float* staging = nullptr;
    int64_t staging_cap = 0;
    SplatWork sw{};

    int32_t* nfluid = nullptr;
    unsigned* status = nullptr;
    unsigned* warn = nullptr;
    int32_t* index_tmp = nullptr;

    CgSystem* d_sys = nullptr;
    double* partials = nullptr;
    CgResult* results = nullptr;
    int32_t* d_order = nullptr;
    std::vector<ClassPlan> plan;
    std::vector<int> plan_chunks;  // chunks each simulation's cluster is sized for
    int plan_target = 8;
    bool counted = false;  // a step has counted every simulation's fluid cells

    int front = 0, vfront = 0;
    int n_ext = 2;
    int fp64 = 0;
    bool graphs = true;
    std::vector<BatchGraph> gcache;
    int64_t launches = 0;
    std::string err;

    Launch L() { return Launch{stream, &launches, 0}; }
};

namespace {

int fail(fs_batch* b, int code, const std::string& msg)
{
    if (b) b->err = msg;
    return code;
}

int cuda_fail(fs_batch* b, cudaError_t e, const char* what)
{
    return fail(b, e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

void clear_graphs(fs_batch* b)
{
    for (auto& g : b->gcache) cudaGraphExecDestroy(g.exec);
    b->gcache.clear();
}

int64_t interior(const Seg& s) { return (int64_t)std::max(0, s.g.nx - 2) * std::max(0, s.g.ny - 2); }

int max_chunks(const Seg& s) { return (int)std::max<int64_t>(1, (interior(s) + 1023) / 1024); }

// Cluster shape of each simulation for a target of `target` chunks per CTA:
// the smallest power-of-two cluster (<= 8) that keeps the chunks per CTA at or
// under the target, for the chunk count the simulation is planned for
// (plan_chunks); the shared-memory footprint is 4 chunks (two CTAs per SM) or
// 8 (one CTA per SM).  A simulation that later outgrows its cluster still
// solves correctly, from global memory.
int make_plan(fs_batch* b, int target)
{
    std::vector<std::vector<int>> groups(8);
    auto key = [](int K, int C) { return (K == 8 ? 4 : 0) + (C == 1 ? 0 : C == 2 ? 1 : C == 4 ? 2 : 3); };
    for (int s = 0; s < b->n; ++s) {
        const int ch = b->plan_chunks[s];
        int C = 1;
        while (C < 8 && (ch + C - 1) / C > target) C *= 2;
        const int per = (ch + C - 1) / C;
        const int K = per <= 4 ? 4 : 8;
        groups[key(K, C)].push_back(s);
    }
    std::vector<int32_t> order;
    std::vector<ClassPlan> plan;
    for (int g = 0; g < 8; ++g) {
        if (groups[g].empty()) continue;
        std::vector<int>& v = groups[g];
        std::stable_sort(v.begin(), v.end(), [&](int a, int c) { return b->plan_chunks[a] > b->plan_chunks[c]; });
        ClassPlan cp;
        cp.K = g >= 4 ? 8 : 4;
        cp.C = 1 << (g & 3);
        cp.first = (int)order.size();
        cp.count = (int)v.size();
        if (cg_cluster_capacity(cp.K, cp.C) < 1) {
            return fail(b, FS_ERR_CUDA,
                        "cluster shape of " + std::to_string(cp.C) + " CTAs x " + std::to_string(cp.K) +
                            " chunks cannot run on this device");
        }
        order.insert(order.end(), v.begin(), v.end());
        plan.push_back(cp);
    }
    const cudaError_t e =
        cudaMemcpyAsync(b->d_order, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "CG plan upload");
    b->plan = plan;
    b->plan_target = target;
    clear_graphs(b);
    return FS_OK;
}

// Plans clusters for the current fluid cells of every simulation plus a 25%
// margin (never more than its interior), as the tuner does.
int refresh_plan_chunks(fs_batch* b)
{
    std::vector<int32_t> nf(b->n);
    cudaError_t e = cudaMemcpyAsync(nf.data(), b->nfluid, sizeof(int32_t) * b->n, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "fluid counts");
    for (int s = 0; s < b->n; ++s) {
        const int64_t want = ((int64_t)nf[s] * 5 / 4 + 1023) / 1024;
        b->plan_chunks[s] = (int)std::max<int64_t>(1, std::min<int64_t>(want, max_chunks(b->seg[s])));
    }
    return FS_OK;
}

cudaError_t ensure_splat_capacity(fs_batch* b, int64_t items)
{
    if (items <= b->sw.cap_items) return cudaSuccess;
    clear_graphs(b);
    return splat_alloc(b->sw, items, b->cells);
}

// Lays out the particles of every simulation after sets: new capacities and
// offsets, existing particles moved, pending ones uploaded.
int flush_layout(fs_batch* b)
{
    if (!b->layout_dirty) return FS_OK;
    std::vector<int64_t> np(b->n), cap(b->n), po(b->n);
    int64_t total = 0;
    for (int s = 0; s < b->n; ++s) {
        np[s] = b->has_pending[s] ? (int64_t)b->pending[s].size() / 4 : b->seg[s].np;
        cap[s] = round_up(np[s], DOMAIN_TPB);
        po[s] = total;
        total += cap[s];
    }
    if (total > (int64_t)INT32_MAX) return fail(b, FS_ERR_TOO_LARGE, "more than 2^31-1 particles in the batch");
    float* na[6] = {};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = dalloc(&na[k], (size_t)total);
    int64_t stage = 0;
    for (int s = 0; s < b->n; ++s)
        if (b->has_pending[s]) stage = std::max(stage, np[s]);
    if (e == cudaSuccess && stage > b->staging_cap) {
        cudaFree(b->staging);
        b->staging = nullptr;
        b->staging_cap = 0;
        e = dalloc(&b->staging, (size_t)stage * 4);
        if (e == cudaSuccess) b->staging_cap = stage;
    }
    if (e != cudaSuccess) {
        for (float* p : na) cudaFree(p);
        return cuda_fail(b, e, "batch particle storage");
    }
    const Launch L = b->L();
    float* old[4] = {b->px, b->py, b->pvx, b->pvy};
    for (int s = 0; s < b->n && e == cudaSuccess; ++s) {
        if (b->has_pending[s]) {
            if (np[s] > 0) {
                e = cudaMemcpyAsync(b->staging, b->pending[s].data(), sizeof(float) * 4 * (size_t)np[s],
                                    cudaMemcpyHostToDevice, b->stream);
                aos_to_soa(L, b->staging, np[s], na[0] + po[s], na[1] + po[s], na[2] + po[s], na[3] + po[s]);
                // the staging buffer is reused by the next simulation
                if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
            }
        } else if (np[s] > 0) {
            for (int k = 0; k < 4 && e == cudaSuccess; ++k)
                e = cudaMemcpyAsync(na[k] + po[s], old[k] + b->seg[s].po, sizeof(float) * (size_t)np[s],
                                    cudaMemcpyDeviceToDevice, b->stream);
        }
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        for (float* p : na) cudaFree(p);
        return cuda_fail(b, e, "batch particle layout");
    }
    for (float* p : {b->px, b->py, b->pvx, b->pvy, b->yu, b->xv}) cudaFree(p);
    b->px = na[0];
    b->py = na[1];
    b->pvx = na[2];
    b->pvy = na[3];
    b->yu = na[4];
    b->xv = na[5];
    std::vector<int2> pblk;
    pblk.reserve((size_t)(total / DOMAIN_TPB));
    for (int s = 0; s < b->n; ++s) {
        b->seg[s].np = np[s];
        b->seg[s].po = po[s];
        b->cap[s] = cap[s];
        for (int64_t k = 0; k < cap[s]; k += DOMAIN_TPB) pblk.push_back(make_int2(s, (int)k));
        b->pending[s].clear();
        b->pending[s].shrink_to_fit();
        b->has_pending[s] = 0;
    }
    b->parts = total;
    cudaFree(b->d_pblk);
    b->d_pblk = nullptr;
    e = dalloc(&b->d_pblk, pblk.size());
    if (e == cudaSuccess && !pblk.empty())
        e = cudaMemcpyAsync(b->d_pblk, pblk.data(), sizeof(int2) * pblk.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_seg, b->seg.data(), sizeof(Seg) * b->n, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = ensure_splat_capacity(b, std::max(b->parts, b->cells));
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "batch particle tables");
    b->npblk = (unsigned)pblk.size();
    b->layout_dirty = false;
    ++b->layout_version;
    clear_graphs(b);
    return FS_OK;
}

Domain domain(const fs_batch* b)
{
    Domain d;
    d.segs = b->d_seg;
    d.cblk = b->d_cblk;
    d.ncblk = b->ncblk;
    d.pblk = b->d_pblk;
    d.npblk = b->npblk;
    d.nsim = b->n;
    d.cells = b->cells;
    d.parts = b->parts;
    return d;
}

void batch_solve(void* owner, const Launch& L)
{
    fs_batch* b = static_cast<fs_batch*>(owner);
    CgBatchArgs ba{};
    ba.systems = b->d_sys;
    ba.order = b->d_order;
    ba.nfluid = b->nfluid;
    ba.b = b->cg_b;
    ba.down = b->cg_down;
    ba.up = b->cg_up;
    ba.flags = b->cg_flags;
    ba.x = b->cx;
    ba.r = b->cr;
    ba.z = b->cz;
    ba.p = b->cp;
    ba.q = b->cq;
    ba.partials = b->partials;
    ba.status = b->status;
    ba.result = b->results;
    ba.fp64 = b->fp64;
    const int nc = (int)b->plan.size();
    if (nc > 1) cudaEventRecord(b->fork, L.stream);
    for (int c = 1; c < nc; ++c) {
        cudaStreamWaitEvent(b->aux[c - 1], b->fork, 0);
        const Launch La{b->aux[c - 1], L.counter, 0};
        CgBatchArgs bc = ba;
        bc.order = b->d_order + b->plan[c].first;
        cg_solve_clusters(La, bc, b->plan[c].count, b->plan[c].K, b->plan[c].C);
        cudaEventRecord(b->join[c - 1], b->aux[c - 1]);
    }
    if (nc > 0) {
        CgBatchArgs bc = ba;
        bc.order = b->d_order + b->plan[0].first;
        cg_solve_clusters(L, bc, b->plan[0].count, b->plan[0].K, b->plan[0].C);
    }
    for (int c = 1; c < nc; ++c) cudaStreamWaitEvent(L.stream, b->join[c - 1], 0);
}

StepState state(fs_batch* b)
{
    StepState st{};
    st.d = domain(b);
    st.front = &b->front;
    st.vfront = &b->vfront;
    for (int k = 0; k < 2; ++k) {
        st.u[k] = b->u[k];
        st.v[k] = b->v[k];
        st.vmx[k] = b->vmx[k];
        st.vmy[k] = b->vmy[k];
        st.sl_ok[k] = b->sl_ok[k];
    }
    st.u_prev = b->u_prev;
    st.v_prev = b->v_prev;
    st.u_diff = b->u_diff;
    st.v_diff = b->v_diff;
    st.labels = b->labels;
    st.solid = b->solid;
    st.fidx = b->fidx;
    st.cell_of = b->cell_of;
    st.counts32 = b->counts32;
    st.counts8 = b->counts8;
    for (int k = 0; k < 4; ++k) st.acc[k] = b->acc[k];
    for (int k = 0; k < 6; ++k) st.sl[k] = b->sl[k];
    st.px = b->px;
    st.py = b->py;
    st.pvx = b->pvx;
    st.pvy = b->pvy;
    st.yu = b->yu;
    st.xv = b->xv;
    st.sw = &b->sw;
    st.cg_b = b->cg_b;
    st.cg_down = b->cg_down;
    st.cg_up = b->cg_up;
    st.cg_flags = b->cg_flags;
    st.cg_x = b->cx;
    st.nfluid = b->nfluid;
    st.warn = b->warn;
    st.index_tmp = b->index_tmp;
    st.n_ext = b->n_ext;
    st.solve = batch_solve;
    st.mark = nullptr;
    st.owner = b;
    return st;
}

cudaError_t ensure_sl_scratch(fs_batch* b)
{
    if (b->sl[0]) return cudaSuccess;
    cudaError_t e;
    for (int k = 0; k < 6; ++k)
        if ((e = dalloc(&b->sl[k], (size_t)b->cells)) != cudaSuccess) return e;
    for (int k = 0; k < 2; ++k)
        if ((e = dalloc(&b->sl_ok[k], (size_t)b->cells)) != cudaSuccess) return e;
    clear_graphs(b);
    return cudaSuccess;
}

// FluidSolver::validate (src/FluidSolver.cpp:89-97) per simulation.
int validate_all(fs_batch* b)
{
    for (int s = 0; s < b->n; ++s) {
        const Geom& g = b->seg[s].g;
        if (!(std::fabs(g.dy - g.pdy) < 0.0000001))
            return fail(b, FS_ERR_VALIDATE,
                        "simulation " + std::to_string(s) +
                            ": Memory pool and fluid domain does not match. Initialize the fluid solver with a memory "
                            "pool corresponding to the right fluid domain!");
    }
    return FS_OK;
}

int run_step(fs_batch* b, int method, float dt)
{
    StepState st = state(b);
    enqueue_step(b->L(), st, method, dt);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FS_OK : cuda_fail(b, e, "batch step");
}

int step_graph(fs_batch* b, int method, float dt)
{
    if (!b->graphs) return run_step(b, method, dt);
    const uint32_t db = float_bits(dt);
    for (auto& g : b->gcache) {
        if (g.method == method && g.dt_bits == db && g.front_in == b->front && g.vfront_in == b->vfront &&
            g.plan == b->plan_target && g.layout == b->layout_version) {
            const cudaError_t e = cudaGraphLaunch(g.exec, b->stream);
            if (e != cudaSuccess) return cuda_fail(b, e, "batch graph launch");
            b->front = g.front_out;
            b->vfront = g.vfront_out;
            b->launches += g.kernels;
            return FS_OK;
        }
    }
    BatchGraph g{};
    g.method = method;
    g.dt_bits = db;
    g.front_in = b->front;
    g.vfront_in = b->vfront;
    g.plan = b->plan_target;
    g.layout = b->layout_version;
    const int64_t l0 = b->launches;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(b, e, "begin capture");
    StepState st = state(b);
    enqueue_step(b->L(), st, method, dt);
    const cudaError_t el = cudaGetLastError();
    e = cudaStreamEndCapture(b->stream, &graph);
    g.front_out = b->front;
    g.vfront_out = b->vfront;
    g.kernels = b->launches - l0;
    b->launches = l0;
    b->front = g.front_in;
    b->vfront = g.vfront_in;
    if (e != cudaSuccess || el != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        b->graphs = false;
        return run_step(b, method, dt);
    }
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b->graphs = false;
        return run_step(b, method, dt);
    }
    b->gcache.push_back(g);
    e = cudaGraphLaunch(g.exec, b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "batch graph launch");
    b->front = g.front_out;
    b->vfront = g.vfront_out;
    b->launches += g.kernels;
    return FS_OK;
}

int device_status(fs_batch* b)
{
    unsigned st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, b->status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "batch synchronize");
    if (st) {
        cudaMemsetAsync(b->status, 0, sizeof(unsigned), b->stream);
        cudaStreamSynchronize(b->stream);
    }
    if (st & ST_TOO_LARGE) return fail(b, FS_ERR_TOO_LARGE, "a simulation exceeded its CG cluster capacity");
    if (st & ST_INTERNAL) return fail(b, FS_ERR_INTERNAL, "internal consistency check failed on the device");
    return FS_OK;
}

// The state a step reads and writes (everything but scratch), for the tuner's
// save and restore.
struct Region
{
    void* p;
    size_t bytes;
};

std::vector<Region> persistent(fs_batch* b)
{
    const size_t C = (size_t)b->cells, P = (size_t)b->parts;
    std::vector<Region> r = {{b->u[0], 4 * C},   {b->u[1], 4 * C},   {b->v[0], 4 * C},     {b->v[1], 4 * C},
                             {b->u_prev, 4 * C}, {b->v_prev, 4 * C}, {b->u_diff, 4 * C},   {b->v_diff, 4 * C},
                             {b->labels, C},     {b->vmx[0], C},     {b->vmx[1], C},       {b->vmy[0], C},
                             {b->vmy[1], C},     {b->fidx, 4 * C},   {b->counts8, C},      {b->cx, 4 * C},
                             {b->px, 4 * P},     {b->py, 4 * P},     {b->pvx, 4 * P},      {b->pvy, 4 * P},
                             {b->nfluid, 4 * (size_t)b->n},          {b->results, sizeof(CgResult) * b->n},
                             {b->warn, 4}};
    return r;
}

void free_all(fs_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    clear_graphs(b);
    void* ptrs[] = {b->d_seg, b->d_cblk, b->d_pblk, b->u[0], b->u[1], b->v[0], b->v[1], b->u_prev, b->v_prev,
                    b->u_diff, b->v_diff, b->labels, b->solid, b->vmx[0], b->vmx[1], b->vmy[0], b->vmy[1], b->fidx,
                    b->cell_of, b->counts32, b->counts8, b->acc[0], b->acc[1], b->acc[2], b->acc[3], b->grid_tmp,
                    b->sl[0], b->sl[1], b->sl[2], b->sl[3], b->sl[4], b->sl[5], b->sl_ok[0], b->sl_ok[1], b->cg_b,
                    b->cg_down, b->cg_up, b->cg_flags, b->cx, b->cr, b->cz, b->cp, b->cq, b->px, b->py, b->pvx,
                    b->pvy, b->yu, b->xv, b->staging, b->nfluid, b->status, b->warn,
                    b->index_tmp, b->d_sys, b->partials, b->results, b->d_order};
    for (void* p : ptrs) cudaFree(p);
    splat_free(b->sw);
    for (cudaStream_t s : b->aux)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

bool sim_ok(const fs_batch* b, int sim) { return b && sim >= 0 && sim < b->n; }

template <class T>
int copy_out(fs_batch* b, T* host, const T* dev, size_t count)
{
    if (!host) return fail(b, FS_ERR_INVALID_ARGUMENT, "null output pointer");
    cudaError_t e = cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(b, e, "copy to host");
    return FS_OK;
}

float* grid_ptr(fs_batch* b, int which)
{
    switch (which) {
        case FS_U_FRONT: return b->u[b->front];
        case FS_V_FRONT: return b->v[b->front];
        case FS_U_BACK: return b->u[1 - b->front];
        case FS_V_BACK: return b->v[1 - b->front];
        case FS_U_PREV: return b->u_prev;
        case FS_V_PREV: return b->v_prev;
        case FS_U_DIFF: return b->u_diff;
        case FS_V_DIFF: return b->v_diff;
        default: return nullptr;
    }
}

}  // namespace

extern "C" {

const char* fs_batch_last_error(const fs_batch* b) { return b ? b->err.c_str() : g_batch_error.c_str(); }

int fs_batch_create(int n, const fs_config* cfgs, fs_batch** out)
{
    g_batch_error.clear();
    if (!out || !cfgs || n < 1) {
        g_batch_error = "invalid batch arguments";
        return FS_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    fs_batch* b = new fs_batch();
    b->n = n;
    b->device = cfgs[0].device;
    b->cfg.assign(cfgs, cfgs + n);
    b->seg.resize(n);
    b->cap.assign(n, 0);
    b->pending.resize(n);
    b->has_pending.assign(n, 0);
    b->n_ext = cfgs[0].extension_iterations;
    if (cfgs[0].cg_precision == FS_CG_DS) {
        g_batch_error = "double-single CG dot products are not available for batches";
        delete b;
        return FS_ERR_INVALID_ARGUMENT;
    }
    b->fp64 = cfgs[0].cg_precision == FS_CG_DOUBLE ? 1 : 0;
    std::vector<int2> cblk;
    std::vector<CgSystem> sys(n);
    int64_t cells = 0, part_off = 0;
    for (int s = 0; s < n; ++s) {
        const fs_config& c = cfgs[s];
        if (c.size_x < 1 || c.size_y < 1 || !(c.length_x > 0) || !(c.length_y > 0) || !std::isfinite(c.length_x) ||
            !std::isfinite(c.length_y) || c.device != b->device || c.extension_iterations < 0 ||
            !(c.cg_tolerance >= 0) || c.cg_max_iterations < 0) {
            g_batch_error = "simulation " + std::to_string(s) + ": invalid configuration";
            delete b;
            return FS_ERR_INVALID_ARGUMENT;
        }
        Seg& sg = b->seg[s];
        Geom& g = sg.g;
        g.nx = c.size_x;
        g.ny = c.size_y;
        g.dx = c.length_x / (float)c.size_x;
        g.dy = c.length_y / (float)c.size_y;
        g.lx = (float)g.nx * g.dx;
        g.ly = (float)g.ny * g.dy;
        g.pdx = g.dx;
        g.pdy = g.dx;  // the solver pool's copy keeps delta_x for delta_y (src/FluidSolver.cpp:56-62)
        if (interior(sg) > BATCH_MAX_INTERIOR) {
            g_batch_error = "simulation " + std::to_string(s) + ": more than 65536 interior cells for a batch";
            delete b;
            return FS_ERR_TOO_LARGE;
        }
        // FluidDomain::setPicRatio clamps (src/FluidDomain.cpp:99-102); the constructor stores as given (:64).
        sg.pic = c.pic_ratio;
        sg.rho = c.density;
        sg.gx = c.gravity_x;
        sg.gy = c.gravity_y;
        sg.sim = s;
        sg.co = cells;
        sg.cb0 = (int)cblk.size();
        const int64_t nc = (int64_t)g.nx * g.ny;
        for (int64_t k = 0; k < nc; k += DOMAIN_TPB) cblk.push_back(make_int2(s, (int)k));
        sg.ncb = (int)cblk.size() - sg.cb0;
        cells += round_up(nc, DOMAIN_TPB);
        if (cells > BATCH_MAX_CELLS) {
            g_batch_error = "batch larger than 16 Mi cells";
            delete b;
            return FS_ERR_TOO_LARGE;
        }
        CgSystem& cs = sys[s];
        cs.co = sg.co;
        cs.max_chunks = (int)((nc + 1023) / 1024);
        cs.part_off = part_off;
        part_off += 4 * (int64_t)cs.max_chunks;
        // Matrix coefficients through double pow() as in src/FluidSolver.cpp:381-410.
        const double dx2 = std::pow((double)g.dx, 2);
        cs.off = (float)(1 / dx2);
        for (int k = 0; k < 5; ++k) {
            cs.dtab[k] = (float)(-k / dx2);
            cs.itab[k] = cs.dtab[k] != 0.0f ? 1.0f / cs.dtab[k] : 1.0f;
        }
        cs.tol = c.cg_tolerance;
        cs.maxit = c.cg_max_iterations;
    }
    b->cells = cells;
    b->ncblk = (unsigned)cblk.size();
    const size_t C = (size_t)cells;
    cudaError_t e = cudaSetDevice(b->device);
    bool ok = e == cudaSuccess;
    auto A = [&](cudaError_t r) {
        if (r != cudaSuccess && ok) {
            ok = false;
            e = r;
        }
    };
    A(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    for (int k = 0; k < MAX_CLASSES - 1; ++k) {
        A(cudaStreamCreateWithFlags(&b->aux[k], cudaStreamNonBlocking));
        A(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    }
    A(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    A(dalloc(&b->d_seg, (size_t)n));
    A(dalloc(&b->d_cblk, cblk.size()));
    A(dalloc(&b->d_pblk, 1));
    for (int k = 0; k < 2; ++k) {
        A(dalloc(&b->u[k], C));
        A(dalloc(&b->v[k], C));
        A(dalloc(&b->vmx[k], C));
        A(dalloc(&b->vmy[k], C));
    }
    for (float** p : {&b->u_prev, &b->v_prev, &b->u_diff, &b->v_diff, &b->grid_tmp, &b->cg_b, &b->cx, &b->cr, &b->cz,
                      &b->cp, &b->cq, &b->acc[0], &b->acc[1], &b->acc[2], &b->acc[3]})
        A(dalloc(p, C));
    A(dalloc(&b->labels, C));
    A(dalloc(&b->fidx, C));
    A(dalloc(&b->cell_of, C));
    A(dalloc(&b->counts32, C));
    A(dalloc(&b->counts8, C));
    A(dalloc(&b->cg_down, C));
    A(dalloc(&b->cg_up, C));
    A(dalloc(&b->cg_flags, C));
    A(dalloc(&b->nfluid, (size_t)n));
    A(dalloc(&b->status, 1));
    A(dalloc(&b->warn, 1));
    A(dalloc(&b->d_sys, (size_t)n));
    A(dalloc(&b->partials, (size_t)std::max<int64_t>(part_off, 1)));
    A(dalloc(&b->results, (size_t)n));
    A(dalloc(&b->d_order, (size_t)n));
    if (ok) {
        Domain d = domain(b);
        A(dalloc(&b->index_tmp, fluid_index_batch_tmp_ints(d)));
    }
    if (ok) A(ensure_splat_capacity(b, b->cells));
    if (ok) {
        A(cudaMemcpyAsync(b->d_seg, b->seg.data(), sizeof(Seg) * n, cudaMemcpyHostToDevice, b->stream));
        A(cudaMemcpyAsync(b->d_cblk, cblk.data(), sizeof(int2) * cblk.size(), cudaMemcpyHostToDevice, b->stream));
        A(cudaMemcpyAsync(b->d_sys, sys.data(), sizeof(CgSystem) * n, cudaMemcpyHostToDevice, b->stream));
        // Zero-initialised state, as the reference's Grid<T> ctor (include/Grid.h:129-139).
        for (float* p : {b->u[0], b->u[1], b->v[0], b->v[1], b->u_prev, b->v_prev, b->u_diff, b->v_diff, b->cx,
                         b->acc[0], b->acc[1], b->acc[2], b->acc[3]})
            A(cudaMemsetAsync(p, 0, C * 4, b->stream));
        for (uint8_t* p : {b->vmx[0], b->vmx[1], b->vmy[0], b->vmy[1], b->counts8}) A(cudaMemsetAsync(p, 0, C, b->stream));
        // padding cells between simulations read as SOLID and are never written
        A(cudaMemsetAsync(b->labels, SOLID, C, b->stream));
        A(cudaMemsetAsync(b->fidx, 0, C * 4, b->stream));
        A(cudaMemsetAsync(b->nfluid, 0, 4 * (size_t)n, b->stream));
        A(cudaMemsetAsync(b->status, 0, 4, b->stream));
        A(cudaMemsetAsync(b->warn, 0, 4, b->stream));
        A(cudaMemsetAsync(b->results, 0, sizeof(CgResult) * n, b->stream));
        A(cudaMemsetAsync(b->partials, 0, sizeof(double) * (size_t)std::max<int64_t>(part_off, 1), b->stream));
        if (ok) labels_clear(b->L(), domain(b), b->labels);  // MacGrid ctor -> clearCellTypeBuffer (src/MacGrid.cpp:24)
        A(cudaGetLastError());
        A(cudaStreamSynchronize(b->stream));
    }
    if (!ok) {
        g_batch_error = std::string("fs_batch_create: ") + cudaGetErrorString(e);
        const int code = e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA;
        free_all(b);
        return code;
    }
    b->plan_chunks.resize(n);
    for (int s = 0; s < n; ++s) b->plan_chunks[s] = max_chunks(b->seg[s]);
    const int rc = make_plan(b, 8);
    if (rc != FS_OK) {
        g_batch_error = b->err;
        free_all(b);
        return rc;
    }
    *out = b;
    return FS_OK;
}

int fs_batch_destroy(fs_batch* b)
{
    free_all(b);
    return FS_OK;
}

int fs_batch_size(const fs_batch* b) { return b ? b->n : 0; }

int fs_batch_set_particles(fs_batch* b, int sim, const float* xyuv, int64_t n)
{
    if (!sim_ok(b, sim) || n < 0 || (n > 0 && !xyuv))
        return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "invalid particles") : FS_ERR_INVALID_ARGUMENT;
    if (n > (int64_t)INT32_MAX) return fail(b, FS_ERR_TOO_LARGE, "more than 2^31-1 particles");
    b->pending[sim].assign(xyuv, xyuv + 4 * n);
    b->has_pending[sim] = 1;
    b->layout_dirty = true;
    return FS_OK;
}

int fs_batch_num_particles(fs_batch* b, int sim, int64_t* n)
{
    if (!sim_ok(b, sim) || !n) return FS_ERR_INVALID_ARGUMENT;
    *n = b->has_pending[sim] ? (int64_t)b->pending[sim].size() / 4 : b->seg[sim].np;
    return FS_OK;
}

int fs_batch_get_particles(fs_batch* b, int sim, float* xyuv, int64_t n)
{
    if (!sim_ok(b, sim)) return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "no such simulation") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    int rc = flush_layout(b);
    if (rc) return rc;
    const Seg& s = b->seg[sim];
    if (n != s.np) return fail(b, FS_ERR_INVALID_ARGUMENT, "particle count mismatch");
    if (n == 0) return FS_OK;
    if (b->staging_cap < n) {
        cudaFree(b->staging);
        b->staging = nullptr;
        b->staging_cap = 0;
        const cudaError_t e = dalloc(&b->staging, (size_t)n * 4);
        if (e != cudaSuccess) return cuda_fail(b, e, "staging");
        b->staging_cap = n;
    }
    soa_to_aos(b->L(), b->px + s.po, b->py + s.po, b->pvx + s.po, b->pvy + s.po, n, b->staging);
    return copy_out(b, xyuv, b->staging, (size_t)n * 4);
}

int fs_batch_set_solid_mask(fs_batch* b, int sim, const uint8_t* mask)
{
    if (!sim_ok(b, sim)) return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "no such simulation") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    const Seg& s = b->seg[sim];
    const size_t nc = (size_t)s.g.nx * s.g.ny;
    cudaError_t e = cudaSuccess;
    if (!b->solid) {
        if (!mask) return FS_OK;
        e = dalloc(&b->solid, (size_t)b->cells);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->solid, 0, (size_t)b->cells, b->stream);
        clear_graphs(b);
    }
    if (e == cudaSuccess) {
        e = mask ? cudaMemcpyAsync(b->solid + s.co, mask, nc, cudaMemcpyHostToDevice, b->stream)
                 : cudaMemsetAsync(b->solid + s.co, 0, nc, b->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? FS_OK : cuda_fail(b, e, "solid mask");
}

int fs_batch_get_grid(fs_batch* b, int sim, int which, float* out)
{
    if (!sim_ok(b, sim)) return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "no such simulation") : FS_ERR_INVALID_ARGUMENT;
    float* p = grid_ptr(b, which);
    if (!p) return fail(b, FS_ERR_INVALID_ARGUMENT, "unknown grid");
    cudaSetDevice(b->device);
    const Seg& s = b->seg[sim];
    return copy_out(b, out, p + s.co, (size_t)s.g.nx * s.g.ny);
}

int fs_batch_get_labels(fs_batch* b, int sim, uint8_t* out)
{
    if (!sim_ok(b, sim)) return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "no such simulation") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    const Seg& s = b->seg[sim];
    return copy_out(b, out, b->labels + s.co, (size_t)s.g.nx * s.g.ny);
}

int fs_batch_get_pressure(fs_batch* b, int sim, float* out)
{
    if (!sim_ok(b, sim)) return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "no such simulation") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    pressure_to_grid(b->L(), domain(b), b->fidx, b->nfluid, b->cx, b->grid_tmp);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(b, e, "pressure");
    const Seg& s = b->seg[sim];
    return copy_out(b, out, b->grid_tmp + s.co, (size_t)s.g.nx * s.g.ny);
}

int fs_batch_step(fs_batch* b, int method, float dt)
{
    if (!b) return FS_ERR_INVALID_ARGUMENT;
    if (method < FS_STEP_SEMI_LAGRANGIAN || method > FS_STEP_PICFLIP)
        return fail(b, FS_ERR_INVALID_ARGUMENT, "unknown step method");
    int rc = validate_all(b);
    if (rc) return rc;
    cudaSetDevice(b->device);
    rc = flush_layout(b);
    if (rc) return rc;
    if (method == FS_STEP_SEMI_LAGRANGIAN) {
        const cudaError_t e = ensure_sl_scratch(b);
        if (e != cudaSuccess) return cuda_fail(b, e, "semi-Lagrangian scratch");
    }
    rc = step_graph(b, method, dt);
    if (rc == FS_OK) b->counted = true;
    return rc;
}

int fs_batch_synchronize(fs_batch* b)
{
    if (!b) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    return device_status(b);
}

int fs_batch_get_stats(fs_batch* b, int sim, fs_step_stats* out)
{
    if (!sim_ok(b, sim) || !out) return FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    const int rc = device_status(b);
    std::memset(out, 0, sizeof(*out));
    CgResult r{};
    int32_t nf = 0;
    unsigned warn = 0;
    cudaMemcpy(&r, b->results + sim, sizeof(r), cudaMemcpyDeviceToHost);
    cudaMemcpy(&nf, b->nfluid + sim, sizeof(nf), cudaMemcpyDeviceToHost);
    cudaMemcpy(&warn, b->warn, sizeof(warn), cudaMemcpyDeviceToHost);
    out->cg_iterations = r.iterations;
    out->n_fluid = nf;
    out->cg_residual = r.bb > 0 ? std::sqrt(r.rr / r.bb) : 0.0;
    const fs_config& c = b->cfg[sim];
    if (nf > 0 && r.bb > 0 && r.iterations >= c.cg_max_iterations && std::sqrt(r.rr / r.bb) >= c.cg_tolerance)
        warn |= FS_WARN_CG_NOT_CONVERGED;
    out->warnings = warn;
    cudaGetLastError();
    return rc;
}

int fs_batch_set_tuning(fs_batch* b, int chunks_per_cta)
{
    if (!b || (chunks_per_cta != 1 && chunks_per_cta != 2 && chunks_per_cta != 4 && chunks_per_cta != 8))
        return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "chunks per CTA must be 1, 2, 4 or 8") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    // after a step, plan for the fluid cells that step counted, as the tuner does
    if (b->counted) {
        const int rc = refresh_plan_chunks(b);
        if (rc) return rc;
    } else if (chunks_per_cta == b->plan_target) {
        return FS_OK;
    }
    return make_plan(b, chunks_per_cta);
}

int fs_batch_get_tuning(const fs_batch* b) { return b ? b->plan_target : 0; }

int fs_batch_tune(fs_batch* b, int method, float dt, int steps, float* ms_out)
{
    if (!b || steps < 1) return b ? fail(b, FS_ERR_INVALID_ARGUMENT, "steps must be positive") : FS_ERR_INVALID_ARGUMENT;
    int rc = validate_all(b);
    if (rc) return rc;
    cudaSetDevice(b->device);
    rc = flush_layout(b);
    if (rc) return rc;
    if (method == FS_STEP_SEMI_LAGRANGIAN) {
        const cudaError_t e = ensure_sl_scratch(b);
        if (e != cudaSuccess) return cuda_fail(b, e, "semi-Lagrangian scratch");
    }
    rc = refresh_plan_chunks(b);
    if (rc) return rc;
    // Save the state, time `steps` steps per candidate from that state, restore.
    const std::vector<Region> regs = persistent(b);
    size_t total = 0;
    for (const Region& r : regs) total += (r.bytes + 255) / 256 * 256;
    unsigned char* save = nullptr;
    cudaError_t e = cudaMalloc(&save, total);
    if (e != cudaSuccess) return cuda_fail(b, e, "tuner state copy");
    auto copy_all = [&](bool to_save) {
        size_t off = 0;
        for (const Region& r : regs) {
            if (to_save) cudaMemcpyAsync(save + off, r.p, r.bytes, cudaMemcpyDeviceToDevice, b->stream);
            else cudaMemcpyAsync(r.p, save + off, r.bytes, cudaMemcpyDeviceToDevice, b->stream);
            off += (r.bytes + 255) / 256 * 256;
        }
    };
    copy_all(true);
    const int front = b->front, vfront = b->vfront;
    const int candidates[4] = {1, 2, 4, 8};
    float best_ms = 0.0f;
    int best = b->plan_target;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    rc = FS_OK;
    for (int ci = 0; ci < 4 && rc == FS_OK; ++ci) {
        rc = make_plan(b, candidates[ci]);
        if (rc) break;
        copy_all(false);
        b->front = front;
        b->vfront = vfront;
        rc = step_graph(b, method, dt);  // capture + first run (not timed)
        if (rc) break;
        copy_all(false);
        b->front = front;
        b->vfront = vfront;
        cudaEventRecord(t0, b->stream);
        for (int k = 0; k < steps && rc == FS_OK; ++k) rc = step_graph(b, method, dt);
        cudaEventRecord(t1, b->stream);
        if (cudaEventSynchronize(t1) != cudaSuccess) rc = cuda_fail(b, cudaGetLastError(), "tuner timing");
        if (rc) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t0, t1);
        ms /= (float)steps;
        if (ms_out) ms_out[ci] = ms;
        if (ci == 0 || ms < best_ms) {
            best_ms = ms;
            best = candidates[ci];
        }
    }
    copy_all(false);
    b->front = front;
    b->vfront = vfront;
    cudaStreamSynchronize(b->stream);
    cudaFree(save);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (rc) return rc;
    rc = make_plan(b, best);
    if (rc) return rc;
    return device_status(b);
}

int fs_batch_set_graphs(fs_batch* b, int enable)
{
    if (!b) return FS_ERR_INVALID_ARGUMENT;
    b->graphs = enable != 0;
    if (!b->graphs) clear_graphs(b);
    return FS_OK;
}

void* fs_batch_get_stream(fs_batch* b) { return b ? (void*)b->stream : nullptr; }

int64_t fs_batch_kernel_launches(fs_batch* b) { return b ? b->launches : 0; }

}  // extern "C"
