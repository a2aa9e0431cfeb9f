// Headless renderer: Renderer (src/Renderer.cpp) drawing a simulation onto a
// Canvas (src/Canvas.cpp) of RGB floats held in device memory.  The reference
// paints shapes one after another (later shapes overwrite earlier ones), so
// every pass here computes, per pixel, what the last shape covering it wrote:
//   * cells: the rectangles are products of an x range and a y range, each
//     monotone in the cell index, so the last cell covering a pixel is (the
//     largest i covering its column, the largest j covering its row);
//   * particles: every point uses one colour, so their order does not matter;
//   * velocity lines: each line marks its pixels with its index (atomicMax),
//     then every marked pixel takes the colour of the line with the largest;
//   * metaballs: each pixel's field value is a float sum over particles in
//     particle order, so particles are grouped by pixel position (each group
//     in particle order) and every pixel merges the groups of its 10 x 10
//     neighbourhood by particle index before adding.
// Float operations follow the reference's types and order (the library is
// built with -fmad=false), so the canvas is bit-identical to the reference's.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fs_render.h"

using namespace fs;

namespace {

constexpr int TPB = 256;
constexpr int MB_CAP = 64;  // metaball contributions merged in registers/local memory before the slow path

unsigned nblk(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

__device__ __forceinline__ void put(float* px, int w, int x, int y, float r, float g, float b)
{
    float* p = px + 3 * ((size_t)x + (size_t)y * w);
    p[0] = r;
    p[1] = g;
    p[2] = b;
}

__global__ void k_fill(float* __restrict__ px, int64_t n, float r, float g, float b)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k >= n) return;
    px[3 * k] = r;
    px[3 * k + 1] = g;
    px[3 * k + 2] = b;
}

// Rectangle bound of cell i along one axis: (int)(-translate + i * cell_size),
// clamped to the canvas through float (Renderer.cpp:49-53, Canvas.cpp:78-81).
__device__ __forceinline__ int bound(float neg_t, float cs, int i, int lim)
{
    return clampi(trunc_i(fadd(neg_t, fmul((float)i, cs))), 0, lim - 1);
}

// The largest cell index whose clamped range [bound(i), bound(i + 1)] holds p, or -1.
__device__ __forceinline__ int last_cover(int p, int n, float neg_t, float cs, int lim)
{
    if (n < 1 || bound(neg_t, cs, 0, lim) > p) return -1;
    int a = 0, b = n - 1;
    while (a < b) {
        const int m = (a + b + 1) / 2;
        if (bound(neg_t, cs, m, lim) <= p) a = m;
        else b = m - 1;
    }
    return bound(neg_t, cs, a + 1, lim) >= p ? a : -1;
}

__device__ __forceinline__ void cell_fill(uint8_t t, float& r, float& g, float& b)
{
    if (t == LIQUID) { r = 0.7f; g = 0.7f; b = 1.0f; }
    else if (t == AIR) { r = 1.0f; g = 1.0f; b = 1.0f; }
    else { r = 0.5f; g = 0.5f; b = 0.5f; }
}

// Renderer::renderGridCellsToCanvas (Renderer.cpp:18-56), or with level-set
// values (lsv non-null) renderLevelSetFunctionValuesToCanvas (:58-91), whose
// cells are filled with (value, value, value).
__device__ __forceinline__ void cell_color(const uint8_t* lab, const float* lsv, size_t c, float& r, float& g, float& b)
{
    if (lsv) r = g = b = lsv[c];
    else cell_fill(lab[c], r, g, b);
}

__global__ void k_cells(float* __restrict__ px, float* __restrict__ colors, int w, int h, View v, float csx,
                        float csy, int nx, int ny, const uint8_t* __restrict__ lab, const float* __restrict__ lsv)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k == 0) {  // the canvas's colours afterwards: white lines, the last cell's fill
        float r, g, b;
        cell_color(lab, lsv, (size_t)(nx - 1) + (size_t)(ny - 1) * nx, r, g, b);
        colors[0] = colors[1] = colors[2] = 1.0f;
        colors[3] = r;
        colors[4] = g;
        colors[5] = b;
    }
    if (k >= (int64_t)w * h) return;
    const int X = (int)(k % w), Y = (int)(k / w);
    const float ntx = -v.translate_x, nty = -v.translate_y;
    const int i = last_cover(X, nx, ntx, csx, w);
    const int j = last_cover(Y, ny, nty, csy, h);
    if (i < 0 || j < 0) return;
    const bool border = X == bound(ntx, csx, i, w) || X == bound(ntx, csx, i + 1, w) || Y == bound(nty, csy, j, h) ||
                        Y == bound(nty, csy, j + 1, h);
    float r = 1.0f, g = 1.0f, b = 1.0f;
    if (!border) cell_color(lab, lsv, (size_t)i + (size_t)j * nx, r, g, b);
    put(px, w, X, Y, r, g, b);
}

// One velocity line of Renderer::renderGridVelocitiesToCanvas (Renderer.cpp:107-137).
struct Line
{
    int fx, fy, tx, ty;
    float r, g, b;
};

__device__ __forceinline__ Line vel_line(int i, int j, int nx, int w, View v, float csx, float csy,
                                         const float* __restrict__ uf, const float* __restrict__ vf)
{
    Line L;
    const size_t c = (size_t)i + (size_t)j * nx;
    // MacGrid::velX / velY (include/MacGrid.h:30-39): the cell's two faces averaged
    const float vel_x = fdiv(fadd(uf[c], uf[c + 1]), 2.0f);
    const float vel_y = fdiv(fadd(vf[c], vf[c + nx]), 2.0f);
    L.fx = __double2int_rz(__dadd_rn((double)(-v.translate_x), __dmul_rn(0.5 + i, (double)csx)));
    L.fy = __double2int_rz(__dadd_rn((double)(-v.translate_y), __dmul_rn(0.5 + j, (double)csy)));
    L.tx = trunc_i(fadd((float)L.fx, fmul(vel_x, 5.0f)));
    L.ty = trunc_i(fadd((float)L.fy, fmul(vel_y, 5.0f)));
    const int dx = L.fx - L.tx, dy = L.fy - L.ty;
    const float len = (float)__dsqrt_rn((double)(dx * dx + dy * dy));
    const float ls = fdiv(len, (float)(w / 40));
    L.b = clampf(fsub(1.0f, ls), 0.0f, 1.0f);
    L.g = fsub(clampf(ls, 0.0f, 1.0f), clampf(fsub(ls, 1.0f), 0.0f, 1.0f));
    L.r = clampf(fsub(ls, 1.0f), 0.0f, 1.0f);
    return L;
}

// Canvas::drawLine's pixels (Canvas.cpp:39-62), marked with the line's index.
__global__ void k_vel_mark(int32_t* __restrict__ owner, float* __restrict__ colors, int w, int h, View v, float csx,
                           float csy, int nx, int ny, const float* __restrict__ uf, const float* __restrict__ vf)
{
    const int nlx = nx - 1, nly = ny - 1;
    const int64_t id = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (id >= (int64_t)nlx * nly) return;
    const int i = (int)(id % nlx), j = (int)(id / nlx);
    const Line L = vel_line(i, j, nx, w, v, csx, csy, uf, vf);
    if (id == (int64_t)nlx * nly - 1) {  // the line colour the canvas keeps afterwards
        colors[0] = L.r;
        colors[1] = L.g;
        colors[2] = L.b;
    }
    const float ddx = (float)(L.tx - L.fx), ddy = (float)(L.ty - L.fy);
    const float dist = __fsqrt_rn(fadd(fmul(ddx, ddx), fmul(ddy, ddy)));
    // Each step moves about one pixel along the line's longer axis (positions
    // come from the step count, not from accumulation), so a line leaves the
    // canvas within about 1.5 * max(w, h) steps: the cap never cuts a pixel
    // the reference paints, and bounds the loop for extreme velocities.
    const int cap = 2 * (w + h) + 16;
    for (int s = 0; (float)s < dist && s < cap; ++s) {
        const int x = trunc_i(fadd((float)L.fx, fmul(fdiv(ddx, dist), (float)s)));
        const int y = trunc_i(fadd((float)L.fy, fmul(fdiv(ddy, dist), (float)s)));
        if (x < 0 || x >= w || y < 0 || y >= h) break;
        atomicMax(&owner[(size_t)x + (size_t)y * w], (int32_t)(id + 1));
    }
}

__global__ void k_vel_paint(float* __restrict__ px, const int32_t* __restrict__ owner, int w, int h, View v, float csx,
                            float csy, int nx, const float* __restrict__ uf, const float* __restrict__ vf)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k >= (int64_t)w * h) return;
    const int o = owner[k];
    if (o == 0) return;
    const int id = o - 1, nlx = nx - 1;
    const Line L = vel_line(id % nlx, id / nlx, nx, w, v, csx, csy, uf, vf);
    put(px, w, (int)(k % w), (int)(k / w), L.r, L.g, L.b);
}

__device__ __forceinline__ void particle_pixel(const View& v, float x, float y, int& X, int& Y)
{
    X = trunc_i(fadd(-v.translate_x, fmul(v.scale_x, x)));
    Y = trunc_i(fadd(-v.translate_y, fmul(v.scale_y, y)));
}

// Renderer::renderParticlesToCanvas (Renderer.cpp:141-161): Canvas::drawPoint
// of size 3, one colour for border and inside.
__global__ void k_particles(float* __restrict__ px, float* __restrict__ colors, int w, int h, View v,
                            const float* __restrict__ pxs, const float* __restrict__ pys, int64_t n)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k == 0) {
        colors[0] = colors[3] = 0.3f;
        colors[1] = colors[4] = 0.6f;
        colors[2] = colors[5] = 0.9f;
    }
    if (k >= n) return;
    int X, Y;
    particle_pixel(v, pxs[k], pys[k], X, Y);
    const int x0 = clampi(X - 1, 0, w - 1), x1 = clampi(X + 1, 0, w - 1);
    const int y0 = clampi(Y - 1, 0, h - 1), y1 = clampi(Y + 1, 0, h - 1);
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) put(px, w, x, y, 0.3f, 0.6f, 0.9f);
}

struct Weights
{
    float w[100];  // [(j + 5) * 10 + (i + 5)] for pixel offsets i, j in [-5, 5)
};

// Metaballs, pass 1: each particle's pixel, and its group: the pixel on a
// grid extended by 5 on each side, or "none" when its 10 x 10 footprint
// misses the canvas.
__global__ void k_mb_keys(int w, int h, View v, const float* __restrict__ pxs, const float* __restrict__ pys,
                          int64_t n, uint32_t none, int32_t* __restrict__ pos, uint32_t* __restrict__ keys)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k >= n) return;
    int X, Y;
    particle_pixel(v, pxs[k], pys[k], X, Y);
    pos[2 * k] = X;
    pos[2 * k + 1] = Y;
    const bool hits = X >= -4 && X <= w + 4 && Y >= -4 && Y <= h + 4;
    keys[k] = hits ? (uint32_t)((X + 5) + (int64_t)(Y + 5) * (w + 10)) : none;
}

// Pass 2: the field of pixel (X, Y) adds, in particle order, the weights of
// the particles at X - 4 .. X + 5, Y - 4 .. Y + 5 (Renderer.cpp:176-199), then
// the thresholds (:200-214).
__global__ void k_mb_paint(float* __restrict__ px, int w, int h, const int32_t* __restrict__ pos,
                           const int32_t* __restrict__ bin_start, const int32_t* __restrict__ sorted, Weights W)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k >= (int64_t)w * h) return;
    const int X = (int)(k % w), Y = (int)(k / w);
    const int ew = w + 10;
    auto weight = [&](int p) { return W.w[(Y - pos[2 * p + 1] + 5) * 10 + (X - pos[2 * p] + 5)]; };
    int idx[MB_CAP];
    float wt[MB_CAP];
    int m = 0;
    bool overflow = false;
    for (int ey = Y + 1; ey <= Y + 10 && !overflow; ++ey)
        for (int ex = X + 1; ex <= X + 10; ++ex) {
            const int64_t b = (int64_t)ex + (int64_t)ey * ew;
            for (int q = bin_start[b]; q < bin_start[b + 1]; ++q) {
                if (m == MB_CAP) {
                    overflow = true;
                    break;
                }
                const int p = sorted[q];
                int t = m++;
                const float wp = weight(p);
                while (t > 0 && idx[t - 1] > p) {  // insertion into particle order
                    idx[t] = idx[t - 1];
                    wt[t] = wt[t - 1];
                    --t;
                }
                idx[t] = p;
                wt[t] = wp;
            }
            if (overflow) break;
        }
    float df = 0.0f;
    if (!overflow) {
        for (int t = 0; t < m; ++t) df = fadd(df, wt[t]);
    } else {
        // many contributions: merge the 100 groups (each in particle order) by repeated minimum
        int cur[100];
        for (int g = 0; g < 100; ++g) cur[g] = bin_start[(int64_t)(X + 1 + g % 10) + (int64_t)(Y + 1 + g / 10) * ew];
        for (;;) {
            int best = INT32_MAX, bg = -1;
            for (int g = 0; g < 100; ++g) {
                const int64_t b = (int64_t)(X + 1 + g % 10) + (int64_t)(Y + 1 + g / 10) * ew;
                if (cur[g] < bin_start[b + 1] && sorted[cur[g]] < best) {
                    best = sorted[cur[g]];
                    bg = g;
                }
            }
            if (bg < 0) break;
            ++cur[bg];
            df = fadd(df, weight(best));
        }
    }
    if ((double)df > 0.6) put(px, w, X, Y, 0.0f, 0.5f, 0.7f);
    else if ((double)df > 0.2) put(px, w, X, Y, 0.5f, 0.9f, 1.0f);
}

__global__ void k_set_colors(float* colors, float lr, float lg, float lb, float fr, float fg, float fb)
{
    colors[0] = lr;
    colors[1] = lg;
    colors[2] = lb;
    colors[3] = fr;
    colors[4] = fg;
    colors[5] = fb;
}

// Renderer::writeCanvasToPpm's conversion (Renderer.cpp:217-240).
__global__ void k_bytes(const float* __restrict__ px, int64_t n, uint8_t* __restrict__ out)
{
    const int64_t k = (int64_t)blockIdx.x * TPB + threadIdx.x;
    if (k < n) out[k] = (uint8_t)__float2uint_rz(fmul(clampf(px[k], 0.0f, 1.0f), 255.0f));
}

// gaussian (include/MathDefinitions.h:29-34) and the weights of
// renderMetaBallsToCanvas (Renderer.cpp:186-187), on the host with the same
// types and library functions as the reference's CPU code.
float gaussian_host(float x, float sigma, float mu)
{
    const float a = (float)(1 / ((double)sigma * std::sqrt(2 * M_PI)));
    const float xm = x - mu;
    return a * expf(-(xm * xm) / (2 * sigma * sigma));
}

Weights metaball_weights()
{
    Weights W;
    for (int j = -5; j < 5; ++j)
        for (int i = -5; i < 5; ++i) {
            const float d = (float)(std::sqrt((double)(i * i + j * j)) / 5);
            const float t0 = d < 0.0f ? 0.0f : d;
            const float t = t0 > 1.0f ? 1.0f : t0;
            W.w[(j + 5) * 10 + (i + 5)] = gaussian_host(t, 0.4f, 0.0f);
        }
    return W;
}

thread_local std::string g_canvas_error;

int cfail(fs_canvas* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    else g_canvas_error = msg;
    return code;
}

int ccuda(fs_canvas* c, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return FS_OK;
    return cfail(c, e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

namespace fs {

View render_view(const float* area, int width, int height)
{
    View v;
    v.scale_x = (float)width / (area[1] - area[0]);
    v.scale_y = (float)height / (area[3] - area[2]);
    v.translate_x = (float)(0.5 * (double)(area[0] * (float)width));
    v.translate_y = (float)(0.5 * (double)(area[2] * (float)height));
    return v;
}

void render_clear(const Launch& L, fs_canvas* c)
{
    const int64_t n = (int64_t)c->width * c->height;
    k_fill<<<nblk(n), TPB, 0, L.stream>>>(c->px, n, 1.0f, 1.0f, 1.0f);  // Renderer::clearCanvas (Renderer.cpp:13-16)
    L.count();
}

void render_cells(const Launch& L, fs_canvas* c, const View& v, const Geom& g, const uint8_t* labels,
                  const float* level_set)
{
    const float csx = g.dx * v.scale_x, csy = g.dy * v.scale_y;
    k_cells<<<nblk((int64_t)c->width * c->height), TPB, 0, L.stream>>>(c->px, c->colors, c->width, c->height, v, csx,
                                                                        csy, g.nx, g.ny, labels, level_set);
    L.count();
}

void render_velocities(const Launch& L, fs_canvas* c, const View& v, const Geom& g, const float* uf, const float* vf)
{
    if (g.nx < 2 || g.ny < 2) return;
    const float csx = g.dx * v.scale_x, csy = g.dy * v.scale_y;
    const int64_t np = (int64_t)c->width * c->height;
    cudaMemsetAsync(c->owner, 0, 4 * (size_t)np, L.stream);
    k_vel_mark<<<nblk((int64_t)(g.nx - 1) * (g.ny - 1)), TPB, 0, L.stream>>>(c->owner, c->colors, c->width, c->height,
                                                                              v, csx, csy, g.nx, g.ny, uf, vf);
    k_vel_paint<<<nblk(np), TPB, 0, L.stream>>>(c->px, c->owner, c->width, c->height, v, csx, csy, g.nx, uf, vf);
    L.count(2);
}

void render_particles(const Launch& L, fs_canvas* c, const View& v, const float* px, const float* py, int64_t n)
{
    if (n == 0) {
        k_set_colors<<<1, 1, 0, L.stream>>>(c->colors, 0.3f, 0.6f, 0.9f, 0.3f, 0.6f, 0.9f);
        L.count();
        return;
    }
    k_particles<<<nblk(n), TPB, 0, L.stream>>>(c->px, c->colors, c->width, c->height, v, px, py, n);
    L.count();
}

cudaError_t render_metaballs(const Launch& L, fs_canvas* c, const View& v, const float* px, const float* py, int64_t n)
{
    const int w = c->width, h = c->height;
    const int64_t nbins = (int64_t)(w + 10) * (h + 10);
    if (n > c->cap_items) {
        for (void* p : {(void*)c->keys, (void*)c->pos, (void*)c->sorted}) cudaFree(p);
        c->keys = nullptr;
        c->pos = c->sorted = nullptr;
        c->cap_items = 0;
        cudaError_t e = cudaMalloc(&c->keys, 4 * (size_t)n);
        if (e == cudaSuccess) e = cudaMalloc(&c->pos, 8 * (size_t)n);
        if (e == cudaSuccess) e = cudaMalloc(&c->sorted, 4 * (size_t)n);
        if (e != cudaSuccess) return e;
        c->cap_items = n;
    }
    k_set_colors<<<1, 1, 0, L.stream>>>(c->colors, 0.5f, 0.9f, 1.0f, 0.0f, 0.5f, 0.7f);
    L.count();
    if (n > 0) {
        k_mb_keys<<<nblk(n), TPB, 0, L.stream>>>(w, h, v, px, py, n, (uint32_t)nbins, c->pos, c->keys);
        L.count();
    }
    group_by_key(L, n, c->keys, nbins, c->bin_count, c->bin_start, c->scan_tmp, c->sorted);
    k_mb_paint<<<nblk((int64_t)w * h), TPB, 0, L.stream>>>(c->px, w, h, c->pos, c->bin_start, c->sorted,
                                                            metaball_weights());
    L.count();
    return cudaSuccess;
}

}  // namespace fs

extern "C" {

const char* fs_canvas_last_error(const fs_canvas* c) { return c ? c->err.c_str() : g_canvas_error.c_str(); }

int fs_canvas_create(int width, int height, int device, fs_canvas** out)
{
    g_canvas_error.clear();
    if (!out || width < 1 || height < 1 || (int64_t)(width + 10) * (height + 10) > (int64_t)INT32_MAX / 4)
        return cfail(nullptr, FS_ERR_INVALID_ARGUMENT, "invalid canvas size");
    *out = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return ccuda(nullptr, e, "cudaSetDevice");
    fs_canvas* c = new fs_canvas();
    c->width = width;
    c->height = height;
    c->device = device;
    const size_t np = (size_t)width * height, nbins = (size_t)(width + 10) * (height + 10) + 1;
    auto A = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    A((void**)&c->px, 12 * np);
    A((void**)&c->colors, 6 * sizeof(float));
    A((void**)&c->owner, 4 * np);
    A((void**)&c->bin_count, 4 * nbins);
    A((void**)&c->bin_start, 4 * nbins);
    A((void**)&c->scan_tmp, 4 * scan_tmp_ints((int64_t)nbins));
    if (e == cudaSuccess) {
        // Canvas(width, height): pixels of Color() = white, line colour black, fill white (Canvas.cpp:5-33)
        k_fill<<<nblk((int64_t)np), TPB>>>(c->px, (int64_t)np, 1.0f, 1.0f, 1.0f);
        k_set_colors<<<1, 1>>>(c->colors, 0.0f, 0.0f, 0.0f, 1.0f, 1.0f, 1.0f);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        const int rc = ccuda(nullptr, e, "fs_canvas_create");
        fs_canvas_destroy(c);
        return rc;
    }
    *out = c;
    return FS_OK;
}

int fs_canvas_destroy(fs_canvas* c)
{
    if (!c) return FS_OK;
    cudaSetDevice(c->device);
    for (void* p : {(void*)c->px, (void*)c->colors, (void*)c->owner, (void*)c->keys, (void*)c->pos, (void*)c->sorted,
                    (void*)c->bin_count, (void*)c->bin_start, (void*)c->scan_tmp})
        cudaFree(p);
    delete c;
    return FS_OK;
}

int fs_canvas_set_pixels(fs_canvas* c, const float* rgb)
{
    if (!c || !rgb) return c ? cfail(c, FS_ERR_INVALID_ARGUMENT, "null pixels") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    return ccuda(c, cudaMemcpy(c->px, rgb, 12 * (size_t)c->width * c->height, cudaMemcpyHostToDevice), "pixels");
}

int fs_canvas_get_pixels(fs_canvas* c, float* rgb)
{
    if (!c || !rgb) return c ? cfail(c, FS_ERR_INVALID_ARGUMENT, "null pixels") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    return ccuda(c, cudaMemcpy(rgb, c->px, 12 * (size_t)c->width * c->height, cudaMemcpyDeviceToHost), "pixels");
}

int fs_canvas_set_colors(fs_canvas* c, const float* line_rgb, const float* fill_rgb)
{
    if (!c || !line_rgb || !fill_rgb) return c ? cfail(c, FS_ERR_INVALID_ARGUMENT, "null colour") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    float k[6] = {line_rgb[0], line_rgb[1], line_rgb[2], fill_rgb[0], fill_rgb[1], fill_rgb[2]};
    return ccuda(c, cudaMemcpy(c->colors, k, sizeof(k), cudaMemcpyHostToDevice), "colours");
}

int fs_canvas_get_colors(fs_canvas* c, float* line_rgb, float* fill_rgb)
{
    if (!c || !line_rgb || !fill_rgb) return c ? cfail(c, FS_ERR_INVALID_ARGUMENT, "null colour") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    float k[6];
    const int rc = ccuda(c, cudaMemcpy(k, c->colors, sizeof(k), cudaMemcpyDeviceToHost), "colours");
    if (rc) return rc;
    std::memcpy(line_rgb, k, 3 * sizeof(float));
    std::memcpy(fill_rgb, k + 3, 3 * sizeof(float));
    return FS_OK;
}

int fs_canvas_get_bytes(fs_canvas* c, uint8_t* rgb8)
{
    if (!c || !rgb8) return c ? cfail(c, FS_ERR_INVALID_ARGUMENT, "null output") : FS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const int64_t n = 3 * (int64_t)c->width * c->height;
    uint8_t* d = nullptr;
    cudaError_t e = cudaMalloc(&d, (size_t)n);
    if (e == cudaSuccess) {
        k_bytes<<<nblk(n), TPB>>>(c->px, n, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(rgb8, d, (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return ccuda(c, e, "canvas bytes");
}

int fs_canvas_write_ppm(fs_canvas* c, const char* path)
{
    if (!c || !path) return c ? cfail(c, FS_ERR_INVALID_ARGUMENT, "null path") : FS_ERR_INVALID_ARGUMENT;
    std::vector<uint8_t> bytes(3 * (size_t)c->width * c->height);
    const int rc = fs_canvas_get_bytes(c, bytes.data());
    if (rc) return rc;
    std::FILE* f = std::fopen(path, "wb");  // Renderer::writeCanvasToPpm (Renderer.cpp:242-247)
    if (!f) return cfail(c, FS_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    std::fprintf(f, "P6\n%d %d\n255\n", c->width, c->height);
    const size_t wrote = std::fwrite(bytes.data(), 1, bytes.size(), f);
    std::fclose(f);
    return wrote == bytes.size() ? FS_OK : cfail(c, FS_ERR_INVALID_ARGUMENT, "short write");
}

int64_t fs_canvas_kernel_launches(const fs_canvas* c) { return c ? c->launches : 0; }

}  // extern "C"
