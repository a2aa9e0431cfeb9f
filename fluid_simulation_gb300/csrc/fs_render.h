// Headless renderer (src/Renderer.cpp, src/Canvas.cpp on the GPU): the canvas
// object and the render passes the C ABI of fs_api.cu drives with a handle's
// state.
#pragma once

#include <string>

#include "fs_internal.h"

struct fs_canvas
{
    int width = 0, height = 0;
    int device = 0;
    float* px = nullptr;      // 3 floats per pixel, row-major (Canvas::_pixel_data)
    float* colors = nullptr;  // line colour, fill colour (Canvas::_line_color / _fill_color), device
    int32_t* owner = nullptr;  // per pixel: 1 + index of the last line drawn there
    // metaball scratch (allocated on first use)
    uint32_t* keys = nullptr;
    int32_t *pos = nullptr, *sorted = nullptr, *bin_count = nullptr, *bin_start = nullptr, *scan_tmp = nullptr;
    int64_t cap_items = 0;
    int64_t launches = 0;
    std::string err;
};

namespace fs {

// The pixel mapping of every Renderer function (src/Renderer.cpp:23-27).
struct View
{
    float scale_x, scale_y, translate_x, translate_y;
};
View render_view(const float* area, int width, int height);

// The render passes, on L.stream (st = the simulation's state).
void render_clear(const Launch& L, fs_canvas* c);
// labels' cell types, or with level_set non-null the level-set values
void render_cells(const Launch& L, fs_canvas* c, const View& v, const Geom& g, const uint8_t* labels,
                  const float* level_set);
void render_velocities(const Launch& L, fs_canvas* c, const View& v, const Geom& g, const float* uf, const float* vf);
void render_particles(const Launch& L, fs_canvas* c, const View& v, const float* px, const float* py, int64_t n);
cudaError_t render_metaballs(const Launch& L, fs_canvas* c, const View& v, const float* px, const float* py, int64_t n);

}  // namespace fs
