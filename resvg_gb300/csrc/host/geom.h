// Host-side path geometry: tight bounds, stroke outlining and dashing.
//
// In resvg these run on the host inside tiny-skia-path: `Path::stroke`
// (crates/resvg/src/path.rs:113 via Pixmap::stroke_path), `Path::dash`
// (usvg `Stroke::to_tiny_skia`, crates/usvg/src/tree/mod.rs:638-663) and
// `Path::compute_tight_bounds` (tree/mod.rs:1321,1452).  The GPU backend keeps
// them on the host, as the reference does; both the GPU renderer and the CPU
// oracle consume the outlines produced here, so stroke geometry is an input to
// the raster parity check rather than part of it.
#pragma once
#include <cstdint>
#include <vector>

namespace rgpu {

struct PathData {
    std::vector<uint8_t> verbs;  // rgpu_verb
    std::vector<float> pts;      // x,y pairs
    void move_to(float x, float y) { verbs.push_back(0); pts.push_back(x); pts.push_back(y); }
    void line_to(float x, float y) { verbs.push_back(1); pts.push_back(x); pts.push_back(y); }
    void quad_to(float x1, float y1, float x, float y) {
        verbs.push_back(2); pts.push_back(x1); pts.push_back(y1); pts.push_back(x); pts.push_back(y);
    }
    void cubic_to(float x1, float y1, float x2, float y2, float x, float y) {
        verbs.push_back(3);
        pts.insert(pts.end(), {x1, y1, x2, y2, x, y});
    }
    void close() { verbs.push_back(4); }
    bool empty() const { return verbs.empty(); }
};

struct StrokeStyle {
    float width = 1.0f;
    float miter_limit = 4.0f;
    uint32_t cap = 0;   // rgpu_cap
    uint32_t join = 0;  // rgpu_join
};

// Tight bounds (curve extrema included).  Returns false for empty/non-finite.
bool tight_bounds(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, float out[4]);

// Stroke outline, to be filled with the non-zero rule.  `res_scale` is the
// device/user scale (tiny-skia's compute_resolution_scale) and sets the curve
// flattening tolerance.  Returns false when nothing is produced.
bool stroke_path(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, const StrokeStyle &st,
                 float res_scale, PathData &out);

// Dash a path (SVG stroke-dasharray/offset).  Returns false when the dash
// array is invalid (all zero) — the caller then strokes the undashed path.
bool dash_path(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, const float *dashes, size_t nd,
               float offset, float res_scale, PathData &out);

// tiny-skia PathStroker::compute_resolution_scale for a transform.
float resolution_scale(float sx, float ky, float kx, float sy);

}  // namespace rgpu
