// CPU oracle — test infrastructure only.
//
// A sequential restatement of the raster layer resvg 0.48.1 renders through:
// tiny-skia 0.12.0 / tiny-skia-path 0.12.0 (pinned in Cargo.lock, NOT vendored
// in the reference tree).  Their algorithms are Skia's published ones
// (SkEdge, SkEdgeBuilder, SkEdgeClipper, SkScan_Path, SkScan_AntiPath,
// SkRasterPipeline lowp/highp); this file restates them from that public
// description.  Call sites in the reference that define the contract:
//   crates/resvg/src/path.rs:73,113      Pixmap::fill_path / stroke_path
//   crates/resvg/src/render.rs:133       Pixmap::draw_pixmap
//   crates/resvg/src/clip.rs:11-27,88    Pixmap::fill, Mask::from_pixmap/invert, apply_mask
//   crates/resvg/src/mask.rs:13-45       Mask::fill_path, Mask::from_pixmap
// Parity of this restatement with tiny-skia is pinned only by resvg's golden
// PNGs (crates/resvg/tests/tests/**) — see tests/test_golden.py.
//
// Nothing in the product may include or link this file.
#pragma once
#include <cstdint>
#include <cmath>
#include <memory>
#include <vector>
#include "rgpu_tree.h"

namespace ora {

struct Point { float x, y; };

struct Rect {
    float l, t, r, b;
    float w() const { return r - l; }
    float h() const { return b - t; }
};

struct IntRect {
    int32_t x, y;
    int32_t w, h;
    int32_t right() const { return x + w; }
    int32_t bottom() const { return y + h; }
};

struct Transform {
    float sx = 1, ky = 0, kx = 0, sy = 1, tx = 0, ty = 0;
    static Transform from_row(float sx, float ky, float kx, float sy, float tx, float ty) {
        Transform t; t.sx = sx; t.ky = ky; t.kx = kx; t.sy = sy; t.tx = tx; t.ty = ty; return t;
    }
    static Transform translate(float x, float y) { return from_row(1, 0, 0, 1, x, y); }
    static Transform scale(float x, float y) { return from_row(x, 0, 0, y, 0, 0); }
    static Transform from(const rgpu_transform &r) { return from_row(r.sx, r.ky, r.kx, r.sy, r.tx, r.ty); }
    bool is_identity() const { return sx == 1 && ky == 0 && kx == 0 && sy == 1 && tx == 0 && ty == 0; }
    bool has_skew() const { return kx != 0 || ky != 0; }
    bool has_scale() const { return sx != 1 || sy != 1; }
    bool has_translate() const { return tx != 0 || ty != 0; }
    bool is_scale_translate() const { return !has_skew(); }
    bool is_translate() const { return !has_skew() && !has_scale(); }
    Transform pre_concat(const Transform &o) const;
    Transform post_concat(const Transform &o) const;
    Transform pre_translate(float x, float y) const { return pre_concat(translate(x, y)); }
    Transform pre_scale(float x, float y) const { return pre_concat(scale(x, y)); }
    bool invert(Transform *out) const;
    void map_points(Point *p, size_t n) const;
    void get_scale(float *x, float *y) const;
    bool is_finite() const;
};

struct Path {
    std::vector<uint8_t> verbs;   // rgpu_verb
    std::vector<Point> pts;
    Rect bounds{0, 0, 0, 0};
    void compute_bounds();
    bool transform(const Transform &ts);  // false on non-finite result
};

// Pixmap: premultiplied RGBA8, row-major.
struct Pixmap {
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> data;
    Pixmap() {}
    Pixmap(uint32_t w, uint32_t h) : width(w), height(h), data((size_t)w * h * 4, 0) {}
    uint8_t *px(uint32_t x, uint32_t y) { return &data[((size_t)y * width + x) * 4]; }
    const uint8_t *px(uint32_t x, uint32_t y) const { return &data[((size_t)y * width + x) * 4]; }
};

struct Mask {
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> data;
    Mask() {}
    Mask(uint32_t w, uint32_t h) : width(w), height(h), data((size_t)w * h, 0) {}
};

struct ColorF { float r, g, b, a; };

struct GradientStop { float pos; ColorF color; };

enum ShaderKind { SHADER_SOLID, SHADER_LINEAR, SHADER_RADIAL, SHADER_PATTERN };

// A tiny-skia Shader: solid colour, linear gradient, two-point conical radial
// gradient, or a pixmap pattern (nearest, identity/translate only — what
// draw_pixmap needs).
struct Shader {
    ShaderKind kind = SHADER_SOLID;
    ColorF color{0, 0, 0, 1};
    // gradients
    std::vector<GradientStop> stops;
    uint32_t spread = RGPU_SPREAD_PAD;
    Transform transform;          // gradient -> user space (gradientTransform, then paint transform)
    Point p0{0, 0}, p1{0, 0};     // linear start/end; radial: start(focal), end(centre)
    float r0 = 0, r1 = 0;         // radial radii (focal radius, radius)
    // pattern: the tile pixmap (kept alive by pattern_owner), sampled through
    // `transform` (tile -> user space, then the paint transform) with Repeat
    // tiling, bicubic unless the transform is a pure translation
    const Pixmap *pattern = nullptr;
    std::shared_ptr<Pixmap> pattern_owner;
    int quality = 2;              // 0 nearest, 1 bilinear, 2 bicubic; `spread` repeat or pad
    float opacity = 1;
    bool is_opaque() const;
};

struct Paint {
    Shader shader;
    uint32_t blend = RGPU_BLEND_SOURCE_OVER;
    bool anti_alias = true;
};

// tiny-skia Pixmap::fill_path (painter.rs).
void fill_path(Pixmap &pm, const Path &path, const Paint &paint, uint32_t rule, const Transform &ts);
// tiny-skia's anti-aliased hairline (scan/hairline_aa.rs do_anti_hairline and
// its four blitters) for a list of fixed-point line calls, drawn with `paint`
// (already opacity-scaled; its shader in device space).  call = {x0, y0, x1,
// y1 (FDot6), clip l, t, r, b, has_clip}.
void anti_hairlines(Pixmap &pm, const Paint &paint, const int32_t *calls, size_t ncalls);
// tiny-skia Pixmap::fill_rect for an integer-aligned rect, no AA (painter.rs).
void fill_rect(Pixmap &pm, const Rect &r, const Paint &paint);
// tiny-skia Pixmap::draw_pixmap (painter.rs): pattern + fill_rect, highp.
void draw_pixmap(Pixmap &dst, int32_t x, int32_t y, const Pixmap &src, float opacity, uint32_t blend);
// tiny-skia Pixmap::fill(Color).
void pixmap_fill(Pixmap &pm, ColorF c);
// tiny-skia Mask::from_pixmap / invert / Pixmap::apply_mask / Mask::fill_path.
Mask mask_from_pixmap(const Pixmap &pm, bool luminance);
void mask_invert(Mask &m);
void apply_mask(Pixmap &pm, const Mask &m);
void mask_fill_path(Mask &m, const Path &path, uint32_t rule, bool aa, const Transform &ts);

// Host-side helpers shared with the render module.
Rect rect_transform(const Rect &r, const Transform &ts, bool *ok);
bool rect_to_int_rect(const Rect &r, IntRect *out);
int32_t sat_i32(float v);
int32_t sat_i32d(double v);
uint8_t to_u8_norm(float v);   // strict-num NormalizedF32::to_u8
ColorF color_from_rgba8(uint8_t r, uint8_t g, uint8_t b, uint8_t a);

}  // namespace ora
