// CPU oracle — test infrastructure only.
//
// Restatement of resvg 0.48.1's renderer over the raster layer in raster.cpp:
//   crates/resvg/src/lib.rs:34-43,86-97   render, max_filter_bbox
//   crates/resvg/src/render.rs:10-142     render_nodes / render_node / render_group
//   crates/resvg/src/path.rs:6-177        paint order, fill_path, stroke_path, gradients
//   crates/resvg/src/clip.rs:6-98         clip::apply, draw_children, clip_group
//   crates/resvg/src/mask.rs:6-46         mask::apply
//   crates/resvg/src/geom.rs:5-30         fit_to_rect
// Filters are in filter.cpp.  Strokes are outlined by the host stroker
// (resvg_gb300/csrc/host/geom.cpp), the same input preparation the GPU path uses.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "raster.h"
#include "../resvg_gb300/csrc/host/hairline.h"
#include "../resvg_gb300/csrc/host/tree.h"

namespace ora {

bool filter_apply(const rgpu_tree_view &t, const rgpu_filter &f, const Transform &ts, Pixmap &source);

namespace {

struct Ctx {
    const rgpu_tree_view &t;
    IntRect max_bbox;
};

bool fit_to_rect(const IntRect &r, const IntRect &b, IntRect *out) {
    int32_t l = std::max(r.x, b.x), t = std::max(r.y, b.y);
    int32_t rr = std::min(r.right(), b.right()), bb = std::min(r.bottom(), b.bottom());
    if (rr <= l || bb <= t) return false;
    *out = IntRect{l, t, rr - l, bb - t};
    return true;
}

Path tree_path(const rgpu_tree_view &t, const rgpu_path &p) {
    Path out;
    out.verbs.assign(t.verbs + p.verb_offset, t.verbs + p.verb_offset + p.verb_count);
    out.pts.resize(p.point_count);
    for (uint32_t i = 0; i < p.point_count; i++)
        out.pts[i] = Point{t.points[2 * (p.point_offset + i)], t.points[2 * (p.point_offset + i) + 1]};
    out.compute_bounds();
    return out;
}

// path.rs:118-177 (convert_linear/radial/base_gradient) + tiny-skia shader constructors.
void render_nodes(Ctx &c, uint32_t group, const Transform &ts, Pixmap &pm);

// path.rs:179-205 render_pattern_pixmap + the Pattern shader it makes: the
// tile is the pattern content at the fill's device scale, sampled back through
// patternTransform * translate(rect) * scale(1 / scale).
bool make_pattern(Ctx &c, const rgpu_paint &pp, float opacity, const Transform &ts, Shader &sh) {
    const Transform pts = Transform::from(pp.transform);
    float sx, sy;
    ts.pre_concat(pts).get_scale(&sx, &sy);
    auto to_u32 = [](float v) -> uint32_t {
        v = std::round(v);
        if (!(v > 0.0f)) return 0;
        if (v >= 4294967296.0f) return 0xFFFFFFFFu;
        return (uint32_t)v;
    };
    const uint32_t iw = to_u32(pp.x2 * sx), ih = to_u32(pp.y2 * sy);
    if (!iw || !ih || (uint64_t)iw * ih > ((uint64_t)1 << 26)) return false;
    if (pp.stop_offset >= c.t.group_count) return false;
    auto tile = std::make_shared<Pixmap>(iw, ih);
    render_nodes(c, pp.stop_offset, Transform::scale(sx, sy), *tile);
    sh.kind = SHADER_PATTERN;
    sh.pattern = tile.get();
    sh.pattern_owner = tile;
    sh.spread = RGPU_SPREAD_REPEAT;
    sh.quality = 2;
    sh.opacity = opacity;
    sh.transform = pts.pre_concat(Transform::translate(pp.x1, pp.y1)).pre_concat(Transform::scale(1.0f / sx, 1.0f / sy));
    return true;
}

bool make_shader(const rgpu_tree_view &t, int32_t paint_idx, float opacity, Shader &sh) {
    const rgpu_paint &pp = t.paints[paint_idx];
    if (pp.kind == RGPU_PAINT_PATTERN) return false;  // make_pattern: needs the path transform
    if (pp.kind == RGPU_PAINT_IMAGE) {
        // image.rs render_raster: Pattern(raster, Pad, quality, opacity 1, identity)
        if (pp.stop_offset >= t.image_count) return false;
        const rgpu_image &im = t.images[pp.stop_offset];
        auto tile = std::make_shared<Pixmap>(im.width, im.height);
        std::memcpy(tile->data.data(), t.image_pixels + im.pixel_offset, (size_t)im.width * im.height * 4);
        sh.kind = SHADER_PATTERN;
        sh.pattern = tile.get();
        sh.pattern_owner = tile;
        sh.spread = RGPU_SPREAD_PAD;
        sh.quality = (int)std::min<uint32_t>(pp.spread, 2u);
        sh.opacity = 1.0f;
        sh.transform = Transform();
        return true;
    }
    uint8_t a8 = to_u8_norm(opacity);
    if (pp.kind == RGPU_PAINT_SOLID) {
        sh.kind = SHADER_SOLID;
        sh.color = color_from_rgba8(pp.r, pp.g, pp.b, a8);
        return true;
    }
    std::vector<GradientStop> stops;
    for (uint32_t i = 0; i < pp.stop_count; i++) {
        const rgpu_stop &s = t.stops[pp.stop_offset + i];
        float alpha = s.opacity * opacity;
        stops.push_back(GradientStop{s.offset, color_from_rgba8(s.r, s.g, s.b, to_u8_norm(alpha))});
    }
    if (stops.empty()) return false;
    if (stops.size() == 1) {
        sh.kind = SHADER_SOLID;
        sh.color = stops[0].color;
        return true;
    }
    Transform gts = Transform::from(pp.transform);
    if (pp.kind == RGPU_PAINT_LINEAR) {
        float dx = pp.x2 - pp.x1, dy = pp.y2 - pp.y1;
        float length = std::sqrt(dx * dx + dy * dy);
        if (!std::isfinite(length)) return false;
        if (length <= 1.0f / (1 << 15)) {
            sh.kind = SHADER_SOLID;
            sh.color = stops.back().color;
            return true;
        }
        Transform inv;
        if (!gts.invert(&inv)) return false;
        sh.kind = SHADER_LINEAR;
        sh.p0 = Point{pp.x1, pp.y1};
        sh.p1 = Point{pp.x2, pp.y2};
    } else {
        if (!(pp.r_ > 0)) return false;
        Transform inv;
        if (!gts.invert(&inv)) return false;
        sh.kind = SHADER_RADIAL;
        sh.p0 = Point{pp.fx, pp.fy};
        sh.r0 = pp.fr;
        sh.p1 = Point{pp.cx, pp.cy};
        sh.r1 = pp.r_;
    }
    sh.stops = stops;
    sh.spread = pp.spread;
    sh.transform = gts;
    return true;
}

void fill_path_node(Ctx &c, const rgpu_path &p, uint32_t blend, const Transform &ts, Pixmap &pm) {
    if (p.fill_paint < 0) return;
    Path path = tree_path(c.t, p);
    if (path.bounds.w() == 0.0f || path.bounds.h() == 0.0f) return;
    Paint paint;
    if (c.t.paints[p.fill_paint].kind == RGPU_PAINT_PATTERN) {
        if (!make_pattern(c, c.t.paints[p.fill_paint], p.fill_opacity, ts, paint.shader)) return;
    } else if (!make_shader(c.t, p.fill_paint, p.fill_opacity, paint.shader)) {
        return;
    }
    paint.anti_alias = p.anti_alias != 0;
    paint.blend = blend;
    fill_path(pm, path, paint, p.fill_rule, ts);
}

// BlendMode::should_pre_scale_coverage (tiny-skia blend_mode.rs)
bool pre_scale_blend(uint32_t b) {
    return b == RGPU_BLEND_DESTINATION || b == RGPU_BLEND_DESTINATION_OVER || b == RGPU_BLEND_PLUS ||
           b == RGPU_BLEND_DESTINATION_OUT || b == RGPU_BLEND_SOURCE_ATOP || b == RGPU_BLEND_SOURCE_OVER ||
           b == RGPU_BLEND_XOR;
}

void stroke_path_node(Ctx &c, uint32_t pi, uint32_t blend, const Transform &ts, Pixmap &pm) {
    const rgpu_path &p = c.t.paths[pi];
    if (p.stroke_paint < 0) return;
    Paint paint;
    if (c.t.paints[p.stroke_paint].kind == RGPU_PAINT_PATTERN) {
        if (!make_pattern(c, c.t.paints[p.stroke_paint], p.stroke_opacity, ts, paint.shader)) return;
    } else if (!make_shader(c.t, p.stroke_paint, p.stroke_opacity, paint.shader)) {
        return;
    }
    paint.anti_alias = p.anti_alias != 0;
    paint.blend = blend;
    float rs = rgpu::resolution_scale(ts.sx, ts.ky, ts.kx, ts.sy);
    // tiny-skia stroke_path: a stroke at most one device pixel wide is an
    // anti-aliased hairline of the (dashed) path, its paint scaled by coverage
    const rgpu::Xf xts = rgpu::Xf::row(ts.sx, ts.ky, ts.kx, ts.sy, ts.tx, ts.ty);
    float coverage = 1.0f;
    if (rgpu::treat_as_hairline(paint.anti_alias, p.stroke_width, xts, &coverage)) {
        rgpu::PathData src;
        if (!rgpu::hairline_source_view(c.t, pi, rs, src)) return;
        if (coverage != 1.0f && pre_scale_blend(blend)) {
            const float op = rgpu::hairline_opacity(coverage);
            auto scale = [op](ColorF &col) { col.a = std::min(std::max(col.a * std::min(std::max(op, 0.0f), 1.0f), 0.0f), 1.0f); };
            if (paint.shader.kind == SHADER_SOLID) scale(paint.shader.color);
            for (auto &st : paint.shader.stops) scale(st.color);
            if (paint.shader.kind == SHADER_PATTERN)
                paint.shader.opacity = std::min(std::max(paint.shader.opacity * std::min(std::max(op, 0.0f), 1.0f), 0.0f), 1.0f);
        }
        std::vector<rgpu::HairCall> calls;
        rgpu::hairline_calls(src, xts, p.line_cap, (int32_t)pm.width, (int32_t)pm.height, calls);
        if (!ts.is_identity() && paint.shader.kind != SHADER_SOLID)
            paint.shader.transform = paint.shader.transform.post_concat(ts);
        anti_hairlines(pm, paint, reinterpret_cast<const int32_t *>(calls.data()), calls.size());
        return;
    }
    rgpu::PathData out;
    if (!rgpu::stroke_outline_view(c.t, pi, rs, out)) return;
    Path sp;
    sp.verbs = out.verbs;
    sp.pts.resize(out.pts.size() / 2);
    for (size_t i = 0; i < sp.pts.size(); i++) sp.pts[i] = Point{out.pts[2 * i], out.pts[2 * i + 1]};
    sp.compute_bounds();
    fill_path(pm, sp, paint, RGPU_NONZERO, ts);
}

void render_nodes(Ctx &c, uint32_t group, const Transform &ts, Pixmap &pm);

void render_path(Ctx &c, uint32_t pi, const Transform &ts, Pixmap &pm) {
    const rgpu_path &p = c.t.paths[pi];
    if (!p.visible) return;
    if (!p.stroke_first) {
        fill_path_node(c, p, RGPU_BLEND_SOURCE_OVER, ts, pm);
        stroke_path_node(c, pi, RGPU_BLEND_SOURCE_OVER, ts, pm);
    } else {
        stroke_path_node(c, pi, RGPU_BLEND_SOURCE_OVER, ts, pm);
        fill_path_node(c, p, RGPU_BLEND_SOURCE_OVER, ts, pm);
    }
}

void clip_apply(Ctx &c, const rgpu_clip &clip, const Transform &ts, Pixmap &pm);

// clip.rs:30-68
void draw_children(Ctx &c, uint32_t group, uint32_t mode, const Transform &ts, Pixmap &pm);
// clip.rs:70-98
void clip_group(Ctx &c, uint32_t group, const rgpu_clip &clip, const Transform &ts, Pixmap &pm) {
    Pixmap cp(pm.width, pm.height);
    draw_children(c, group, RGPU_BLEND_SOURCE_OVER, ts, cp);
    clip_apply(c, clip, ts, cp);
    draw_pixmap(pm, 0, 0, cp, 1.0f, RGPU_BLEND_XOR);
}
void draw_children(Ctx &c, uint32_t group, uint32_t mode, const Transform &ts, Pixmap &pm) {
    const rgpu_group &g = c.t.groups[group];
    for (uint32_t k = 0; k < g.child_count; k++) {
        const rgpu_node &n = c.t.children[g.child_offset + k];
        if (n.kind == RGPU_NODE_PATH) {
            const rgpu_path &p = c.t.paths[n.index];
            if (!p.visible) continue;
            fill_path_node(c, p, mode, ts, pm);
        } else {
            const rgpu_group &cg = c.t.groups[n.index];
            Transform t2 = ts.pre_concat(Transform::from(cg.transform));
            if (cg.clip_path >= 0) clip_group(c, n.index, c.t.clips[cg.clip_path], t2, pm);
            else draw_children(c, n.index, mode, t2, pm);
        }
    }
}
// clip.rs:6-28
void clip_apply(Ctx &c, const rgpu_clip &clip, const Transform &ts, Pixmap &pm) {
    Pixmap cp(pm.width, pm.height);
    pixmap_fill(cp, ColorF{0, 0, 0, 1});
    draw_children(c, clip.root, RGPU_BLEND_CLEAR, ts.pre_concat(Transform::from(clip.transform)), cp);
    if (clip.clip_path >= 0) clip_apply(c, c.t.clips[clip.clip_path], ts, pm);
    Mask m = mask_from_pixmap(cp, false);
    mask_invert(m);
    apply_mask(pm, m);
}
// mask.rs:6-46
void mask_apply(Ctx &c, const rgpu_mask &mask, const Transform &ts, Pixmap &pm) {
    if (c.t.groups[mask.root].child_count == 0) {
        pixmap_fill(pm, ColorF{0, 0, 0, 0});
        return;
    }
    Pixmap mp(pm.width, pm.height);
    {
        Mask region(pm.width, pm.height);
        Path rect;
        rect.verbs = {RGPU_MOVE, RGPU_LINE, RGPU_LINE, RGPU_LINE, RGPU_CLOSE};
        rect.pts = {{mask.x, mask.y}, {mask.x + mask.w, mask.y}, {mask.x + mask.w, mask.y + mask.h},
                    {mask.x, mask.y + mask.h}};
        rect.compute_bounds();
        mask_fill_path(region, rect, RGPU_NONZERO, true, ts);
        render_nodes(c, mask.root, ts, mp);
        apply_mask(mp, region);
    }
    if (mask.mask >= 0) mask_apply(c, c.t.masks[mask.mask], ts, pm);
    Mask m = mask_from_pixmap(mp, mask.kind == RGPU_MASK_LUMINANCE);
    apply_mask(pm, m);
}

bool should_isolate(const rgpu_group &g) {
    return g.isolate || g.opacity != 1.0f || g.clip_path >= 0 || g.mask >= 0 || g.filter_count > 0 ||
           g.blend != RGPU_BLEND_SOURCE_OVER;
}

// render.rs:49-142
void render_group(Ctx &c, uint32_t gi, const Transform &ts_in, Pixmap &pm) {
    const rgpu_group &g = c.t.groups[gi];
    Transform ts = ts_in.pre_concat(Transform::from(g.transform));
    if (!should_isolate(g)) {
        render_nodes(c, gi, ts, pm);
        return;
    }
    if (!g.has_layer_bbox) return;
    bool ok;
    Rect lb{g.layer_x, g.layer_y, g.layer_x + g.layer_w, g.layer_y + g.layer_h};
    Rect bbox = rect_transform(lb, ts, &ok);
    if (!ok) return;
    IntRect ib;
    if (g.filter_count == 0) {
        int64_t x = (int64_t)sat_i32(std::floor(bbox.l)) - 2, y = (int64_t)sat_i32(std::floor(bbox.t)) - 2;
        int64_t w = (int64_t)(uint32_t)std::max(0.0f, std::ceil(bbox.w())) + 4;
        int64_t h = (int64_t)(uint32_t)std::max(0.0f, std::ceil(bbox.h())) + 4;
        if (x < INT32_MIN || y < INT32_MIN || x + w > INT32_MAX || y + h > INT32_MAX) return;
        ib = IntRect{(int32_t)x, (int32_t)y, (int32_t)w, (int32_t)h};
        if (!fit_to_rect(ib, c.max_bbox, &ib)) return;
    } else {
        int64_t x = sat_i32(std::floor(bbox.l)), y = sat_i32(std::floor(bbox.t));
        int64_t w = (int64_t)std::max(1.0f, std::ceil(bbox.w()));
        int64_t h = (int64_t)std::max(1.0f, std::ceil(bbox.h()));
        if (x + w > INT32_MAX || y + h > INT32_MAX) return;
        ib = IntRect{(int32_t)x, (int32_t)y, (int32_t)w, (int32_t)h};
        if (!fit_to_rect(ib, c.max_bbox, &ib)) return;
    }
    float dx = bbox.l, dy = bbox.t;
    dx -= bbox.l - (float)ib.x;
    dy -= bbox.t - (float)ib.y;
    Transform lts = Transform::translate(-dx, -dy).pre_concat(ts);
    Pixmap sub((uint32_t)ib.w, (uint32_t)ib.h);
    render_nodes(c, gi, lts, sub);
    for (uint32_t k = 0; k < g.filter_count; k++)
        filter_apply(c.t, c.t.filters[c.t.filter_refs[g.filter_offset + k]], lts, sub);
    if (g.clip_path >= 0) clip_apply(c, c.t.clips[g.clip_path], lts, sub);
    if (g.mask >= 0) mask_apply(c, c.t.masks[g.mask], lts, sub);
    draw_pixmap(pm, ib.x, ib.y, sub, g.opacity, g.blend);
}

void render_nodes(Ctx &c, uint32_t group, const Transform &ts, Pixmap &pm) {
    const rgpu_group &g = c.t.groups[group];
    for (uint32_t k = 0; k < g.child_count; k++) {
        const rgpu_node &n = c.t.children[g.child_offset + k];
        if (n.kind == RGPU_NODE_PATH) render_path(c, n.index, ts, pm);
        else render_group(c, n.index, ts, pm);
    }
}

IntRect max_filter_bbox(uint32_t w, uint32_t h) {
    int64_t x = -2 * (int64_t)w, y = -2 * (int64_t)h, ww = 5 * (int64_t)w, hh = 5 * (int64_t)h;
    if (x < INT32_MIN / 2 || ww > INT32_MAX) return IntRect{INT32_MIN / 2, INT32_MIN / 2, INT32_MAX, INT32_MAX};
    return IntRect{(int32_t)x, (int32_t)y, (int32_t)ww, (int32_t)hh};
}

}  // namespace

// filter/mod.rs:861-889 (apply_image): a group's children rendered into a
// pixmap whose own bounds are the layer limit
void render_group_children(const rgpu_tree_view &t, uint32_t gi, const Transform &ts, Pixmap &pm) {
    Ctx c{t, IntRect{0, 0, (int32_t)pm.width, (int32_t)pm.height}};
    render_nodes(c, gi, ts, pm);
}

// lib.rs:34-43
void render_tree(const rgpu_tree_view &t, const Transform &ts, Pixmap &pm) {
    Ctx c{t, max_filter_bbox(pm.width, pm.height)};
    if (t.group_count == 0) return;
    render_nodes(c, 0, ts, pm);
}

// lib.rs:55-70 (resvg::render_node) behind the C API's id lookup
// (crates/c-api/lib.rs:908-942).  Ids: "<n>" is group n, "p<n>" is path n.
bool render_node_id(const rgpu_tree_view &t, const char *id, const Transform &ts_in, Pixmap &pm) {
    if (!id || !*id) return false;
    const bool is_path = id[0] == 'p';
    char *end = nullptr;
    const unsigned long idx = std::strtoul(id + (is_path ? 1 : 0), &end, 10);
    if (!end || *end || end == id + (is_path ? 1 : 0)) return false;
    if (idx >= (is_path ? (unsigned long)t.path_count : (unsigned long)t.group_count)) return false;
    std::vector<int32_t> gp(t.group_count, -1), pp(t.path_count, -1);
    for (uint32_t g = 0; g < t.group_count; g++)
        for (uint32_t k = 0; k < t.groups[g].child_count; k++) {
            const rgpu_node &n = t.children[t.groups[g].child_offset + k];
            (n.kind == RGPU_NODE_GROUP ? gp : pp)[n.index] = (int32_t)g;
        }
    auto tf = [](const rgpu_transform &x) { return Transform::from_row(x.sx, x.ky, x.kx, x.sy, x.tx, x.ty); };
    Transform abs = is_path ? Transform() : tf(t.groups[idx].transform);
    for (int32_t g = is_path ? pp[idx] : gp[idx]; g >= 0; g = gp[g]) abs = tf(t.groups[g].transform).pre_concat(abs);
    Rect r;
    if (is_path) {
        const rgpu_path &p = t.paths[idx];
        r = Rect{p.bbox_x, p.bbox_y, p.bbox_x + p.bbox_w, p.bbox_y + p.bbox_h};
    } else {
        const rgpu_group &g = t.groups[idx];
        if (!g.has_layer_bbox) return false;
        r = Rect{g.layer_x, g.layer_y, g.layer_x + g.layer_w, g.layer_y + g.layer_h};
    }
    if (!(r.r > r.l && r.b > r.t)) return false;
    // NonZeroRect::transform: bounds of the mapped corners
    Point c[4] = {{r.l, r.t}, {r.r, r.t}, {r.r, r.b}, {r.l, r.b}};
    abs.map_points(c, 4);
    float l = c[0].x, tp = c[0].y, rr = c[0].x, b = c[0].y;
    for (int i = 1; i < 4; i++) {
        l = std::min(l, c[i].x); rr = std::max(rr, c[i].x);
        tp = std::min(tp, c[i].y); b = std::max(b, c[i].y);
    }
    if (!(rr > l && b > tp)) return false;
    Transform ts = ts_in.pre_concat(Transform::translate(-l, -tp));
    Ctx cx{t, max_filter_bbox(pm.width, pm.height)};
    if (is_path) render_path(cx, (uint32_t)idx, ts, pm);
    else render_group(cx, (uint32_t)idx, ts, pm);
    return true;
}

}  // namespace ora

// ---------------------------------------------------------------- C entry points (tests / bench only)
extern "C" {

// resvg_render_node with the same id convention as the product's.
int oracle_render_node(const rgpu_tree_view *tree, const char *id, const float ts6[6], uint32_t w, uint32_t h,
                       uint8_t *pixmap) {
    if (!tree || !pixmap || w == 0 || h == 0) return -1;
    ora::Pixmap pm(w, h);
    std::memcpy(pm.data.data(), pixmap, (size_t)w * h * 4);
    ora::Transform ts = ora::Transform::from_row(ts6[0], ts6[1], ts6[2], ts6[3], ts6[4], ts6[5]);
    if (!ora::render_node_id(*tree, id, ts, pm)) return 1;
    std::memcpy(pixmap, pm.data.data(), (size_t)w * h * 4);
    return 0;
}

// Renders `tree` onto the premultiplied RGBA8 `pixmap` (w*h*4 bytes), drawing
// onto its existing content, as resvg_render does.
int oracle_render(const rgpu_tree_view *tree, const float ts6[6], uint32_t w, uint32_t h, uint8_t *pixmap) {
    if (!tree || !pixmap || w == 0 || h == 0) return -1;
    ora::Pixmap pm(w, h);
    std::memcpy(pm.data.data(), pixmap, (size_t)w * h * 4);
    ora::Transform ts = ora::Transform::from_row(ts6[0], ts6[1], ts6[2], ts6[3], ts6[4], ts6[5]);
    ora::render_tree(*tree, ts, pm);
    std::memcpy(pixmap, pm.data.data(), (size_t)w * h * 4);
    return 0;
}

}

#include <thread>
extern "C" {
// Renders with `threads` host threads, each drawing a horizontal strip of the
// canvas through a translated transform (resvg renders one tree per thread;
// this is the all-core CPU timing of the same workload).
int oracle_render_parallel(const rgpu_tree_view *tree, const float ts6[6], uint32_t w, uint32_t h, uint8_t *pixmap,
                           uint32_t threads) {
    if (!tree || !pixmap || w == 0 || h == 0) return -1;
    if (threads == 0) threads = 1;
    threads = std::min(threads, h);
    std::vector<std::thread> pool;
    uint32_t rows = (h + threads - 1) / threads;
    for (uint32_t k = 0; k < threads; k++) {
        uint32_t y0 = k * rows;
        if (y0 >= h) break;
        uint32_t hh = std::min(rows, h - y0);
        pool.emplace_back([=]() {
            ora::Pixmap pm(w, hh);
            std::memcpy(pm.data.data(), pixmap + (size_t)y0 * w * 4, (size_t)w * hh * 4);
            ora::Transform ts = ora::Transform::from_row(ts6[0], ts6[1], ts6[2], ts6[3], ts6[4], ts6[5]);
            ts = ora::Transform::translate(0.0f, -(float)y0).pre_concat(ts);
            ora::render_tree(*tree, ts, pm);
            std::memcpy(pixmap + (size_t)y0 * w * 4, pm.data.data(), (size_t)w * hh * 4);
        });
    }
    for (auto &t : pool) t.join();
    return 0;
}
}
