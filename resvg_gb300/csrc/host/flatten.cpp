// Host flattener (see flatten.h).
//
// Paint conversion follows resvg's path.rs:118-177 (stop colours with
// (stop_opacity * opacity).to_u8() alpha) and the tiny-skia shader/blitter
// set-up it calls (Gradient::new stop normalisation, points_to_unit transforms,
// RasterPipelineBlitter::new strength reduction of SourceOver to Source for
// opaque paints and the memset fast path).
#include "flatten.h"
#include "hairline.h"
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

namespace rgpu {

static std::atomic<bool> g_device_stroke{true};
void set_device_stroke(bool on) { g_device_stroke.store(on); }
bool device_stroke_enabled() { return g_device_stroke.load(); }

namespace {

struct ColorF { float r, g, b, a; };

inline uint8_t sat_u8(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}
inline uint16_t sat_u16(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 65535.0f) return 65535;
    return (uint16_t)v;
}
inline uint8_t to_u8_norm(float v) { return sat_u8(v * 255.0f + 0.5f); }
inline ColorF rgba8(uint8_t r, uint8_t g, uint8_t b, uint8_t a) { return ColorF{r / 255.0f, g / 255.0f, b / 255.0f, a / 255.0f}; }
inline int32_t sat_i32(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
inline ColorF premul(ColorF c) {
    if (c.a == 1.0f) return c;
    auto cl = [](float v) { return std::min(std::max(v, 0.0f), 1.0f); };
    return ColorF{cl(c.r * c.a), cl(c.g * c.a), cl(c.b * c.a), c.a};
}

struct Stop { float pos; ColorF c; };

enum ShKind { SH_NONE, SH_SOLID, SH_LINEAR, SH_RADIAL };
struct Shader {
    ShKind kind = SH_NONE;
    ColorF color{0, 0, 0, 1};
    std::vector<Stop> stops;
    uint32_t spread = 0;
    Xf ts;
    float x0 = 0, y0 = 0, x1 = 0, y1 = 0, r0 = 0, r1 = 0;
    bool opaque() const {
        if (kind == SH_SOLID) return color.a == 1.0f;
        for (auto &s : stops) if (s.c.a != 1.0f) return false;
        return true;
    }
};

// path.rs:118-177 + LinearGradient::new / RadialGradient::new
bool make_shader(const rgpu_tree_view &t, int32_t pi, float opacity, Shader &sh) {
    const rgpu_paint &pp = t.paints[pi];
    uint8_t a8 = to_u8_norm(opacity);
    if (pp.kind == RGPU_PAINT_SOLID) { sh.kind = SH_SOLID; sh.color = rgba8(pp.r, pp.g, pp.b, a8); return true; }
    for (uint32_t i = 0; i < pp.stop_count; i++) {
        const rgpu_stop &s = t.stops[pp.stop_offset + i];
        sh.stops.push_back(Stop{s.offset, rgba8(s.r, s.g, s.b, to_u8_norm(s.opacity * opacity))});
    }
    if (sh.stops.empty()) return false;
    if (sh.stops.size() == 1) { sh.kind = SH_SOLID; sh.color = sh.stops[0].c; return true; }
    Xf gts = Xf::of(pp.transform), inv;
    if (pp.kind == RGPU_PAINT_LINEAR) {
        float dx = pp.x2 - pp.x1, dy = pp.y2 - pp.y1;
        float len = std::sqrt(dx * dx + dy * dy);
        if (!std::isfinite(len)) return false;
        if (len <= 1.0f / (1 << 15)) { sh.kind = SH_SOLID; sh.color = sh.stops.back().c; return true; }
        if (!invert(gts, &inv)) return false;
        sh.kind = SH_LINEAR;
        sh.x0 = pp.x1; sh.y0 = pp.y1; sh.x1 = pp.x2; sh.y1 = pp.y2;
    } else {
        if (!(pp.r_ > 0)) return false;
        if (!invert(gts, &inv)) return false;
        sh.kind = SH_RADIAL;
        sh.x0 = pp.fx; sh.y0 = pp.fy; sh.r0 = pp.fr;
        sh.x1 = pp.cx; sh.y1 = pp.cy; sh.r1 = pp.r_;
    }
    sh.spread = pp.spread;
    sh.ts = gts;
    return true;
}

// Gradient::new + push_stages, producing the device GradRec.
bool make_grad(const Shader &sh, GradRec &g) {
    std::memset(&g, 0, sizeof(g));
    std::vector<Stop> st = sh.stops;
    bool dummy_first = st[0].pos != 0.0f, dummy_last = st.back().pos != 1.0f;
    if (dummy_first) st.insert(st.begin(), Stop{0.0f, st[0].c});
    if (dummy_last) st.push_back(Stop{1.0f, st.back().c});
    bool opaque = true;
    for (auto &s : st) if (s.c.a != 1.0f) opaque = false;
    size_t start = dummy_first ? 0 : 1;
    float prev = 0.0f;
    bool uniform = true;
    float step = st[start].pos - prev;
    for (size_t i = start; i < st.size(); i++) {
        float curr;
        if (i + 1 == st.size()) curr = 1.0f;
        else { float v = st[i].pos; curr = v > 1.0f ? 1.0f : (v >= prev ? v : prev); }
        uniform = uniform && std::fabs(step - (curr - prev)) <= 1.0f / 4096.0f;
        st[i].pos = std::min(std::max(curr, 0.0f), 1.0f);
        prev = curr;
    }
    g.flags = 0;
    if (!opaque) g.flags |= GRAD_PREMUL;
    if (sh.spread == RGPU_SPREAD_PAD && uniform) g.flags |= GRAD_PAD_CLAMP;
    g.spread = sh.spread;
    if (st.size() == 2) {
        g.flags |= GRAD_TWO_STOP;
        ColorF c0 = st[0].c, c1 = st[1].c;
        g.n = 1;
        g.t[0] = 0;
        g.iv[0].f[0] = c1.r - c0.r; g.iv[0].f[1] = c1.g - c0.g; g.iv[0].f[2] = c1.b - c0.b; g.iv[0].f[3] = c1.a - c0.a;
        g.iv[0].b[0] = c0.r; g.iv[0].b[1] = c0.g; g.iv[0].b[2] = c0.b; g.iv[0].b[3] = c0.a;
    } else {
        auto eq = [](ColorF a, ColorF b) { return a.r == b.r && a.g == b.g && a.b == b.b && a.a == b.a; };
        size_t first = eq(st[0].c, st[1].c) ? 1 : 0;
        size_t last = eq(st.back().c, st[st.size() - 2].c) ? st.size() - 2 : st.size() - 1;
        uint32_t n = 0;
        auto push = [&](const float f[4], const float b[4], float t) {
            if (n >= (uint32_t)kMaxGradStops) { n = kMaxGradStops + 1; return; }
            for (int k = 0; k < 4; k++) { g.iv[n].f[k] = f[k]; g.iv[n].b[k] = b[k]; }
            g.t[n] = t;
            n++;
        };
        float tl = st[first].pos;
        ColorF cl = st[first].c;
        float zero[4] = {0, 0, 0, 0};
        { float b[4] = {cl.r, cl.g, cl.b, cl.a}; push(zero, b, 0.0f); }
        for (size_t i = first; i < last; i++) {
            float tr = st[i + 1].pos;
            ColorF cr = st[i + 1].c;
            if (tl < tr) {
                float d = tr - tl;
                float f[4] = {(cr.r - cl.r) / d, (cr.g - cl.g) / d, (cr.b - cl.b) / d, (cr.a - cl.a) / d};
                float b[4] = {cl.r - f[0] * tl, cl.g - f[1] * tl, cl.b - f[2] * tl, cl.a - f[3] * tl};
                push(f, b, std::min(std::max(tl, 0.0f), 1.0f));
            }
            tl = tr;
            cl = cr;
        }
        { float b[4] = {cl.r, cl.g, cl.b, cl.a}; push(zero, b, std::min(std::max(tl, 0.0f), 1.0f)); }
        if (n > (uint32_t)kMaxGradStops) return false;  // more stops than the device record holds
        g.n = n;
    }
    // device pixel -> unit space
    Xf inv;
    if (!invert(sh.ts, &inv)) return false;
    Xf unit;
    if (sh.kind == SH_LINEAR) {
        float vx = sh.x1 - sh.x0, vy = sh.y1 - sh.y0;
        float mag = std::sqrt(vx * vx + vy * vy);
        float invm = mag != 0.0f ? 1.0f / mag : 0.0f;
        vx *= invm; vy *= invm;
        float sn = -vy, cs = vx, ci = 1.0f - cs;
        unit = Xf::row(cs, sn, -sn, cs, sn * sh.y0 + ci * sh.x0, -sn * sh.x0 + ci * sh.y0);
        unit = post_concat(unit, Xf::translate(-sh.x0, -sh.y0));
        unit = post_concat(unit, Xf::scale(invm, invm));
    } else {
        float ir = 1.0f / sh.r1;
        unit = post_concat(Xf::translate(-sh.x0, -sh.y0), Xf::scale(ir, ir));
        if (sh.x0 == sh.x1 && sh.y0 == sh.y1 && sh.r0 == 0.0f) {
            g.flags |= GRAD_RADIAL_SIMPLE;
        } else {
            g.flags |= GRAD_RADIAL_CONICAL;
            g.fr0 = sh.r0 * ir;
            g.fr1 = 1.0f;
            g.cdx = (sh.x1 - sh.x0) * ir;
            g.cdy = (sh.y1 - sh.y0) * ir;
        }
    }
    Xf full = post_concat(inv, unit);
    g.ts[0] = full.sx; g.ts[1] = full.ky; g.ts[2] = full.kx; g.ts[3] = full.sy; g.ts[4] = full.tx; g.ts[5] = full.ty;
    return true;
}

struct Target {
    int32_t w, h;    // pixmap size
    int32_t ox, oy;  // origin in the stream's output space
};

struct Flattener {
    SceneBuild &sb;
    Tree &tree;
    const rgpu_tree_view &t;
    uint32_t tree_verb_base, tree_pt_base;
    int32_t max_x, max_y, max_w, max_h;  // max_filter_bbox
    StreamBuild *cur = nullptr;          // stream being emitted
    uint32_t depth = 0;
    uint32_t child_level = 0;            // max level of content streams referenced by `cur` (+1)
    bool unsupported = false;

    uint32_t add_paint(const PaintRec &p) { sb.paints.push_back(p); return (uint32_t)sb.paints.size() - 1; }

    // RasterPipelineBlitter::new for the paint; false when nothing is drawn.
    bool paint_rec(const Shader &sh0, uint32_t blend, bool aa, const Xf &ts, PaintRec &pr) {
        std::memset(&pr, 0, sizeof(pr));
        Shader sh = sh0;
        if (sh.kind == SH_LINEAR || sh.kind == SH_RADIAL) sh.ts = post_concat(sh.ts, ts);
        bool opaque = sh.opaque();
        if (blend == RGPU_BLEND_DESTINATION) return false;
        if (blend == RGPU_BLEND_DESTINATION_IN && opaque && sh.kind == SH_SOLID) return false;
        if (opaque && blend == RGPU_BLEND_SOURCE_OVER) blend = RGPU_BLEND_SOURCE;
        bool memset_ok = false;
        if (sh.kind == SH_SOLID) {
            pr.kind = 0;
            ColorF c = premul(sh.color);
            float cf[4] = {c.r, c.g, c.b, c.a};
            for (int i = 0; i < 4; i++) {
                pr.colorf[i] = cf[i];
                pr.rgba16[i] = sat_u16(cf[i] * 255.0f + 0.5f);
                pr.memset_rgba[i] = sat_u8(cf[i] * 255.0f + 0.5f);
            }
            if (blend == RGPU_BLEND_SOURCE) memset_ok = true;
        } else {
            GradRec g;
            if (!make_grad(sh, g)) return false;
            sb.grads.push_back(g);
            pr.kind = 1;
            pr.grad = (uint32_t)sb.grads.size() - 1;
            for (int i = 0; i < 6; i++) pr.gts[i] = g.ts[i];
            pr.gmeta = g.flags | g.spread << 8 | g.n << 16;
        }
        if (blend == RGPU_BLEND_CLEAR && !aa) {
            blend = RGPU_BLEND_SOURCE;
            memset_ok = true;
            std::memset(pr.memset_rgba, 0, 4);
        }
        // tiny-skia runs a solid colour, a linear or a simple radial gradient
        // in the lowp pipeline (two-point conical stages are highp only).
        bool lowp_shader = sh.kind == SH_SOLID || sh.kind == SH_LINEAR ||
                           (sh.kind == SH_RADIAL && (sb.grads.back().flags & GRAD_RADIAL_SIMPLE));
        bool lowp = lowp_shader &&
                    (blend == RGPU_BLEND_SOURCE || blend == RGPU_BLEND_SOURCE_OVER || blend == RGPU_BLEND_CLEAR ||
                     blend == RGPU_BLEND_DESTINATION_OUT || blend == RGPU_BLEND_XOR || blend == RGPU_BLEND_SOURCE_ATOP ||
                     blend == RGPU_BLEND_PLUS || blend == RGPU_BLEND_MODULATE || blend == RGPU_BLEND_SCREEN);
        pr.blend = blend;
        pr.flags = (lowp ? PAINT_LOWP : 0) | (memset_ok ? PAINT_MEMSET : 0);
        return true;
    }

    void emit_draw(uint32_t op, uint32_t verb_off, uint32_t verb_cnt, uint32_t pt_off, uint32_t pt_cnt, const Xf &ts,
                   const Target &tg, uint32_t rule, bool aa, uint32_t paint) {
        DrawRec d;
        std::memset(&d, 0, sizeof(d));
        d.verb_off = verb_off; d.verb_cnt = verb_cnt; d.pt_off = pt_off; d.pt_cnt = pt_cnt;
        d.ts[0] = ts.sx; d.ts[1] = ts.ky; d.ts[2] = ts.kx; d.ts[3] = ts.sy; d.ts[4] = ts.tx; d.ts[5] = ts.ty;
        d.clip_w = tg.w; d.clip_h = tg.h;
        d.ox = tg.ox; d.oy = tg.oy;
        d.flags = (rule == RGPU_EVENODD ? DRAW_EVENODD : 0) | (aa ? DRAW_AA : 0);
        d.paint = paint;
        cur->draws.push_back(d);
        cur->cmds.push_back(Cmd{op, (uint32_t)cur->draws.size() - 1, 0, 0.0f});
    }

    bool path_bounds_empty(const rgpu_path &p) {
        if (p.point_count == 0) return true;
        const float *pts = t.points + 2 * (size_t)p.point_offset;
        float l = pts[0], r = pts[0], tp = pts[1], b = pts[1];
        for (uint32_t i = 1; i < p.point_count; i++) {
            l = std::min(l, pts[2 * i]); r = std::max(r, pts[2 * i]);
            tp = std::min(tp, pts[2 * i + 1]); b = std::max(b, pts[2 * i + 1]);
        }
        return r - l == 0.0f || b - tp == 0.0f;
    }

    // path.rs:179-205 render_pattern_pixmap and the Pattern shader: the tile is
    // the pattern content at the fill's device scale, rendered by its own
    // stream; its shader (patternTransform * translate(rect) * scale(1 / s),
    // then the fill transform) is evaluated per layer pixel by a job after
    // that stream's pass, and the fill reads the result as an image paint.
    bool pattern_paint(const rgpu_paint &pp, float opacity, uint32_t blend, const Xf &ts, const Target &tg,
                       PaintRec &pr) {
        const Xf pts = Xf::of(pp.transform);
        const Xf t2 = pre_concat(ts, pts);
        const float sx = std::sqrt(t2.sx * t2.sx + t2.kx * t2.kx), sy = std::sqrt(t2.ky * t2.ky + t2.sy * t2.sy);
        auto to_u32 = [](float v) -> uint32_t {  // (v).round() as u32
            v = std::round(v);
            if (!(v > 0.0f)) return 0;
            if (v >= 4294967296.0f) return 0xFFFFFFFFu;
            return (uint32_t)v;
        };
        const uint32_t iw = to_u32(pp.x2 * sx), ih = to_u32(pp.y2 * sy);
        if (!iw || !ih || (uint64_t)iw * ih > ((uint64_t)1 << 26) || pp.stop_offset >= t.group_count) return false;
        if ((uint64_t)tg.w * tg.h > ((uint64_t)1 << 26)) { unsupported = true; return false; }
        const Xf st = pre_concat(pre_concat(pts, Xf::translate(pp.x1, pp.y1)), Xf::row(1.0f / sx, 0, 0, 1.0f / sy, 0, 0));
        Xf inv;
        if (!invert(pre_concat(ts, st), &inv)) return false;
        const uint32_t tile = (uint32_t)sb.surfaces.size();
        sb.surfaces.push_back(SurfaceReq{(int32_t)iw, (int32_t)ih});
        StreamBuild ps;
        ps.out_w = (int32_t)iw; ps.out_h = (int32_t)ih;
        ps.stride = iw * 4;
        ps.surface = (int32_t)tile;
        StreamBuild *sv = cur;
        uint32_t sd = depth, sc = child_level;
        cur = &ps;
        depth = 0;
        child_level = 0;
        render_nodes(pp.stop_offset, Xf::row(sx, 0, 0, sy, 0, 0), Target{(int32_t)iw, (int32_t)ih, 0, 0});
        ps.level = child_level;
        cur = sv;
        depth = sd;
        child_level = std::max(sc, ps.level + 1);
        sb.append_stream(ps);
        const uint32_t shade = (uint32_t)sb.surfaces.size();
        sb.surfaces.push_back(SurfaceReq{tg.w * 4, tg.h});
        GradRec g;
        std::memset(&g, 0, sizeof(g));
        const uint32_t gi = (uint32_t)sb.grads.size();
        sb.grads.push_back(g);
        const bool nearest = inv.sx == 1.0f && inv.sy == 1.0f && inv.kx == 0.0f && inv.ky == 0.0f;
        sb.patterns.push_back(PatternReq{gi, tile, (int32_t)iw, (int32_t)ih, shade, 0, 0, tg.w, tg.h, inv,
                                         nearest ? 0 : 2, 1, opacity, ps.level});
        std::memset(&pr, 0, sizeof(pr));
        pr.kind = 2;
        pr.blend = blend;
        pr.grad = gi;
        if (blend == RGPU_BLEND_DESTINATION) pr.flags = PAINT_SKIP;
        return true;
    }

    // image.rs:167-201 render_raster: the decoded image as a padded pattern in
    // the path's user space, evaluated per layer pixel before the first raster
    // pass (the stream drawing it is pushed to level 1 or later).
    bool image_paint(const rgpu_paint &pp, uint32_t blend, const Xf &ts, const Target &tg, PaintRec &pr) {
        if (pp.stop_offset >= t.image_count) return false;
        if ((uint64_t)tg.w * tg.h > ((uint64_t)1 << 26)) { unsupported = true; return false; }
        const rgpu_image &im = t.images[pp.stop_offset];
        Xf inv;
        if (!invert(ts, &inv)) return false;
        const uint32_t tile = (uint32_t)sb.surfaces.size();
        sb.surfaces.push_back(SurfaceReq{(int32_t)im.width, (int32_t)im.height, t.image_pixels + im.pixel_offset});
        const uint32_t shade = (uint32_t)sb.surfaces.size();
        sb.surfaces.push_back(SurfaceReq{tg.w * 4, tg.h});
        GradRec g;
        std::memset(&g, 0, sizeof(g));
        const uint32_t gi = (uint32_t)sb.grads.size();
        sb.grads.push_back(g);
        const bool translate = inv.sx == 1.0f && inv.sy == 1.0f && inv.kx == 0.0f && inv.ky == 0.0f;
        sb.patterns.push_back(PatternReq{gi, tile, (int32_t)im.width, (int32_t)im.height, shade, 0, 0, tg.w, tg.h,
                                         inv, translate ? 0 : (int32_t)std::min<uint32_t>(pp.spread, 2u), 0, 1.0f,
                                         0});
        child_level = std::max<uint32_t>(child_level, 1);
        std::memset(&pr, 0, sizeof(pr));
        pr.kind = 2;
        pr.blend = blend;
        pr.grad = gi;
        if (blend == RGPU_BLEND_DESTINATION) pr.flags = PAINT_SKIP;
        return true;
    }

    // path.rs:26-75
    void fill_path(const rgpu_path &p, uint32_t blend, const Xf &ts, const Target &tg) {
        if (p.fill_paint < 0) return;
        if (path_bounds_empty(p)) return;
        Shader sh;
        PaintRec pr;
        if (t.paints[p.fill_paint].kind == RGPU_PAINT_PATTERN) {
            if (!pattern_paint(t.paints[p.fill_paint], p.fill_opacity, blend, ts, tg, pr)) return;
        } else if (t.paints[p.fill_paint].kind == RGPU_PAINT_IMAGE) {
            if (!image_paint(t.paints[p.fill_paint], blend, ts, tg, pr)) return;
        } else {
            if (!make_shader(t, p.fill_paint, p.fill_opacity, sh)) return;
            if (!paint_rec(sh, blend, p.anti_alias != 0, ts, pr)) return;
        }
        emit_draw(CMD_FILL, tree_verb_base + p.verb_offset, p.verb_count, tree_pt_base + p.point_offset, p.point_count,
                  ts, tg, p.fill_rule, p.anti_alias != 0, add_paint(pr));
    }
    // path.rs:77-116 (outline from the host stroker, filled non-zero)
    // tiny-skia stroke_path: a stroke at most one device pixel wide is drawn as
    // an anti-aliased hairline of the (dashed) path; for blend modes that
    // pre-scale coverage its paint is scaled by the stroke's coverage.
    static bool pre_scale_blend(uint32_t blend) {
        return blend == RGPU_BLEND_DESTINATION || blend == RGPU_BLEND_DESTINATION_OVER || blend == RGPU_BLEND_PLUS ||
               blend == RGPU_BLEND_DESTINATION_OUT || blend == RGPU_BLEND_SOURCE_ATOP ||
               blend == RGPU_BLEND_SOURCE_OVER || blend == RGPU_BLEND_XOR;
    }
    bool hairline(uint32_t pi, Shader sh, uint32_t blend, const Xf &ts, const Target &tg, float rs) {
        const rgpu_path &p = t.paths[pi];
        float coverage = 1.0f;
        if (!treat_as_hairline(p.anti_alias != 0, p.stroke_width, ts, &coverage)) return false;
        PathData src;
        if (!hairline_source_view(t, pi, rs, src)) return true;
        const bool pre_scale = blend == RGPU_BLEND_DESTINATION || blend == RGPU_BLEND_DESTINATION_OVER ||
                               blend == RGPU_BLEND_PLUS || blend == RGPU_BLEND_DESTINATION_OUT ||
                               blend == RGPU_BLEND_SOURCE_ATOP || blend == RGPU_BLEND_SOURCE_OVER ||
                               blend == RGPU_BLEND_XOR;
        if (coverage != 1.0f && pre_scale) {
            const float op = std::min(std::max(hairline_opacity(coverage), 0.0f), 1.0f);
            auto scale = [op](ColorF &c) { c.a = std::min(std::max(c.a * op, 0.0f), 1.0f); };
            if (sh.kind == SH_SOLID) scale(sh.color);
            for (auto &st : sh.stops) scale(st.c);
        }
        PaintRec pr;
        if (!paint_rec(sh, blend, true, ts, pr)) return true;
        emit_hairline(pi, pr, src, ts, tg);
        return true;
    }
    void emit_hairline(uint32_t pi, PaintRec &pr, const PathData &src, const Xf &ts, const Target &tg) {
        const rgpu_path &p = t.paths[pi];
        std::vector<HairCall> calls;
        hairline_calls(src, ts, p.line_cap, tg.w, tg.h, calls);
        HairRec hr;
        std::memset(&hr, 0, sizeof(hr));
        hr.span_off = (uint32_t)sb.hair_spans.size();
        for (const HairCall &c : calls) hairline_spans(c, sb.hair_spans);
        // the blitters never write outside the layer: fold it into each span's rect
        size_t keep = hr.span_off;
        hr.x0 = hr.y0 = INT32_MAX;
        hr.x1 = hr.y1 = INT32_MIN;
        for (size_t k = hr.span_off; k < sb.hair_spans.size(); k++) {
            HairSpan s = sb.hair_spans[k];
            s.x0 = std::max(s.x0, 0); s.y0 = std::max(s.y0, 0);
            s.x1 = std::min(s.x1, tg.w); s.y1 = std::min(s.y1, tg.h);
            if (s.x0 >= s.x1 || s.y0 >= s.y1) continue;
            hr.x0 = std::min(hr.x0, s.x0); hr.y0 = std::min(hr.y0, s.y0);
            hr.x1 = std::max(hr.x1, s.x1); hr.y1 = std::max(hr.y1, s.y1);
            sb.hair_spans[keep++] = s;
        }
        sb.hair_spans.resize(keep);
        hr.span_cnt = (uint32_t)sb.hair_spans.size() - hr.span_off;
        if (!hr.span_cnt) return;
        hr.paint = add_paint(pr);
        hr.ox = tg.ox; hr.oy = tg.oy;
        sb.hairs.push_back(hr);
        cur->cmds.push_back(Cmd{CMD_HAIR, (uint32_t)sb.hairs.size() - 1, 0, 0.0f});
    }
    void stroke_path(uint32_t pi, uint32_t blend, const Xf &ts, const Target &tg) {
        const rgpu_path &p = t.paths[pi];
        if (p.stroke_paint < 0) return;
        Shader sh;
        float rs = resolution_scale(ts.sx, ts.ky, ts.kx, ts.sy);
        PaintRec pr;
        if (t.paints[p.stroke_paint].kind == RGPU_PAINT_IMAGE) return;  // images are fills only
        if (t.paints[p.stroke_paint].kind == RGPU_PAINT_PATTERN) {
            float coverage = 1.0f;
            if (treat_as_hairline(p.anti_alias != 0, p.stroke_width, ts, &coverage)) {
                PathData src;
                if (!hairline_source_view(t, pi, rs, src)) return;
                float op = p.stroke_opacity;
                if (coverage != 1.0f && pre_scale_blend(blend))
                    op = std::min(std::max(op * std::min(std::max(hairline_opacity(coverage), 0.0f), 1.0f), 0.0f), 1.0f);
                if (!pattern_paint(t.paints[p.stroke_paint], op, blend, ts, tg, pr)) return;
                emit_hairline(pi, pr, src, ts, tg);
                return;
            }
            if (!pattern_paint(t.paints[p.stroke_paint], p.stroke_opacity, blend, ts, tg, pr)) return;
        } else {
            if (!make_shader(t, p.stroke_paint, p.stroke_opacity, sh)) return;
            if (hairline(pi, sh, blend, ts, tg, rs)) return;
            if (!paint_rec(sh, blend, p.anti_alias != 0, ts, pr)) return;
        }
        bool cached = false;
        std::shared_ptr<PathData> outline;
        if (device_stroke_enabled()) outline = tree.cached_stroke_outline(pi, rs, &cached);
        if (device_stroke_enabled() && !cached) {
            // stroked on the device (kernels/stroke.cu): a job over the source
            // path, whose outline the draw fills; the outline then goes to the
            // tree's cache for later flattens
            if (!(p.stroke_width > 0)) return;
            StrokeJob j;
            std::memset(&j, 0, sizeof(j));
            j.src_verb_off = tree_verb_base + p.verb_offset; j.src_verb_cnt = p.verb_count;
            j.src_pt_off = tree_pt_base + p.point_offset; j.src_pt_cnt = p.point_count;
            if (p.dash_count) {
                // dash.rs on the device too: the job dashes, then strokes the dashed path
                j.dash_off = (uint32_t)sb.dashes.size();
                j.dash_cnt = p.dash_count;
                j.dash_phase = p.dash_phase;
                sb.dashes.insert(sb.dashes.end(), t.dashes + p.dash_offset, t.dashes + p.dash_offset + p.dash_count);
            }
            j.width = p.stroke_width;
            j.miter_limit = p.miter_limit;
            j.res_scale = rs;
            j.cap_join = (p.line_cap & 0xFFu) | (p.line_join & 0xFFu) << 8;
            j.draw = (uint32_t)cur->draws.size();
            cur->strokes.push_back(j);
            cur->stroke_keys.push_back(StrokeKey{&tree, pi, rs});
            emit_draw(CMD_FILL, 0, 0, 0, 0, ts, tg, RGPU_NONZERO, p.anti_alias != 0, add_paint(pr));
            cur->draws.back().flags |= DRAW_STROKED;
            return;
        }
        if (!cached) outline = tree.stroke_outline(pi, rs);
        if (!outline || outline->verbs.empty()) return;
        uint32_t vo = (uint32_t)sb.verbs.size(), po = (uint32_t)(sb.pts.size() / 2);
        sb.verbs.insert(sb.verbs.end(), outline->verbs.begin(), outline->verbs.end());
        sb.pts.insert(sb.pts.end(), outline->pts.begin(), outline->pts.end());
        emit_draw(CMD_FILL, vo, (uint32_t)outline->verbs.size(), po, (uint32_t)(outline->pts.size() / 2), ts, tg,
                  RGPU_NONZERO, p.anti_alias != 0, add_paint(pr));
    }
    void render_path(uint32_t pi, const Xf &ts, const Target &tg) {
        const rgpu_path &p = t.paths[pi];
        if (!p.visible) return;
        if (!p.stroke_first) {
            fill_path(p, RGPU_BLEND_SOURCE_OVER, ts, tg);
            stroke_path(pi, RGPU_BLEND_SOURCE_OVER, ts, tg);
        } else {
            stroke_path(pi, RGPU_BLEND_SOURCE_OVER, ts, tg);
            fill_path(p, RGPU_BLEND_SOURCE_OVER, ts, tg);
        }
    }
    uint32_t push_layer(const Target &tg, uint32_t init, int32_t surf = -1) {
        LayerRec L;
        std::memset(&L, 0, sizeof(L));
        L.x = tg.ox; L.y = tg.oy; L.w = tg.w; L.h = tg.h;
        L.surf = surf;
        cur->layers.push_back(L);
        uint32_t li = (uint32_t)cur->layers.size() - 1;
        cur->cmds.push_back(Cmd{CMD_PUSH, li, init, 0.0f});
        depth++;
        cur->max_depth = std::max(cur->max_depth, depth);
        return li;
    }
    void pop(uint32_t op, uint32_t li, uint32_t b, float f) {
        cur->cmds.push_back(Cmd{op, li, b, f});
        depth--;
    }
    // clip.rs:30-68
    void draw_children(uint32_t gi, uint32_t mode, const Xf &ts, const Target &tg) {
        const rgpu_group &g = t.groups[gi];
        for (uint32_t k = 0; k < g.child_count; k++) {
            const rgpu_node &n = t.children[g.child_offset + k];
            if (n.kind == RGPU_NODE_PATH) {
                const rgpu_path &p = t.paths[n.index];
                if (!p.visible) continue;
                fill_path(p, mode, ts, tg);
            } else {
                const rgpu_group &cg = t.groups[n.index];
                Xf t2 = pre_concat(ts, Xf::of(cg.transform));
                if (cg.clip_path >= 0) {
                    // clip_group (clip.rs:70-98)
                    uint32_t li = push_layer(tg, 0);
                    draw_children(n.index, RGPU_BLEND_SOURCE_OVER, t2, tg);
                    clip_apply(t.clips[cg.clip_path], t2, tg);
                    pop(CMD_POP_COMPOSITE, li, RGPU_BLEND_XOR, 1.0f);
                } else {
                    draw_children(n.index, mode, t2, tg);
                }
            }
        }
    }
    // clip.rs:6-28; the nested clip is applied to the layer first, then this
    // clip's own mask (the same order resvg applies them in).
    void clip_apply(const rgpu_clip &clip, const Xf &ts, const Target &tg) {
        if (clip.clip_path >= 0) clip_apply(t.clips[clip.clip_path], ts, tg);
        uint32_t li = push_layer(tg, 1);
        draw_children(clip.root, RGPU_BLEND_CLEAR, pre_concat(ts, Xf::of(clip.transform)), tg);
        pop(CMD_POP_CLIP, li, 0, 0.0f);
    }
    // mask.rs:6-46
    void mask_apply(const rgpu_mask &mask, const Xf &ts, const Target &tg) {
        if (t.groups[mask.root].child_count == 0) {
            cur->cmds.push_back(Cmd{CMD_CLEAR, 0, 0, 0.0f});
            return;
        }
        if (mask.mask >= 0) mask_apply(t.masks[mask.mask], ts, tg);
        uint32_t li = push_layer(tg, 0);
        render_nodes(mask.root, ts, tg);
        // region: Mask::fill_path(rect, winding, aa, ts), then apply_mask
        uint32_t vo = (uint32_t)sb.verbs.size(), po = (uint32_t)(sb.pts.size() / 2);
        uint8_t v[5] = {RGPU_MOVE, RGPU_LINE, RGPU_LINE, RGPU_LINE, RGPU_CLOSE};
        sb.verbs.insert(sb.verbs.end(), v, v + 5);
        float r[8] = {mask.x, mask.y, mask.x + mask.w, mask.y, mask.x + mask.w, mask.y + mask.h, mask.x, mask.y + mask.h};
        sb.pts.insert(sb.pts.end(), r, r + 8);
        PaintRec pr;
        std::memset(&pr, 0, sizeof(pr));
        pr.flags = PAINT_SKIP;
        emit_draw(CMD_APPLY_REGION, vo, 5, po, 4, ts, tg, RGPU_NONZERO, true, add_paint(pr));
        pop(CMD_POP_MASK, li, mask.kind == RGPU_MASK_LUMINANCE ? 0 : 1, 0.0f);
    }
    static bool fit(int64_t x, int64_t y, int64_t w, int64_t h, int32_t bx, int32_t by, int32_t bw, int32_t bh,
                    int32_t out[4]) {
        int64_t l = std::max<int64_t>(x, bx), tp = std::max<int64_t>(y, by);
        int64_t r = std::min<int64_t>(x + w, (int64_t)bx + bw), b = std::min<int64_t>(y + h, (int64_t)by + bh);
        if (r <= l || b <= tp) return false;
        out[0] = (int32_t)l; out[1] = (int32_t)tp; out[2] = (int32_t)(r - l); out[3] = (int32_t)(b - tp);
        return true;
    }
    // Flattens a filtered group's content into its own stream and records the
    // filter job; returns the surface holding the filtered result.
    int32_t filtered_content(uint32_t gi, const Xf &lts, int32_t w, int32_t h) {
        const rgpu_group &g = t.groups[gi];
        uint32_t content = (uint32_t)sb.surfaces.size();
        sb.surfaces.push_back(SurfaceReq{w, h});
        uint32_t result = (uint32_t)sb.surfaces.size();
        sb.surfaces.push_back(SurfaceReq{w, h});
        StreamBuild sub;
        sub.out_w = w; sub.out_h = h;
        sub.stride = (uint32_t)w * 4;
        sub.surface = (int32_t)content;
        StreamBuild *saved = cur;
        uint32_t saved_depth = depth, saved_child = child_level;
        cur = &sub;
        depth = 0;
        child_level = 0;
        render_nodes(gi, lts, Target{w, h, 0, 0});
        sub.level = child_level;
        cur = saved;
        depth = saved_depth;
        child_level = std::max(saved_child, sub.level + 1);
        sb.append_stream(sub);
        // feImage of an element (filter/mod.rs:861-889): the element's group,
        // scaled by the layer's scale and moved to the primitive subregion,
        // rendered into a layer-sized surface of its own
        uint32_t image_first = (uint32_t)sb.fe_images.size(), level = sub.level;
        for (uint32_t fi = 0; fi < g.filter_count; fi++) {
            const rgpu_filter &f = t.filters[t.filter_refs[g.filter_offset + fi]];
            for (uint32_t pi = 0; pi < f.prim_count; pi++) {
                const rgpu_primitive &p = t.prims[f.prim_offset + pi];
                if (p.kind != RGPU_FE_IMAGE) continue;
                uint32_t surf = (uint32_t)sb.surfaces.size();
                sb.surfaces.push_back(SurfaceReq{w, h});
                float b[4];
                float sx = std::sqrt(lts.sx * lts.sx + lts.kx * lts.kx), sy = std::sqrt(lts.ky * lts.ky + lts.sy * lts.sy);
                float ox = 0.0f, oy = 0.0f;
                if (map_rect(lts, p.x, p.y, p.x + p.w, p.y + p.h, b)) {
                    ox = (float)sat_i32(std::floor(b[0]));
                    oy = (float)sat_i32(std::floor(b[1]));
                }
                StreamBuild im;
                im.out_w = w; im.out_h = h;
                im.stride = (uint32_t)w * 4;
                im.surface = (int32_t)surf;
                StreamBuild *sv = cur;
                uint32_t sd = depth, sc = child_level;
                cur = &im;
                depth = 0;
                child_level = 0;
                if (p.i[0] >= 0 && (uint32_t)p.i[0] < t.group_count)
                    render_nodes((uint32_t)p.i[0], Xf::row(sx, 0, 0, sy, ox, oy), Target{w, h, 0, 0});
                im.level = child_level;
                cur = sv;
                depth = sd;
                child_level = std::max(sc, im.level + 1);
                sb.append_stream(im);
                level = std::max(level, im.level);
                sb.fe_images.push_back(FeImageReq{f.prim_offset + pi, surf});
            }
        }
        FilterJob job;
        job.image_first = image_first;
        job.image_count = (uint32_t)sb.fe_images.size() - image_first;
        job.content = content;
        job.result = result;
        job.w = w; job.h = h;
        job.ts = lts;
        job.tree = &t;
        job.filter_ref_offset = g.filter_offset;
        job.filter_count = g.filter_count;
        job.level = level;
        sb.jobs.push_back(job);
        return (int32_t)result;
    }
    // render.rs:49-142
    void render_group(uint32_t gi, const Xf &ts_in, const Target &tg) {
        const rgpu_group &g = t.groups[gi];
        Xf ts = pre_concat(ts_in, Xf::of(g.transform));
        bool isolate = g.isolate || g.opacity != 1.0f || g.clip_path >= 0 || g.mask >= 0 || g.filter_count > 0 ||
                       g.blend != RGPU_BLEND_SOURCE_OVER;
        if (!isolate) { render_nodes(gi, ts, tg); return; }
        if (!g.has_layer_bbox) return;
        float bb[4];
        if (!map_rect(ts, g.layer_x, g.layer_y, g.layer_x + g.layer_w, g.layer_y + g.layer_h, bb)) return;
        float bw = bb[2] - bb[0], bh = bb[3] - bb[1];
        int32_t ib[4];
        if (g.filter_count == 0) {
            int64_t x = (int64_t)sat_i32(std::floor(bb[0])) - 2, y = (int64_t)sat_i32(std::floor(bb[1])) - 2;
            int64_t w = (int64_t)(uint32_t)std::max(0.0f, std::ceil(bw)) + 4;
            int64_t h = (int64_t)(uint32_t)std::max(0.0f, std::ceil(bh)) + 4;
            if (x < INT32_MIN || y < INT32_MIN || x + w > INT32_MAX || y + h > INT32_MAX) return;
            if (!fit(x, y, w, h, max_x, max_y, max_w, max_h, ib)) return;
        } else {
            int64_t x = sat_i32(std::floor(bb[0])), y = sat_i32(std::floor(bb[1]));
            int64_t w = (int64_t)std::max(1.0f, std::ceil(bw)), h = (int64_t)std::max(1.0f, std::ceil(bh));
            if (x + w > INT32_MAX || y + h > INT32_MAX) return;
            if (!fit(x, y, w, h, max_x, max_y, max_w, max_h, ib)) return;
        }
        float dx = bb[0], dy = bb[1];
        dx -= bb[0] - (float)ib[0];
        dy -= bb[1] - (float)ib[1];
        Xf lts = pre_concat(Xf::translate(-dx, -dy), ts);
        Target lt{ib[2], ib[3], tg.ox + ib[0], tg.oy + ib[1]};
        uint32_t li;
        if (g.filter_count) {
            if ((int64_t)ib[2] * ib[3] > (int64_t)1 << 28) { unsupported = true; return; }
            int32_t surf = filtered_content(gi, lts, ib[2], ib[3]);
            li = push_layer(lt, 2, surf);
        } else {
            li = push_layer(lt, 0);
            render_nodes(gi, lts, lt);
        }
        if (g.clip_path >= 0) clip_apply(t.clips[g.clip_path], lts, lt);
        if (g.mask >= 0) mask_apply(t.masks[g.mask], lts, lt);
        pop(CMD_POP_COMPOSITE, li, g.blend, g.opacity);
    }
    void render_nodes(uint32_t gi, const Xf &ts, const Target &tg) {
        const rgpu_group &g = t.groups[gi];
        for (uint32_t k = 0; k < g.child_count; k++) {
            const rgpu_node &n = t.children[g.child_offset + k];
            if (n.kind == RGPU_NODE_PATH) render_path(n.index, ts, tg);
            else render_group(n.index, ts, tg);
        }
    }
};

}  // namespace

uint32_t SceneBuild::append_stream(StreamBuild &b) {
    StreamRec st;
    std::memset(&st, 0, sizeof(st));
    uint32_t si = (uint32_t)streams.size();
    st.cmd_off = (uint32_t)cmds.size();
    st.cmd_cnt = (uint32_t)b.cmds.size();
    st.draw_off = (uint32_t)draws.size();
    st.draw_cnt = (uint32_t)b.draws.size();
    st.layer_off = (uint32_t)layers.size();
    st.out_w = b.out_w; st.out_h = b.out_h;
    st.out_stride = b.stride;
    st.out_ptr = b.out_ptr;
    st.max_depth = b.max_depth;
    st.surface = b.surface;
    st.level = b.level;
    max_level = std::max(max_level, b.level);
    for (auto &d : b.draws) {
        d.seg_base = (uint32_t)nsegs;
        d.tpt_base = (uint32_t)ntpts;
        d.stream = si;
        nsegs += d.verb_cnt + 1;
        ntpts += d.pt_cnt;
        draws.push_back(d);
    }
    for (auto j : b.strokes) {
        j.draw += st.draw_off;
        stroke_jobs.push_back(j);
    }
    stroke_keys.insert(stroke_keys.end(), b.stroke_keys.begin(), b.stroke_keys.end());
    for (auto c : b.cmds) {
        if (c.op == CMD_FILL || c.op == CMD_APPLY_REGION) c.a += st.draw_off;
        cmds.push_back(c);
    }
    layers.insert(layers.end(), b.layers.begin(), b.layers.end());
    streams.push_back(st);
    return si;
}

void SceneBuild::merge(std::vector<SceneBuild> &parts, unsigned threads) {
    // Every index a part's records hold into another array moves by where
    // that array's part starts; the result equals flattening the parts' trees
    // one after another into one build.  Arrays are sized first, then each part
    // is copied into its ranges with the index fix-ups, parts in parallel.
    struct Off {
        size_t verbs, pts, draws, paints, grads, layers, cmds, streams, surfaces, jobs, fe, patterns, hairs, hspans, strokes,
            dashes;
        uint64_t nsegs, ntpts;
    };
    const size_t n = parts.size();
    std::vector<Off> off(n + 1);
    Off cur{verbs.size(), pts.size(), draws.size(), paints.size(), grads.size(), layers.size(), cmds.size(),
            streams.size(), surfaces.size(), jobs.size(), fe_images.size(), patterns.size(), hairs.size(),
            hair_spans.size(), stroke_jobs.size(), dashes.size(), nsegs, ntpts};
    for (size_t k = 0; k < n; k++) {
        const SceneBuild &o = parts[k];
        off[k] = cur;
        cur.verbs += o.verbs.size(); cur.pts += o.pts.size(); cur.draws += o.draws.size();
        cur.paints += o.paints.size(); cur.grads += o.grads.size(); cur.layers += o.layers.size();
        cur.cmds += o.cmds.size(); cur.streams += o.streams.size(); cur.surfaces += o.surfaces.size();
        cur.jobs += o.jobs.size(); cur.fe += o.fe_images.size(); cur.patterns += o.patterns.size();
        cur.hairs += o.hairs.size(); cur.hspans += o.hair_spans.size(); cur.strokes += o.stroke_jobs.size();
        cur.dashes += o.dashes.size();
        cur.nsegs += o.nsegs; cur.ntpts += o.ntpts;
        max_level = std::max(max_level, o.max_level);
    }
    off[n] = cur;
    verbs.resize(cur.verbs); pts.resize(cur.pts); draws.resize(cur.draws); paints.resize(cur.paints);
    grads.resize(cur.grads); layers.resize(cur.layers); cmds.resize(cur.cmds); streams.resize(cur.streams);
    surfaces.resize(cur.surfaces); jobs.resize(cur.jobs); fe_images.resize(cur.fe); patterns.resize(cur.patterns);
    hairs.resize(cur.hairs); hair_spans.resize(cur.hspans); stroke_jobs.resize(cur.strokes);
    stroke_keys.resize(cur.strokes);
    dashes.resize(cur.dashes);
    nsegs = cur.nsegs;
    ntpts = cur.ntpts;
    auto copy_part = [&](size_t k) {
        const SceneBuild &o = parts[k];
        const Off &b = off[k];
        const uint32_t V = (uint32_t)b.verbs, P = (uint32_t)(b.pts / 2), D = (uint32_t)b.draws;
        const uint32_t PA = (uint32_t)b.paints, G = (uint32_t)b.grads, L = (uint32_t)b.layers, C = (uint32_t)b.cmds;
        const uint32_t S = (uint32_t)b.streams, SU = (uint32_t)b.surfaces, FE = (uint32_t)b.fe;
        const uint32_t H = (uint32_t)b.hairs, HS = (uint32_t)b.hspans;
        std::copy(o.verbs.begin(), o.verbs.end(), verbs.begin() + b.verbs);
        std::copy(o.pts.begin(), o.pts.end(), pts.begin() + b.pts);
        for (size_t i = 0; i < o.draws.size(); i++) {
            DrawRec d = o.draws[i];
            d.verb_off += V;
            d.pt_off += P;
            d.paint += PA;
            d.seg_base += (uint32_t)b.nsegs;
            d.tpt_base += (uint32_t)b.ntpts;
            d.stream += S;
            draws[b.draws + i] = d;
        }
        for (size_t i = 0; i < o.paints.size(); i++) {
            PaintRec q = o.paints[i];
            if (q.kind != 0) q.grad += G;
            paints[b.paints + i] = q;
        }
        std::copy(o.grads.begin(), o.grads.end(), grads.begin() + b.grads);
        for (size_t i = 0; i < o.stroke_jobs.size(); i++) {
            StrokeJob j = o.stroke_jobs[i];
            j.src_verb_off += V;
            j.src_pt_off += P;
            j.draw += D;
            if (j.dash_cnt) j.dash_off += (uint32_t)b.dashes;
            stroke_jobs[b.strokes + i] = j;
        }
        std::copy(o.dashes.begin(), o.dashes.end(), dashes.begin() + b.dashes);
        std::copy(o.stroke_keys.begin(), o.stroke_keys.end(), stroke_keys.begin() + b.strokes);
        for (size_t i = 0; i < o.layers.size(); i++) {
            LayerRec l = o.layers[i];
            if (l.surf >= 0) l.surf += (int32_t)SU;
            layers[b.layers + i] = l;
        }
        for (size_t i = 0; i < o.cmds.size(); i++) {
            Cmd c = o.cmds[i];
            if (c.op == CMD_FILL || c.op == CMD_APPLY_REGION) c.a += D;
            else if (c.op == CMD_HAIR) c.a += H;
            cmds[b.cmds + i] = c;
        }
        for (size_t i = 0; i < o.streams.size(); i++) {
            StreamRec st = o.streams[i];
            st.cmd_off += C;
            st.draw_off += D;
            st.layer_off += L;
            if (st.surface >= 0) st.surface += (int32_t)SU;
            streams[b.streams + i] = st;
        }
        std::copy(o.surfaces.begin(), o.surfaces.end(), surfaces.begin() + b.surfaces);
        for (size_t i = 0; i < o.jobs.size(); i++) {
            FilterJob j = o.jobs[i];
            j.content += SU;
            j.result += SU;
            j.image_first += FE;
            jobs[b.jobs + i] = j;
        }
        for (size_t i = 0; i < o.fe_images.size(); i++) {
            FeImageReq f = o.fe_images[i];
            f.surface += SU;
            fe_images[b.fe + i] = f;
        }
        for (size_t i = 0; i < o.patterns.size(); i++) {
            PatternReq q = o.patterns[i];
            q.grad += G;
            q.tile += SU;
            q.shade += SU;
            patterns[b.patterns + i] = q;
        }
        for (size_t i = 0; i < o.hairs.size(); i++) {
            HairRec h = o.hairs[i];
            h.span_off += HS;
            h.paint += PA;
            hairs[b.hairs + i] = h;
        }
        std::copy(o.hair_spans.begin(), o.hair_spans.end(), hair_spans.begin() + b.hspans);
    };
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= n) return;
            copy_part(k);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < std::max(1u, threads) && t < n; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
}

int SceneBuild::add_tree(Tree &tree, const Xf &ts, int32_t w, int32_t h, uint64_t out_ptr, uint32_t stride) {
    return add_node(tree, RGPU_NODE_GROUP, UINT32_MAX, ts, w, h, out_ptr, stride);
}

int SceneBuild::add_node(Tree &tree, uint32_t node_kind, uint32_t node_index, const Xf &ts, int32_t w, int32_t h,
                         uint64_t out_ptr, uint32_t stride) {
    const rgpu_tree_view &t = tree.finalized ? tree.view : *tree.get_view();
    Flattener f{*this, tree, t, (uint32_t)verbs.size(), (uint32_t)(pts.size() / 2)};
    verbs.insert(verbs.end(), t.verbs, t.verbs + t.verb_count);
    pts.insert(pts.end(), t.points, t.points + 2 * (size_t)t.point_count);
    int64_t mx = -2 * (int64_t)w, my = -2 * (int64_t)h, mw = 5 * (int64_t)w, mh = 5 * (int64_t)h;
    f.max_x = (int32_t)mx; f.max_y = (int32_t)my; f.max_w = (int32_t)mw; f.max_h = (int32_t)mh;
    StreamBuild root;
    root.out_w = w; root.out_h = h;
    root.stride = stride;
    root.out_ptr = out_ptr;
    f.cur = &root;
    if (node_index == UINT32_MAX) {
        if (t.group_count) f.render_nodes(0, ts, Target{w, h, 0, 0});  // resvg::render: the root's children
    } else if (node_kind == RGPU_NODE_GROUP && node_index < t.group_count) {
        f.render_group(node_index, ts, Target{w, h, 0, 0});
    } else if (node_kind == RGPU_NODE_PATH && node_index < t.path_count) {
        f.render_path(node_index, ts, Target{w, h, 0, 0});
    }
    if (f.unsupported) {
        error = "not supported on the device: a pattern paint, or a filter region of more than 2^28 pixels";
        return -1;
    }
    root.level = f.child_level;
    return (int)append_stream(root);
}

}  // namespace rgpu
