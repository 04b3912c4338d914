// Host driver of a filter job over device images (see filter_exec.h).
//
// Follows crates/resvg/src/filter/mod.rs: the filter region is the filter rect
// mapped by the layer transform (:362-373); each primitive takes its inputs
// (SourceGraphic, SourceAlpha or an earlier result, :523-564), converts them
// to the primitive's colour space (:286-308), runs, and is cropped to its
// subregion (:457-508); the last result goes back to sRGB and replaces the
// layer (:1100-1114).  On an invalid region the layer is cleared (:343-346).
#include "filter_exec.h"
#include <cmath>
#include <cstring>
#include <vector>
#include "../kernels/kernels.h"
#include "resvg_gpu.h"

namespace rgpu {
namespace {

inline int32_t sat_i32(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}

struct IRect { int32_t x, y, w, h; };

// rect.transform(ts).to_int_rect()
bool map_int_rect(const Xf &ts, float x, float y, float w, float h, IRect *out) {
    float b[4];
    if (!map_rect(ts, x, y, x + w, y + h, b)) return false;
    int64_t ix = sat_i32(std::floor(b[0])), iy = sat_i32(std::floor(b[1]));
    int64_t iw = std::max<int64_t>(1, (int64_t)std::ceil(b[2] - b[0]));
    int64_t ih = std::max<int64_t>(1, (int64_t)std::ceil(b[3] - b[1]));
    if (ix + iw > INT32_MAX || iy + ih > INT32_MAX) return false;
    *out = IRect{(int32_t)ix, (int32_t)iy, (int32_t)iw, (int32_t)ih};
    return true;
}

bool approx_zero_ulps(float v) {
    int32_t a;
    std::memcpy(&a, &v, 4);
    if (a < 0) return v == 0.0f;
    return a <= 4;
}

// resolve_std_dev (mod.rs:1119-1142): the sigmas scaled by the transform;
// false when both are zero; sigmas under 0.05 become 0; a box blur when either
// is at least 2, else IIR.
bool resolve_std_dev(const Xf &ts, float sdx, float sdy, float *ox, float *oy, bool *box) {
    const float sx = std::sqrt(ts.sx * ts.sx + ts.kx * ts.kx);
    const float sy = std::sqrt(ts.ky * ts.ky + ts.sy * ts.sy);
    float x = sdx * sx, y = sdy * sy;
    if (approx_zero_ulps(x) && approx_zero_ulps(y)) return false;
    if (x < 0.05f) x = 0.0f;
    if (y < 0.05f) y = 0.0f;
    *ox = x; *oy = y;
    *box = x >= 2.0f || y >= 2.0f;
    return true;
}

inline uint32_t sat_u8(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint32_t)v;
}

// One channel of feComponentTransfer (component_transfer.rs:41-78) at value c8;
// the same f32 operations in the same order, NaN saturating to 0.
uint32_t transfer_value(const rgpu_primitive &p, int ch, uint32_t c8) {
    const float *v = p.f + 16 * ch;
    float c = (float)c8 / 255.0f;
    switch (p.i[ch]) {
    case RGPU_TF_TABLE: {
        const int n = p.i[4 + ch] - 1;
        const float fk = std::floor(c * (float)n);
        const int k = fk >= (float)n ? n : (int)fk;
        if (k == n) {
            c = v[k];
        } else {
            const float vk = v[k], vk1 = v[k + 1], kf = (float)k, nf = (float)n;
            c = vk + (c - kf / nf) * nf * (vk1 - vk);
        }
        break;
    }
    case RGPU_TF_DISCRETE: {
        const int n = p.i[4 + ch];
        const float fk = std::floor(c * (float)n);
        c = v[fk >= (float)(n - 1) ? n - 1 : (int)fk];
        break;
    }
    case RGPU_TF_LINEAR: c = v[0] * c + v[1]; break;
    case RGPU_TF_GAMMA: c = v[0] * std::pow(c, v[1]) + v[2]; break;
    default: break;
    }
    const float b = c > 1.0f ? 1.0f : (c >= 0.0f ? c : 0.0f);
    return sat_u8(b * 255.0f);
}

// The four channels as one table of packed results; a channel whose function
// is the identity or an empty table keeps its value (is_dummy).
bool transfer_lut(const rgpu_primitive &p, uint32_t lut[256], std::string &err) {
    for (int ch = 0; ch < 4; ch++) {
        const int kind = p.i[ch];
        const bool tab = kind == RGPU_TF_TABLE || kind == RGPU_TF_DISCRETE;
        if (tab && (p.i[4 + ch] < 0 || p.i[4 + ch] > RGPU_TF_MAX_VALUES)) {
            err = "component transfer table longer than the primitive record";
            return false;
        }
    }
    for (uint32_t c = 0; c < 256; c++) {
        uint32_t o = 0;
        for (int ch = 0; ch < 4; ch++) {
            const int kind = p.i[ch];
            const bool dummy = (kind == RGPU_TF_TABLE || kind == RGPU_TF_DISCRETE) ? p.i[4 + ch] == 0
                               : !(kind == RGPU_TF_LINEAR || kind == RGPU_TF_GAMMA);
            o |= (dummy ? c : transfer_value(p, ch, c)) << (8 * ch);
        }
        lut[c] = o;
    }
    return true;
}

// A filter image: a device buffer holding a w x h image (stride w), its colour
// space, and the region the reference's Image carries (feOffset and feTile read
// it): the filter region for SourceGraphic / SourceAlpha, the primitive
// subregion after a crop, else the whole image (reg.w < 0 here).  Images are
// layer-sized (the inputs and what input-sized primitives make) or
// region-sized (what flood, composite, merge, blend, tile, turbulence,
// lighting, displacement map and feImage make), as tiny-skia pixmaps are in
// the reference; a region-sized image sits at the layer origin.
struct Img {
    uint32_t *p;
    bool linear;
    int32_t w, h;
    IRect reg{0, 0, -1, -1};
    size_t n() const { return (size_t)w * h; }
};

struct Runner {
    FilterScratch &sc;
    cudaStream_t s;
    int32_t w, h;
    size_t n;
    uint32_t next = 0;
    cudaError_t e = cudaSuccess;

    // scratch buffers are layer-sized: any image of this job fits
    uint32_t *fresh() { return sc.image(next++, n); }
    void ck(cudaError_t x) { if (e == cudaSuccess) e = x; }
    // a private copy of `in` in colour space `lin`
    Img private_in(Img in, bool lin) {
        uint32_t *o = fresh();
        if (in.linear != lin) ck(filter_color_space_copy(in.p, o, in.n(), lin, s));
        else ck(filter_copy(in.p, o, in.n(), s));
        return Img{o, lin, in.w, in.h};
    }
    Img in_space(Img in, bool lin) { return in.linear == lin ? in : private_in(in, lin); }
    // a cleared image of the given size
    Img blank(int32_t iw, int32_t ih, bool lin) {
        uint32_t *o = fresh();
        ck(filter_fill(o, (size_t)iw * ih, 0u, s));
        return Img{o, lin, iw, ih};
    }
};

}  // namespace

int run_filter_job(const FilterJob &job, uint32_t *content, uint32_t *result, FilterScratch &scratch, cudaStream_t s,
                   std::string &err, const std::vector<FeImageSurface> *images) {
    const rgpu_tree_view &t = *job.tree;
    Runner r{scratch, s, job.w, job.h, (size_t)job.w * job.h};
    // the layer the filters act on, in place, one filter after another
    uint32_t *source = content;
    for (uint32_t fi = 0; fi < job.filter_count; fi++) {
        const rgpu_filter &f = t.filters[t.filter_refs[job.filter_ref_offset + fi]];
        // the filter region: filter.rect.transform(ts).to_int_rect() fitted to
        // the layer (mod.rs:362-373)
        IRect region;
        bool ok = map_int_rect(job.ts, f.x, f.y, f.w, f.h, &region);
        if (ok) {
            int32_t l = std::max(region.x, 0), tp = std::max(region.y, 0);
            int32_t rr = std::min(region.x + region.w, job.w), b = std::min(region.y + region.h, job.h);
            ok = rr > l && b > tp;
            region = IRect{l, tp, rr - l, b - tp};
        }
        // A failure inside the filter (an invalid region or subregion, a tile
        // outside its input, sizes the reference cannot combine, a primitive
        // this device build does not run) clears the layer and rendering goes
        // on, as apply() does (mod.rs:343-354); the reason becomes a warning.
        std::string why = ok ? "" : "filter has an invalid region";
        std::vector<Img> results;
        auto input = [&](int32_t in) -> Img {
            if (in >= 0 && (size_t)in < results.size()) return results[in];
            if (in == RGPU_IN_SOURCE_ALPHA) {
                // SourceAlpha: RGB set to zero, alpha kept
                uint32_t *o = r.fresh();
                r.ck(filter_copy(source, o, r.n, s));
                r.ck(filter_alpha_only(o, r.n, s));
                return Img{o, false, job.w, job.h, region};
            }
            return Img{source, false, job.w, job.h, region};
        };
        for (uint32_t pi = 0; pi < f.prim_count && why.empty(); pi++) {
            const rgpu_primitive &p = t.prims[f.prim_offset + pi];
            IRect sub;
            if (!map_int_rect(job.ts, p.x, p.y, p.w, p.h, &sub)) { why = "primitive has an invalid subregion"; break; }
            // feOffset inherits its subregion from a referenced input (mod.rs:384-391)
            if (p.kind == RGPU_FE_OFFSET && p.in1 >= 0 && (size_t)p.in1 < results.size()) {
                sub = results[p.in1].reg;
                if (sub.w < 0) sub = IRect{0, 0, results[p.in1].w, results[p.in1].h};
            }
            const bool lin = p.linear_rgb != 0;
            const int32_t rw = region.w, rh = region.h;
            Img res{nullptr, lin, 0, 0};
            switch (p.kind) {
            case RGPU_FE_BLUR: {
                Img in = input(p.in1);
                float x, y;
                bool box;
                if (!resolve_std_dev(job.ts, p.f[0], p.f[1], &x, &y, &box)) { res = in; break; }
                res = r.private_in(in, lin);
                if (box) r.ck(filter_box_blur(res.p, r.fresh(), res.w, res.h, x, y, s));
                else r.ck(filter_iir_blur(res.p, scratch.plane(4 * r.n), res.w, res.h, x, y, s));
                break;
            }
            case RGPU_FE_COLOR_MATRIX: {
                // out of place from the input in the primitive's space: the
                // reference's copy-then-modify without the copy pass
                Img in = r.in_space(input(p.in1), lin);
                res = Img{r.fresh(), lin, in.w, in.h};
                r.ck(filter_color_matrix_to(in.p, res.p, res.n(), p.i[0], p.f, s));
                break;
            }
            case RGPU_FE_MORPHOLOGY: {
                Img in = r.in_space(input(p.in1), lin);
                res = Img{r.fresh(), lin, in.w, in.h};
                float sx = std::sqrt(job.ts.sx * job.ts.sx + job.ts.kx * job.ts.kx);
                float sy = std::sqrt(job.ts.ky * job.ts.ky + job.ts.sy * job.ts.sy);
                float rx = p.f[0] * sx, ry = p.f[1] * sy;
                if (!(rx > 0.0f && ry > 0.0f)) r.ck(filter_fill(res.p, res.n(), 0u, s));
                else r.ck(filter_morphology_to(in.p, res.p, r.fresh(), res.w, res.h, p.i[0] == 1, rx, ry, s));
                break;
            }
            case RGPU_FE_COMPOSITE: {
                // apply_composite (mod.rs:731-793): a region-sized image; the
                // arithmetic form pairs pixels by index, the others draw both
                // inputs at the origin
                Img a = r.in_space(input(p.in1), lin), b = r.in_space(input(p.in2), lin);
                if (p.i[0] == RGPU_OP_ARITHMETIC) res = Img{r.fresh(), lin, rw, rh};  // every pixel is written
                else res = r.blank(rw, rh, lin);
                if (p.i[0] == RGPU_OP_ARITHMETIC) {
                    const float k[4] = {p.f[0], p.f[1], p.f[2], p.f[3]};
                    if (a.n() < res.n() || b.n() < res.n()) { why = "arithmetic composite of images smaller than the region"; break; }
                    r.ck(filter_arithmetic(a.p, b.p, res.p, res.n(), k, s));
                } else {
                    uint32_t bm = RGPU_BLEND_SOURCE_OVER;
                    switch (p.i[0]) {
                    case RGPU_OP_IN: bm = RGPU_BLEND_SOURCE_IN; break;
                    case RGPU_OP_OUT: bm = RGPU_BLEND_SOURCE_OUT; break;
                    case RGPU_OP_ATOP: bm = RGPU_BLEND_SOURCE_ATOP; break;
                    case RGPU_OP_XOR: bm = RGPU_BLEND_XOR; break;
                    default: break;
                    }
                    r.ck(filter_draw(b.p, b.w, b.h, res.p, rw, rh, 0, 0, RGPU_BLEND_SOURCE_OVER, s));
                    r.ck(filter_draw(a.p, a.w, a.h, res.p, rw, rh, 0, 0, bm, s));
                }
                break;
            }
            case RGPU_FE_BLEND: {
                Img a = r.in_space(input(p.in1), lin), b = r.in_space(input(p.in2), lin);
                res = r.blank(rw, rh, lin);
                r.ck(filter_draw(b.p, b.w, b.h, res.p, rw, rh, 0, 0, RGPU_BLEND_SOURCE_OVER, s));
                r.ck(filter_draw(a.p, a.w, a.h, res.p, rw, rh, 0, 0, (uint32_t)p.i[0], s));
                break;
            }
            case RGPU_FE_MERGE: {
                res = r.blank(rw, rh, lin);
                for (int32_t k = 0; k < p.i[1]; k++) {
                    Img in = r.in_space(input(t.merge_inputs[p.i[0] + k]), lin);
                    r.ck(filter_draw(in.p, in.w, in.h, res.p, rw, rh, 0, 0, RGPU_BLEND_SOURCE_OVER, s));
                }
                break;
            }
            case RGPU_FE_FLOOD: {
                // Pixmap::fill(Color::from_rgba8(r, g, b, opacity.to_u8())): premultiplied
                float a = (float)(uint8_t)std::min(255.0f, std::max(0.0f, p.f[0] * 255.0f + 0.5f)) / 255.0f;
                auto pm = [&](int c) {
                    float v = (float)(uint8_t)c / 255.0f;
                    if (a != 1.0f) v = std::min(std::max(v * a, 0.0f), 1.0f);
                    return (uint32_t)(uint8_t)std::min(255.0f, v * 255.0f + 0.5f);
                };
                uint32_t a8 = (uint32_t)(uint8_t)std::min(255.0f, a * 255.0f + 0.5f);
                uint32_t v = pm(p.i[0]) | (pm(p.i[1]) << 8) | (pm(p.i[2]) << 16) | (a8 << 24);
                res = Img{r.fresh(), false, rw, rh};
                r.ck(filter_fill(res.p, res.n(), v, s));
                break;
            }
            case RGPU_FE_OFFSET: {
                Img in = input(p.in1);
                float sx = std::sqrt(job.ts.sx * job.ts.sx + job.ts.kx * job.ts.kx);
                float sy = std::sqrt(job.ts.ky * job.ts.ky + job.ts.sy * job.ts.sy);
                float dx = p.f[0] * sx, dy = p.f[1] * sy;
                if (approx_zero_ulps(dx) && approx_zero_ulps(dy)) { res = in; break; }
                res = r.blank(in.w, in.h, in.linear);
                r.ck(filter_draw(in.p, in.w, in.h, res.p, in.w, in.h, sat_i32(dx), sat_i32(dy), RGPU_BLEND_SOURCE_OVER,
                                 s));
                break;
            }
            case RGPU_FE_CONVOLVE: {
                // apply_convolve_matrix (mod.rs:919-933)
                Img in = r.in_space(input(p.in1), lin);
                ConvolveParams cp{};
                cp.cols = p.i[0]; cp.rows = p.i[1]; cp.tx = p.i[2]; cp.ty = p.i[3];
                cp.edge = p.i[4]; cp.preserve_alpha = p.i[5];
                cp.divisor = p.f[0]; cp.bias = p.f[1];
                if (cp.cols <= 0 || cp.rows <= 0 || cp.cols * cp.rows > (int)(sizeof(cp.k) / sizeof(float))) {
                    why = "convolve kernel larger than the primitive record";
                    break;
                }
                for (int k = 0; k < cp.cols * cp.rows; k++) cp.k[k] = p.f[2 + k];
                res = Img{r.fresh(), lin, in.w, in.h};
                r.ck(filter_convolve(in.p, res.p, in.w, in.h, cp, s));
                break;
            }
            case RGPU_FE_DIFFUSE:
            case RGPU_FE_SPECULAR: {
                // apply_diffuse_lighting / apply_specular_lighting + transform_light_source
                // (mod.rs:1020-1098): a region-sized result computed over the
                // input's pixels; lighting.rs indexes both with the input's
                // size, which only holds when the input is region-sized too
                Img in = input(p.in1);
                if (in.w != rw || in.h != rh) { why = "lighting input and filter region differ in size"; break; }
                LightingParams lp{};
                lp.specular = p.kind == RGPU_FE_SPECULAR;
                lp.kind = p.i[0];
                lp.surface_scale = p.f[0];
                lp.constant = p.f[1];
                lp.exponent = p.f[2];
                for (int k = 0; k < 3; k++) lp.color[k] = (uint32_t)(uint8_t)p.i[1 + k];
                const float d2r = 3.14159265358979323846f / 180.0f;
                if (lp.kind == RGPU_LIGHT_DISTANT) {
                    const float az = p.f[4] * d2r, el = p.f[5] * d2r;
                    lp.lv[0] = std::cos(az) * std::cos(el);
                    lp.lv[1] = std::sin(az) * std::cos(el);
                    lp.lv[2] = std::sin(el);
                } else {
                    lp.lv[0] = lp.lv[1] = lp.lv[2] = 1.0f;
                    const float sz = std::sqrt(job.ts.sx * job.ts.sx + job.ts.sy * job.ts.sy) / 1.41421356237309504880f;
                    float lx = p.f[4], ly = p.f[5];
                    map_point(job.ts, lx, ly);
                    lp.pos[0] = lx - (float)region.x;
                    lp.pos[1] = ly - (float)region.y;
                    lp.pos[2] = p.f[6] * sz;
                    if (lp.kind == RGPU_LIGHT_SPOT) {
                        float ax = p.f[7], ay = p.f[8];
                        map_point(job.ts, ax, ay);
                        ax -= (float)region.x;
                        ay -= (float)region.y;
                        const float az = p.f[9] * sz;
                        float dx = ax - lp.pos[0], dy = ay - lp.pos[1], dz = az - lp.pos[2];
                        const float len = std::sqrt(dx * dx + dy * dy + dz * dz);
                        if (!approx_zero_ulps(len)) { dx = dx / len; dy = dy / len; dz = dz / len; }
                        lp.dir[0] = dx; lp.dir[1] = dy; lp.dir[2] = dz;
                        lp.spot_exponent = p.f[10];
                        lp.has_cone = !std::isnan(p.f[11]);
                        lp.cone_cos = lp.has_cone ? std::cos(p.f[11] * d2r) : 0.0f;
                    }
                }
                res = r.blank(rw, rh, lin);
                r.ck(filter_lighting(in.p, res.p, rw, rh, lp, s));
                break;
            }
            case RGPU_FE_IMAGE: {
                // apply_image (mod.rs:861-889): the element was rendered into a
                // layer-sized surface of its own before the job; the result is
                // its region-sized corner, in sRGB
                const uint32_t *src = nullptr;
                if (images)
                    for (const auto &im : *images)
                        if (im.prim == f.prim_offset + pi) src = im.p;
                if (!src) { why = "feImage without its rendered element"; break; }
                res = r.blank(rw, rh, false);
                if (rw == job.w && rh == job.h) r.ck(filter_copy(src, res.p, res.n(), s));
                else r.ck(filter_draw(src, job.w, job.h, res.p, rw, rh, 0, 0, RGPU_BLEND_SOURCE, s));
                break;
            }
            case RGPU_FE_TILE: {
                // apply_tile (mod.rs:835-859): the input's region, cut from its
                // image, repeated over a region-sized image
                Img in = input(p.in1);
                IRect ir = in.reg.w < 0 ? IRect{0, 0, in.w, in.h} : in.reg;
                const int32_t sx0 = ir.x - region.x, sy0 = ir.y - region.y;
                const int32_t l = std::max(sx0, 0), tp = std::max(sy0, 0);
                const int32_t rr = std::min(sx0 + ir.w, in.w), bb = std::min(sy0 + ir.h, in.h);
                if (rr <= l || bb <= tp) { why = "feTile input region outside its image"; break; }
                res = Img{r.fresh(), false, rw, rh};
                r.ck(filter_tile(in.p, in.w, in.h, res.p, rw, rh, sx0, sy0, l, tp, rr - l, bb - tp, s));
                break;
            }
            case RGPU_FE_DISPLACEMENT_MAP: {
                // apply_displacement_map (mod.rs:958-986): displacement_map.rs
                // walks the map with the source's width and writes the
                // region-sized result at the same index, which only holds when
                // all three are the same size
                Img a = r.in_space(input(p.in1), lin), b = r.in_space(input(p.in2), lin);
                if (a.w != rw || a.h != rh || b.w != rw || b.h != rh) {
                    why = "displacement map inputs and filter region differ in size";
                    break;
                }
                const float sx = std::sqrt(job.ts.sx * job.ts.sx + job.ts.kx * job.ts.kx);
                const float sy = std::sqrt(job.ts.ky * job.ts.ky + job.ts.sy * job.ts.sy);
                res = Img{r.fresh(), lin, rw, rh};
                r.ck(filter_displacement_map(a.p, b.p, res.p, rw, rh, p.f[0] * sx, p.f[0] * sy, p.f[0], p.i[0], p.i[1],
                                             s));
                break;
            }
            case RGPU_FE_TURBULENCE: {
                // apply_turbulence (mod.rs:988-1018): a region-sized image
                if (p.i[0] > RGPU_TURB_MAX_OCTAVES) { why = "feTurbulence numOctaves above the device limit"; break; }
                res = r.blank(rw, rh, lin);
                const float sx = std::sqrt(job.ts.sx * job.ts.sx + job.ts.kx * job.ts.kx);
                const float sy = std::sqrt(job.ts.ky * job.ts.ky + job.ts.sy * job.ts.sy);
                if (!approx_zero_ulps(sx) && !approx_zero_ulps(sy)) {
                    // turbulence.rs init: the seed clamped into the generator's range;
                    // -seed wraps as in Rust, and -1 (from INT32_MIN) is M - 1 mod M
                    const int32_t m = 2147483647;
                    int32_t seed = p.i[1];
                    if (seed <= 0) seed = (int32_t)(0u - (uint32_t)seed) % (m - 1) + 1;
                    if (seed > m - 1) seed = m - 1;
                    TurbParams tp{};
                    tp.ox = (double)region.x - (double)job.ts.tx;
                    tp.oy = (double)region.y - (double)job.ts.ty;
                    tp.sx = sx; tp.sy = sy;
                    tp.bfx = p.f[0]; tp.bfy = p.f[1];
                    tp.octaves = p.i[0]; tp.stitch = p.i[2] != 0; tp.fractal = p.i[3] != 0;
                    tp.seed0 = (uint32_t)(((int64_t)seed % m + m) % m);
                    r.ck(filter_turbulence(res.p, rw, rh, tp, s));
                }
                break;
            }
            case RGPU_FE_COMPONENT_TRANSFER: {
                // apply_component_transfer (mod.rs:891-903)
                uint32_t lut[256];
                if (!transfer_lut(p, lut, why)) break;
                res = r.private_in(input(p.in1), lin);
                r.ck(filter_component_transfer(res.p, res.n(), lut, s));
                break;
            }
            case RGPU_FE_DROP_SHADOW: {
                // apply_drop_shadow (mod.rs:581-649): an input-sized image
                Img in = r.in_space(input(p.in1), lin);
                const float sx = std::sqrt(job.ts.sx * job.ts.sx + job.ts.kx * job.ts.kx);
                const float sy = std::sqrt(job.ts.ky * job.ts.ky + job.ts.sy * job.ts.sy);
                const float dx = p.f[2] * sx, dy = p.f[3] * sy;
                Img sh = r.private_in(in, lin);
                float x, y;
                bool box;
                if (resolve_std_dev(job.ts, p.f[0], p.f[1], &x, &y, &box)) {
                    if (box) r.ck(filter_box_blur(sh.p, r.fresh(), sh.w, sh.h, x, y, s));
                    else r.ck(filter_iir_blur(sh.p, scratch.plane(4 * r.n), sh.w, sh.h, x, y, s));
                }
                const uint32_t op8 = sat_u8(p.f[4] * 255.0f + 0.5f);
                const uint32_t flood = (uint32_t)(uint8_t)p.i[0] | ((uint32_t)(uint8_t)p.i[1] << 8) |
                                       ((uint32_t)(uint8_t)p.i[2] << 16) | (op8 << 24);
                res = Img{r.fresh(), lin, in.w, in.h};
                r.ck(filter_drop_shadow(in.p, sh.p, res.p, in.w, in.h, sat_i32(dx), sat_i32(dy), flood, lin, s));
                break;
            }
            default:
                why = "filter primitive not supported on the device";
                break;
            }
            if (!why.empty()) break;
            if (sub.x != region.x || sub.y != region.y || sub.w != region.w || sub.h != region.h) {
                // clip the result by clearing outside the subregion, in the
                // result's own pixel space (mod.rs:457-508)
                Img o{r.fresh(), res.linear, res.w, res.h, sub};
                r.ck(filter_copy(res.p, o.p, res.n(), s));
                if (p.kind == RGPU_FE_OFFSET) {
                    // feOffset is cropped to the region's size at the origin
                    r.ck(filter_crop(o.p, o.w, o.h, 0, 0, region.w, region.h, s));
                } else {
                    int32_t l = sub.x - region.x, tp = sub.y - region.y;
                    r.ck(filter_crop(o.p, o.w, o.h, l, tp, l + sub.w, tp + sub.h, s));
                }
                res = o;
            }
            results.push_back(res);
        }
        if (why.empty() && results.empty()) why = "filter has no primitives";  // Error::NoResults
        uint32_t *dst = (fi + 1 == job.filter_count) ? result : r.fresh();
        if (!why.empty()) {
            if (why != "filter has no primitives") {
                if (!err.empty()) err += "; ";
                err += why;
            }
            r.ck(filter_fill(dst, r.n, 0u, s));
        } else {
            // apply_to_canvas (mod.rs:1100-1114): back to sRGB, the layer
            // cleared, the result drawn at the origin
            Img last = results.back();
            if (last.w == job.w && last.h == job.h) {
                if (last.linear) r.ck(filter_color_space_copy(last.p, dst, r.n, false, s));
                else r.ck(filter_copy(last.p, dst, r.n, s));
            } else {
                Img srgb = last.linear ? r.private_in(last, false) : last;
                r.ck(filter_fill(dst, r.n, 0u, s));
                r.ck(filter_draw(srgb.p, srgb.w, srgb.h, dst, job.w, job.h, 0, 0, RGPU_BLEND_SOURCE_OVER, s));
            }
        }
        source = dst;
    }
    if (job.filter_count == 0) r.ck(filter_copy(content, result, r.n, s));
    if (r.e != cudaSuccess) {
        err = cudaGetErrorString(r.e);
        return RGPU_ERR_CUDA;
    }
    return RGPU_OK;
}

}  // namespace rgpu
