// Per-pixel raster-pipeline arithmetic on the device: tiny-skia's lowp (u16
// lanes, div255 = (v+255)>>8) and highp (f32, store = round-to-nearest-even of
// clamp(v)*255) stage math for the paints and blend modes resvg uses
// (tiny-skia 0.12.0 pipeline/lowp.rs, pipeline/highp.rs, shaders/gradient.rs).
// Compiled with --fmad=false so every product and sum rounds separately.
#pragma once
#include <stdint.h>
#include "../device_types.h"
#include "rgpu_tree.h"

namespace rgpu {
namespace dev {

__device__ __forceinline__ uint16_t div255(uint32_t v) { return (uint16_t)(((uint16_t)(v + 255u)) >> 8); }
__device__ __forceinline__ uint16_t u16(uint32_t v) { return (uint16_t)v; }
__device__ __forceinline__ uint16_t inv16(uint16_t v) { return (uint16_t)(255 - v); }

__device__ __forceinline__ uint8_t unnorm(float v) {
    v = fmaxf(v, 0.0f);
    v = fminf(v, 1.0f);
    return (uint8_t)__float2int_rn(v * 255.0f);
}
__device__ __forceinline__ uint16_t sat_u16(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 65535.0f) return 65535;
    return (uint16_t)v;
}
constexpr float kInv255 = 1.0f / 255.0f;

__device__ __forceinline__ uint32_t pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return (r & 0xff) | ((g & 0xff) << 8) | ((b & 0xff) << 16) | ((a & 0xff) << 24);
}
__device__ __forceinline__ uint32_t ch(uint32_t p, int i) { return (p >> (8 * i)) & 0xff; }

__device__ __forceinline__ bool pre_scale(uint32_t blend) {
    return blend == RGPU_BLEND_DESTINATION || blend == RGPU_BLEND_DESTINATION_OVER || blend == RGPU_BLEND_PLUS ||
           blend == RGPU_BLEND_DESTINATION_OUT || blend == RGPU_BLEND_SOURCE_ATOP ||
           blend == RGPU_BLEND_SOURCE_OVER || blend == RGPU_BLEND_XOR;
}

__device__ __forceinline__ void lowp_blend(uint32_t blend, const uint16_t s[4], const uint16_t d[4], uint16_t o[4]) {
    uint16_t sa = s[3];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        switch (blend) {
        case RGPU_BLEND_CLEAR: o[i] = 0; break;
        case RGPU_BLEND_SOURCE_OVER: o[i] = u16(s[i] + div255(u16(d[i] * inv16(sa)))); break;
        case RGPU_BLEND_DESTINATION_OUT: o[i] = div255(u16(d[i] * inv16(sa))); break;
        case RGPU_BLEND_SOURCE_ATOP: o[i] = div255(u16(s[i] * d[3] + d[i] * inv16(sa))); break;
        case RGPU_BLEND_XOR: o[i] = div255(u16(s[i] * inv16(d[3]) + d[i] * inv16(sa))); break;
        case RGPU_BLEND_PLUS: o[i] = min((uint16_t)u16(s[i] + d[i]), (uint16_t)255); break;
        case RGPU_BLEND_MODULATE: o[i] = div255(u16(s[i] * d[i])); break;
        case RGPU_BLEND_SCREEN: o[i] = u16(s[i] + d[i] - div255(u16(s[i] * d[i]))); break;
        default: o[i] = s[i]; break;
        }
    }
}

__device__ __forceinline__ float hinv(float v) { return 1.0f - v; }

static __device__ __noinline__ float4 blend_generic(uint32_t mode, float4 sv, float4 dv) {
    const float s[4] = {sv.x, sv.y, sv.z, sv.w}, d[4] = {dv.x, dv.y, dv.z, dv.w};
    float o[4];
    float sa = s[3], da = d[3];
    switch (mode) {
    case RGPU_BLEND_CLEAR: return make_float4(0.f, 0.f, 0.f, 0.f);
    case RGPU_BLEND_SOURCE: { for (int i = 0; i < 4; i++) o[i] = s[i]; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_DESTINATION: { for (int i = 0; i < 4; i++) o[i] = d[i]; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_SOURCE_OVER: { for (int i = 0; i < 4; i++) o[i] = d[i] * hinv(sa) + s[i]; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_DESTINATION_OVER: { for (int i = 0; i < 4; i++) o[i] = s[i] * hinv(da) + d[i]; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_SOURCE_IN: { for (int i = 0; i < 4; i++) o[i] = s[i] * da; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_DESTINATION_IN: { for (int i = 0; i < 4; i++) o[i] = d[i] * sa; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_SOURCE_OUT: { for (int i = 0; i < 4; i++) o[i] = s[i] * hinv(da); return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_DESTINATION_OUT: { for (int i = 0; i < 4; i++) o[i] = d[i] * hinv(sa); return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_SOURCE_ATOP: { for (int i = 0; i < 4; i++) o[i] = s[i] * da + d[i] * hinv(sa); return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_DESTINATION_ATOP: { for (int i = 0; i < 4; i++) o[i] = d[i] * sa + s[i] * hinv(da); return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_XOR: { for (int i = 0; i < 4; i++) o[i] = s[i] * hinv(da) + d[i] * hinv(sa); return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_PLUS: { for (int i = 0; i < 4; i++) o[i] = fminf(s[i] + d[i], 1.0f); return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_MODULATE: { for (int i = 0; i < 4; i++) o[i] = s[i] * d[i]; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_SCREEN: { for (int i = 0; i < 4; i++) o[i] = s[i] + d[i] - s[i] * d[i]; return make_float4(o[0], o[1], o[2], o[3]); }
    case RGPU_BLEND_MULTIPLY:
        { for (int i = 0; i < 4; i++) o[i] = s[i] * hinv(da) + d[i] * hinv(sa) + s[i] * d[i];
          return make_float4(o[0], o[1], o[2], o[3]); }
    default: break;
    }
    if (mode <= RGPU_BLEND_MULTIPLY) {
        // separable modes with alpha = source-over
        for (int i = 0; i < 3; i++) {
            float s_ = s[i], d_ = d[i], x;
            switch (mode) {
            case RGPU_BLEND_DARKEN: x = s_ + d_ - fmaxf(s_ * da, d_ * sa); break;
            case RGPU_BLEND_LIGHTEN: x = s_ + d_ - fminf(s_ * da, d_ * sa); break;
            case RGPU_BLEND_DIFFERENCE: { float m = fminf(s_ * da, d_ * sa); x = s_ + d_ - (m + m); break; }
            case RGPU_BLEND_EXCLUSION: { float m = s_ * d_; x = s_ + d_ - (m + m); break; }
            case RGPU_BLEND_COLOR_BURN:
                if (d_ == da) x = d_ + s_ * hinv(da);
                else if (s_ == 0.0f) x = d_ * hinv(sa);
                else x = sa * (da - fminf(da, (da - d_) * sa * __fdiv_rn(1.0f, s_))) + s_ * hinv(da) + d_ * hinv(sa);
                break;
            case RGPU_BLEND_COLOR_DODGE:
                if (d_ == 0.0f) x = s_ * hinv(da);
                else if (s_ == sa) x = s_ + d_ * hinv(sa);
                else x = sa * fminf(da, (d_ * sa) * __fdiv_rn(1.0f, sa - s_)) + s_ * hinv(da) + d_ * hinv(sa);
                break;
            case RGPU_BLEND_HARD_LIGHT: {
                float y = (s_ + s_ <= sa) ? (s_ * d_) + (s_ * d_) : sa * da - 2.0f * ((da - d_) * (sa - s_));
                x = s_ * hinv(da) + d_ * hinv(sa) + y;
                break;
            }
            case RGPU_BLEND_OVERLAY: {
                float y = (d_ + d_ <= da) ? (s_ * d_) + (s_ * d_) : sa * da - 2.0f * ((da - d_) * (sa - s_));
                x = s_ * hinv(da) + d_ * hinv(sa) + y;
                break;
            }
            case RGPU_BLEND_SOFT_LIGHT: {
                float m = da > 0.0f ? __fdiv_rn(d_, da) : 0.0f;
                float s2 = s_ + s_;
                float m4 = (m + m) + (m + m);
                float dark_src = d_ * (sa + (s2 - sa) * (1.0f - m));
                float dark_dst = (m4 * m4 + m4) * (m - 1.0f) + 7.0f * m;
                float lite_dst = __fsqrt_rn(m) - m;
                float lite_src = d_ * sa + da * (s2 - sa) * ((d_ + d_) + (d_ + d_) <= da ? dark_dst : lite_dst);
                x = s_ * hinv(da) + d_ * hinv(sa) + (s2 <= sa ? dark_src : lite_src);
                break;
            }
            default: x = s_; break;
            }
            o[i] = x;
        }
        o[3] = sa + da * hinv(sa);
        return make_float4(o[0], o[1], o[2], o[3]);
    }
    // non-separable modes
    auto lum = [](float r, float g, float b) { return r * 0.30f + g * 0.59f + b * 0.11f; };
    auto sat = [](float r, float g, float b) { return fmaxf(fmaxf(r, g), b) - fminf(fminf(r, g), b); };
    float r, g, b;
    auto set_sat = [&](float s_) {
        float mn = fminf(fminf(r, g), b), mx = fmaxf(fmaxf(r, g), b);
        float st = mx - mn;
        r = st == 0.0f ? 0.0f : __fdiv_rn((r - mn) * s_, st);
        g = st == 0.0f ? 0.0f : __fdiv_rn((g - mn) * s_, st);
        b = st == 0.0f ? 0.0f : __fdiv_rn((b - mn) * s_, st);
    };
    auto set_lum = [&](float l) {
        float diff = l - lum(r, g, b);
        r += diff; g += diff; b += diff;
    };
    // tiny-skia's clip_color pulls channels above `a` back towards the
    // luminance and clamps negatives to zero; it has no separate pull-up of a
    // negative minimum (pinned against resvg's mix-blend-mode goldens).
    auto clip_color = [&](float a) {
        float mx = fmaxf(fmaxf(r, g), b);
        float l = lum(r, g, b);
        auto clip = [&](float c) {
            if (mx > a && mx - l != 0.0f) c = l + __fdiv_rn((c - l) * (a - l), mx - l);
            return fmaxf(c, 0.0f);
        };
        r = clip(r); g = clip(g); b = clip(b);
    };
    if (mode == RGPU_BLEND_HUE) {
        r = s[0] * sa; g = s[1] * sa; b = s[2] * sa;
        set_sat(sat(d[0], d[1], d[2]) * sa);
        set_lum(lum(d[0], d[1], d[2]) * sa);
        clip_color(sa * da);
    } else if (mode == RGPU_BLEND_SATURATION) {
        r = d[0] * sa; g = d[1] * sa; b = d[2] * sa;
        set_sat(sat(s[0], s[1], s[2]) * da);
        set_lum(lum(d[0], d[1], d[2]) * sa);
        clip_color(sa * da);
    } else if (mode == RGPU_BLEND_COLOR) {
        r = s[0] * da; g = s[1] * da; b = s[2] * da;
        set_lum(lum(d[0], d[1], d[2]) * sa);
        clip_color(sa * da);
    } else {
        r = d[0] * sa; g = d[1] * sa; b = d[2] * sa;
        set_lum(lum(s[0], s[1], s[2]) * da);
        clip_color(sa * da);
    }
    o[0] = r + d[0] * hinv(sa) + s[0] * hinv(da);
    o[1] = g + d[1] * hinv(sa) + s[1] * hinv(da);
    o[2] = b + d[2] * hinv(sa) + s[2] * hinv(da);
    o[3] = sa + da - sa * da;
    return make_float4(o[0], o[1], o[2], o[3]);
}


// highp blend with the common modes inlined.
__device__ __forceinline__ float4 blend4(uint32_t mode, float4 s, float4 d) {
    if (mode == RGPU_BLEND_SOURCE_OVER) {
        float ia = hinv(s.w);
        return make_float4(d.x * ia + s.x, d.y * ia + s.y, d.z * ia + s.z, d.w * ia + s.w);
    }
    if (mode == RGPU_BLEND_SOURCE) return s;
    if (mode == RGPU_BLEND_CLEAR) return make_float4(0.f, 0.f, 0.f, 0.f);
    return blend_generic(mode, s, d);
}
__device__ __forceinline__ void blend_sep(uint32_t mode, const float *s, const float *d, float *o) {
    float4 r = blend4(mode, make_float4(s[0], s[1], s[2], s[3]), make_float4(d[0], d[1], d[2], d[3]));
    o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = r.w;
}

// Gradient colour at device pixel (px, py) (premultiplied f32); false when the
// pixel lies in a two-point-conical region with no circle through it. The
// transform, flags, spread and interval count come from the paint (held in
// shared memory by the raster kernel); the rest from g, a record in global
// memory that no kernel writes while this one runs, so it is read through the
// read-only data path (__ldg).
__device__ __forceinline__ bool gradient_eval(const PaintRec &pr, const GradRec &g, int32_t px, int32_t py,
                                              float *c, bool premul_stage = true) {
    const uint32_t meta = pr.gmeta;
    const uint32_t gflags = meta & 0xFFu, gspread = (meta >> 8) & 0xFFu, gn = meta >> 16;
    float x = (float)px + 0.5f, y = (float)py + 0.5f;
    float tx = x * pr.gts[0] + y * pr.gts[2] + pr.gts[4];
    float ty = x * pr.gts[1] + y * pr.gts[3] + pr.gts[5];
    float t;
    if (gflags & GRAD_RADIAL_SIMPLE) {
        t = __fsqrt_rn(tx * tx + ty * ty);
    } else if (gflags & GRAD_RADIAL_CONICAL) {
        float dr = __ldg(&g.fr1) - __ldg(&g.fr0);
        float a = __ldg(&g.cdx) * __ldg(&g.cdx) + __ldg(&g.cdy) * __ldg(&g.cdy) - dr * dr;
        float b = tx * __ldg(&g.cdx) + ty * __ldg(&g.cdy) + __ldg(&g.fr0) * dr;
        float cc = tx * tx + ty * ty - __ldg(&g.fr0) * __ldg(&g.fr0);
        if (a == 0.0f) {
            if (b == 0.0f) return false;
            t = __fdiv_rn(cc, 2.0f * b);
            if (__ldg(&g.fr0) + t * dr < 0.0f) return false;
        } else {
            float disc = b * b - a * cc;
            if (disc < 0.0f) return false;
            float sq = __fsqrt_rn(disc);
            float t1 = __fdiv_rn(b + sq, a), t2 = __fdiv_rn(b - sq, a);
            float hi = fmaxf(t1, t2), lo = fminf(t1, t2);
            if (__ldg(&g.fr0) + hi * dr >= 0.0f) t = hi;
            else if (__ldg(&g.fr0) + lo * dr >= 0.0f) t = lo;
            else return false;
        }
    } else {
        t = tx;
    }
    if (gspread == RGPU_SPREAD_REFLECT) {
        float u = t - 1.0f;
        t = fabsf(u - 2.0f * floorf(u * 0.5f) - 1.0f);
        t = fminf(fmaxf(t, 0.0f), 1.0f);
    } else if (gspread == RGPU_SPREAD_REPEAT) {
        t = t - floorf(t);
        t = fminf(fmaxf(t, 0.0f), 1.0f);
    } else if (gflags & GRAD_PAD_CLAMP) {
        t = fminf(fmaxf(t, 0.0f), 1.0f);
    }
    // the interval: how many of t[1..n) are <= t. t[] is non-decreasing (the
    // host makes the stop positions monotonic), so this count is the index a
    // scan that stops at the first larger value finds; counting needs no
    // chain of dependent loads: t[] is read as up to three 16-byte vectors
    uint32_t idx = 0;
    if (!(gflags & GRAD_TWO_STOP)) {
        const float4 *tv = reinterpret_cast<const float4 *>(g.t);
        const float4 q0 = __ldg(tv);
        idx = (uint32_t)(1u < gn && t >= q0.y) + (uint32_t)(2u < gn && t >= q0.z) + (uint32_t)(3u < gn && t >= q0.w);
        if (gn > 4u) {
            const float4 q1 = __ldg(tv + 1);
            idx += (uint32_t)(t >= q1.x) + (uint32_t)(5u < gn && t >= q1.y) + (uint32_t)(6u < gn && t >= q1.z) +
                   (uint32_t)(7u < gn && t >= q1.w);
            if (gn > 8u) {
                const float4 q2 = __ldg(tv + 2);
                idx += (uint32_t)(t >= q2.x) + (uint32_t)(9u < gn && t >= q2.y) + (uint32_t)(10u < gn && t >= q2.z) +
                       (uint32_t)(11u < gn && t >= q2.w);
            }
        }
    }
    const float4 fv = __ldg(reinterpret_cast<const float4 *>(g.iv[idx].f));
    const float4 bv = __ldg(reinterpret_cast<const float4 *>(g.iv[idx].b));
    c[0] = t * fv.x + bv.x;
    c[1] = t * fv.y + bv.y;
    c[2] = t * fv.z + bv.z;
    c[3] = t * fv.w + bv.w;
    if ((gflags & GRAD_PREMUL) && premul_stage) { c[0] *= c[3]; c[1] *= c[3]; c[2] *= c[3]; }
    return true;
}

// lowp gradient colour (pipeline/lowp.rs gradient / evenly_spaced_2_stop_gradient
// + premultiply): the f32 interpolation is clamped, rounded to u16 by
// truncating v * 255 + 0.5, then premultiplied with div255.
__device__ __forceinline__ void gradient_eval_lowp(const PaintRec &pr, const GradRec &g, int32_t px, int32_t py,
                                                   uint16_t s[4]) {
    float c[4];
    gradient_eval(pr, g, px, py, c, false);
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] = (uint16_t)(fminf(fmaxf(c[k], 0.0f), 1.0f) * 255.0f + 0.5f);
    if (pr.gmeta & GRAD_PREMUL) {
#pragma unroll
        for (int k = 0; k < 3; k++) s[k] = div255((uint16_t)(s[k] * s[3]));
    }
}

// Two u16 lanes per register (r | b << 16, g | a << 16): every lane value of
// the lowp source-over path stays <= 255 * 255 + 255, so lanes never carry into
// each other and div255 = (v + 255) >> 8 runs on both at once.
__device__ __forceinline__ uint32_t div255_2(uint32_t v) { return ((v + 0x00FF00FFu) >> 8) & 0x00FF00FFu; }

// lowp gradient colour as two lane pairs (same arithmetic as gradient_eval_lowp).
__device__ __forceinline__ void gradient_eval_lowp2(const PaintRec &pr, const GradRec &g, int32_t px, int32_t py,
                                                    uint32_t &rb, uint32_t &ga) {
    float c[4];
    gradient_eval(pr, g, px, py, c, false);
    uint32_t s[4];
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] = (uint32_t)(fminf(fmaxf(c[k], 0.0f), 1.0f) * 255.0f + 0.5f);
    rb = s[0] | s[2] << 16;
    ga = s[1] | s[3] << 16;
    if (pr.gmeta & GRAD_PREMUL) {
        rb = div255_2(rb * s[3]);
        ga = (div255_2(ga * s[3]) & 0xFFFFu) | s[3] << 16;
    }
}

__device__ __forceinline__ float4 unpack_f(uint32_t p) {
    return make_float4((float)ch(p, 0) * kInv255, (float)ch(p, 1) * kInv255, (float)ch(p, 2) * kInv255,
                       (float)ch(p, 3) * kInv255);
}
__device__ __forceinline__ uint32_t pack_f(float4 o) { return pack(unnorm(o.x), unnorm(o.y), unnorm(o.z), unnorm(o.w)); }

// shade_pixel for the paints and blend modes off the inline fast path.
__device__ __forceinline__ uint32_t shade_pixel_slow(const PaintRec &pr, const GradRec *grad, int32_t lx,
                                                         int32_t ly, uint32_t cov, uint32_t dst) {
    const uint32_t blend = pr.blend;
    if (pr.flags & PAINT_LOWP) {
        uint16_t s[4] = {pr.rgba16[0], pr.rgba16[1], pr.rgba16[2], pr.rgba16[3]};
        if (pr.kind != 0) gradient_eval_lowp(pr, *grad, lx, ly, s);
        uint16_t d[4] = {(uint16_t)ch(dst, 0), (uint16_t)ch(dst, 1), (uint16_t)ch(dst, 2), (uint16_t)ch(dst, 3)};
        uint16_t o[4];
        if (cov == 255) {
            if (blend == RGPU_BLEND_SOURCE) {
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = s[i];
            } else lowp_blend(blend, s, d, o);
        } else {
            uint16_t c = sat_u16(((float)cov * kInv255) * 255.0f + 0.5f);
            if (pre_scale(blend)) {
#pragma unroll
                for (int i = 0; i < 4; i++) s[i] = div255(u16(s[i] * c));
                lowp_blend(blend, s, d, o);
            } else {
                uint16_t b[4];
                lowp_blend(blend, s, d, b);
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = div255(u16(d[i] * inv16(c) + b[i] * c));
            }
        }
        return pack(o[0], o[1], o[2], o[3]);
    }
    float4 s;
    if (pr.kind == 0) {
        s = make_float4(pr.colorf[0], pr.colorf[1], pr.colorf[2], pr.colorf[3]);
    } else if (pr.kind == 2) {
        // an image paint: the precomputed shader over the whole layer target
        // (bx = by = 0, bw = its width), which holds every covered pixel
        const ImageRec &im = *reinterpret_cast<const ImageRec *>(grad);
        s = __ldg(reinterpret_cast<const float4 *>(im.ptr) + (uint32_t)(ly * im.bw + lx));
    } else {
        float c[4];
        if (gradient_eval(pr, *grad, lx, ly, c)) s = make_float4(c[0], c[1], c[2], c[3]);
        else s = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float4 d = unpack_f(dst);
    float4 o;
    if (cov == 255) {
        o = blend4(blend, s, d);
    } else {
        const float c = (float)cov * kInv255;
        if (pre_scale(blend)) {
            s = make_float4(s.x * c, s.y * c, s.z * c, s.w * c);
            o = blend4(blend, s, d);
        } else {
            float4 b = blend4(blend, s, d);
            o = make_float4((b.x - d.x) * c + d.x, (b.y - d.y) * c + d.y, (b.z - d.z) * c + d.z, (b.w - d.w) * c + d.w);
        }
    }
    return pack_f(o);
}

// Blits one pixel of a fill with coverage `cov` (1..255) onto `dst`: the
// common lowp source-over case inline, every other paint and blend mode out of
// line (rare in practice, and kept out of the caller's registers).
__device__ __forceinline__ uint32_t shade_pixel(const PaintRec &pr, const GradRec *grad, int32_t lx, int32_t ly,
                                                uint32_t cov, uint32_t dst) {
    if (cov == 255 && (pr.flags & PAINT_MEMSET))
        return pack(pr.memset_rgba[0], pr.memset_rgba[1], pr.memset_rgba[2], pr.memset_rgba[3]);
    const uint32_t blend = pr.blend;
    if ((pr.flags & PAINT_LOWP) && blend == RGPU_BLEND_SOURCE_OVER) {
        // lowp source-over (pre-scaled by coverage), two lanes per register
        uint32_t rb, ga;
        if (pr.kind != 0) gradient_eval_lowp2(pr, *grad, lx, ly, rb, ga);
        else {
            const uint32_t w0 = *reinterpret_cast<const uint32_t *>(&pr.rgba16[0]);
            const uint32_t w1 = *reinterpret_cast<const uint32_t *>(&pr.rgba16[2]);
            rb = __byte_perm(w0, w1, 0x5410);
            ga = __byte_perm(w0, w1, 0x7632);
        }
        if (cov != 255) {
            rb = div255_2(rb * cov);
            ga = div255_2(ga * cov);
        }
        const uint32_t inv = 255u - (ga >> 16);
        rb += div255_2((dst & 0x00FF00FFu) * inv);
        ga += div255_2(((dst >> 8) & 0x00FF00FFu) * inv);
        return (rb & 0x00FF00FFu) | ((ga & 0x00FF00FFu) << 8);
    }
    return shade_pixel_slow(pr, grad, lx, ly, cov, dst);
}

// draw_pixmap of one pixel: highp pattern (already at the right pixel),
// opacity scale, blend, store.
__device__ __forceinline__ uint32_t composite_pixel(uint32_t src, uint32_t dst, float opacity, uint32_t blend) {
    if (blend == RGPU_BLEND_DESTINATION) return dst;
    float4 s = unpack_f(src);
    if (opacity != 1.0f) s = make_float4(s.x * opacity, s.y * opacity, s.z * opacity, s.w * opacity);
    return pack_f(blend4(blend, s, unpack_f(dst)));
}

// Pixmap::apply_mask (lowp): every channel *= m / 255 via div255.
__device__ __forceinline__ uint32_t mask_pixel(uint32_t p, uint32_t m) {
    return pack(div255(ch(p, 0) * m), div255(ch(p, 1) * m), div255(ch(p, 2) * m), div255(ch(p, 3) * m));
}

// Mask::from_pixmap value for one pixel.
__device__ __forceinline__ uint32_t mask_value(uint32_t p, bool luminance) {
    uint32_t a8 = ch(p, 3);
    if (!luminance) return a8;
    float r = (float)ch(p, 0) / 255.0f, g = (float)ch(p, 1) / 255.0f, b = (float)ch(p, 2) / 255.0f;
    float a = (float)a8 / 255.0f;
    if (a8 != 0) { r = __fdiv_rn(r, a); g = __fdiv_rn(g, a); b = __fdiv_rn(b, a); }
    // Rec. 709 luma coefficients (tiny-skia mask.rs from_pixmap)
    float luma = r * 0.2126f + g * 0.7152f + b * 0.0722f;
    float v = ceilf(fminf(fmaxf((luma * a) * 255.0f, 0.0f), 255.0f));
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint32_t)v;
}

}  // namespace dev
}  // namespace rgpu
