// Host-side f32 affine transforms with tiny-skia-path's arithmetic
// (transform.rs: concat with f64 products for skewed matrices, invert via an
// f64 determinant).  The host flattener composes every draw's transform with
// these so the device sees bit-identical matrices.
#pragma once
#include <cmath>
#include "rgpu_tree.h"

namespace rgpu {

struct Xf {
    float sx = 1, ky = 0, kx = 0, sy = 1, tx = 0, ty = 0;
    static Xf row(float a, float b, float c, float d, float e, float f) {
        Xf t; t.sx = a; t.ky = b; t.kx = c; t.sy = d; t.tx = e; t.ty = f; return t;
    }
    static Xf of(const rgpu_transform &t) { return row(t.sx, t.ky, t.kx, t.sy, t.tx, t.ty); }
    static Xf translate(float x, float y) { return row(1, 0, 0, 1, x, y); }
    static Xf scale(float x, float y) { return row(x, 0, 0, y, 0, 0); }
    bool identity() const { return sx == 1 && ky == 0 && kx == 0 && sy == 1 && tx == 0 && ty == 0; }
    bool skew() const { return kx != 0 || ky != 0; }
    bool has_scale() const { return sx != 1 || sy != 1; }
    bool finite() const {
        return std::isfinite(sx) && std::isfinite(ky) && std::isfinite(kx) && std::isfinite(sy) &&
               std::isfinite(tx) && std::isfinite(ty);
    }
};

inline float mam(float a, float b, float c, float d) { return (float)((double)a * (double)b + (double)c * (double)d); }

// a.pre_concat(b) == a * b
inline Xf concat(const Xf &a, const Xf &b) {
    if (a.identity()) return b;
    if (b.identity()) return a;
    if (!a.skew() && !b.skew())
        return Xf::row(a.sx * b.sx, 0, 0, a.sy * b.sy, a.sx * b.tx + a.tx, a.sy * b.ty + a.ty);
    return Xf::row(mam(a.sx, b.sx, a.kx, b.ky), mam(a.ky, b.sx, a.sy, b.ky), mam(a.sx, b.kx, a.kx, b.sy),
                   mam(a.ky, b.kx, a.sy, b.sy), mam(a.sx, b.tx, a.kx, b.ty) + a.tx, mam(a.ky, b.tx, a.sy, b.ty) + a.ty);
}
inline Xf pre_concat(const Xf &a, const Xf &b) { return concat(a, b); }
inline Xf post_concat(const Xf &a, const Xf &b) { return concat(b, a); }

inline bool invert(const Xf &t, Xf *out) {
    if (t.identity()) { *out = t; return true; }
    if (!t.skew()) {
        if (t.has_scale()) {
            float ix = 1.0f / t.sx, iy = 1.0f / t.sy;
            *out = Xf::row(ix, 0, 0, iy, -t.tx * ix, -t.ty * iy);
        } else {
            *out = Xf::translate(-t.tx, -t.ty);
        }
        return true;
    }
    double det = (double)t.sx * (double)t.sy - (double)t.kx * (double)t.ky;
    const float nz = 1.0f / 4096.0f;
    if (std::fabs((float)det) <= nz * nz * nz) return false;
    double inv = 1.0 / det;
    Xf r = Xf::row((float)(t.sy * inv), (float)(-t.ky * inv), (float)(-t.kx * inv), (float)(t.sx * inv),
                   (float)(((double)t.kx * t.ty - (double)t.sy * t.tx) * inv),
                   (float)(((double)t.ky * t.tx - (double)t.sx * t.ty) * inv));
    if (!r.finite()) return false;
    *out = r;
    return true;
}

// One point mapped by t (tiny-skia Transform::map_point).
inline void map_point(const Xf &t, float &x, float &y) {
    if (t.identity()) return;
    if (!t.skew() && !t.has_scale()) { x += t.tx; y += t.ty; return; }
    if (!t.skew()) { x = x * t.sx + t.tx; y = y * t.sy + t.ty; return; }
    const float nx = x * t.sx + y * t.kx + t.tx, ny = x * t.ky + y * t.sy + t.ty;
    x = nx; y = ny;
}

// Bounds of a rect mapped by t (4 corners, as NonZeroRect::transform).
inline bool map_rect(const Xf &t, float l, float tp, float r, float b, float out[4]) {
    float xs[4] = {l, r, r, l}, ys[4] = {tp, tp, b, b};
    float ml = 0, mt = 0, mr = 0, mb = 0;
    for (int i = 0; i < 4; i++) {
        float x, y;
        if (t.identity()) { x = xs[i]; y = ys[i]; }
        else if (!t.skew() && !t.has_scale()) { x = xs[i] + t.tx; y = ys[i] + t.ty; }
        else if (!t.skew()) { x = xs[i] * t.sx + t.tx; y = ys[i] * t.sy + t.ty; }
        else { x = xs[i] * t.sx + ys[i] * t.kx + t.tx; y = xs[i] * t.ky + ys[i] * t.sy + t.ty; }
        if (i == 0) { ml = mr = x; mt = mb = y; }
        else { ml = std::fmin(ml, x); mr = std::fmax(mr, x); mt = std::fmin(mt, y); mb = std::fmax(mb, y); }
    }
    out[0] = ml; out[1] = mt; out[2] = mr; out[3] = mb;
    return std::isfinite(ml) && std::isfinite(mt) && std::isfinite(mr) && std::isfinite(mb) && mr > ml && mb > mt;
}

}  // namespace rgpu
