// Stroke outlining shared by the host and the device: tiny-skia-path 0.12's
// stroker (tiny-skia-path/src/stroker.rs, itself a port of Skia's
// SkStroke.cpp) with the curve helpers it uses (path_geometry.rs: quad/cubic
// evaluation, inflections, max curvature, cusps; conic.rs / path_builder.rs:
// conic to quads, unit arcs, circles).
//
// The outline is built in f32 exactly as tiny-skia builds it so that the
// filled stroke covers the same supersamples: offset curves are approximated
// by quads found by intersecting the tangent rays at both ends of a curve
// span and checking the mid-point against `inv_res_scale`, joins and caps
// are emitted with the same topology, round joins/caps are conics split into
// quads.  resvg strokes every path through this (crates/resvg/src/path.rs:113
// -> Pixmap::stroke_path -> Path::stroke) and fills the result with the
// non-zero rule.
//
// One source, two compilers: host/stroke.cpp instantiates it over
// std::vector storage, kernels/stroke.cu over fixed per-path slices of device
// memory (one thread per stroked path).  Both use IEEE f32/f64 arithmetic
// with no contraction; acos, cos and pow are evaluated in f64 and rounded to
// f32 on both sides, so host and device outlines agree bit for bit.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <cmath>

#if defined(__CUDACC__)
#define SK_HD __host__ __device__
#else
#define SK_HD
#endif

namespace rgpu {
namespace sk {

SK_HD inline float sk_sqrt(float v) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(v);
#else
    return std::sqrt(v);
#endif
}
SK_HD inline double sk_sqrt(double v) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(v);
#else
    return std::sqrt(v);
#endif
}
SK_HD inline float sk_fabs(float v) {
#ifdef __CUDA_ARCH__
    return fabsf(v);
#else
    return std::fabs(v);
#endif
}
SK_HD inline bool sk_isfinite(float v) {
#ifdef __CUDA_ARCH__
    return isfinite(v);
#else
    return std::isfinite(v);
#endif
}
// IEEE maxNum / minNum (a NaN operand yields the other one)
SK_HD inline float sk_fmax(float a, float b) {
#ifdef __CUDA_ARCH__
    return fmaxf(a, b);
#else
    return std::fmax(a, b);
#endif
}
SK_HD inline float sk_fmin(float a, float b) {
#ifdef __CUDA_ARCH__
    return fminf(a, b);
#else
    return std::fmin(a, b);
#endif
}
// f64 evaluation rounded to f32: the same f32 on both compilers
SK_HD inline float sk_acos(float v) {
#ifdef __CUDA_ARCH__
    return (float)acos((double)v);
#else
    return (float)std::acos((double)v);
#endif
}
SK_HD inline float sk_cos(float v) {
#ifdef __CUDA_ARCH__
    return (float)cos((double)v);
#else
    return (float)std::cos((double)v);
#endif
}
SK_HD inline float sk_pow(float a, float b) {
#ifdef __CUDA_ARCH__
    return (float)pow((double)a, (double)b);
#else
    return (float)std::pow((double)a, (double)b);
#endif
}
template <class T> SK_HD inline void sk_swap(T &a, T &b) {
    T t = a;
    a = b;
    b = t;
}

constexpr float kNearlyZero = 1.0f / 4096.0f;
constexpr float kRoot2Over2 = 0.707106781f;
constexpr float kPi = 3.14159265f;

struct Pt {
    float x = 0, y = 0;
};
SK_HD inline Pt P(float x, float y) { return Pt{x, y}; }
SK_HD inline Pt operator+(Pt a, Pt b) { return P(a.x + b.x, a.y + b.y); }
SK_HD inline Pt operator-(Pt a, Pt b) { return P(a.x - b.x, a.y - b.y); }
SK_HD inline Pt operator-(Pt a) { return P(-a.x, -a.y); }
SK_HD inline bool operator==(Pt a, Pt b) { return a.x == b.x && a.y == b.y; }
SK_HD inline bool operator!=(Pt a, Pt b) { return !(a == b); }
SK_HD inline Pt scaled(Pt a, float s) { return P(a.x * s, a.y * s); }
SK_HD inline float dot(Pt a, Pt b) { return a.x * b.x + a.y * b.y; }
SK_HD inline float cross(Pt a, Pt b) { return a.x * b.y - a.y * b.x; }
SK_HD inline float length_sqd(Pt a) { return a.x * a.x + a.y * a.y; }
SK_HD inline float dist_sqd(Pt a, Pt b) {
    float dx = a.x - b.x, dy = a.y - b.y;
    return dx * dx + dy * dy;
}
SK_HD inline bool finite(Pt a) { return sk_isfinite(a.x) && sk_isfinite(a.y); }
SK_HD inline bool can_normalize(Pt a) { return finite(a) && (a.x != 0.0f || a.y != 0.0f); }
SK_HD inline bool nearly_zero(float v) { return sk_fabs(v) <= kNearlyZero; }
SK_HD inline void rotate_ccw(Pt &p) { float t = p.y; p.y = -p.x; p.x = t; }
SK_HD inline void rotate_cw(Pt &p) { float t = p.x; p.x = -p.y; p.y = t; }

// Point::set_length_from: the length is computed in f64.
SK_HD inline bool set_length(Pt &pt, float x, float y, float length) {
    double xx = x, yy = y;
    double dmag = sk_sqrt(xx * xx + yy * yy);
    double dscale = (double)length / dmag;
    x *= (float)dscale;
    y *= (float)dscale;
    if (!sk_isfinite(x) || !sk_isfinite(y) || (x == 0.0f && y == 0.0f)) {
        pt = Pt{};
        return false;
    }
    pt = P(x, y);
    return true;
}
SK_HD inline bool set_length(Pt &pt, float length) { return set_length(pt, pt.x, pt.y, length); }
SK_HD inline bool normalize(Pt &pt) { return set_length(pt, pt.x, pt.y, 1.0f); }

// ---------------------------------------------------------------- path builder
enum : uint8_t { V_MOVE = 0, V_LINE = 1, V_QUAD = 2, V_CUBIC = 3, V_CLOSE = 4 };

// PathBuilder over a storage policy: Tr::Vec<T> is std::vector-like
// (push_back, back, operator[], size, empty, clear).
template <class Tr> struct BuilderT {
    typename Tr::template Vec<uint8_t> verbs;
    typename Tr::template Vec<Pt> pts;
    size_t last_move_to_index = 0;
    bool move_to_required = true;

    SK_HD void clear() {
        verbs.clear();
        pts.clear();
        last_move_to_index = 0;
        move_to_required = true;
    }
    SK_HD bool empty() const { return verbs.empty(); }
    SK_HD bool last_point(Pt *p) const {
        if (pts.empty()) return false;
        *p = pts.back();
        return true;
    }
    SK_HD void move_to(float x, float y) {
        if (!verbs.empty() && verbs.back() == V_MOVE) {
            pts.back() = P(x, y);
        } else {
            last_move_to_index = pts.size();
            move_to_required = false;
            verbs.push_back(V_MOVE);
            pts.push_back(P(x, y));
        }
    }
    SK_HD void inject_move_to_if_needed() {
        if (move_to_required) {
            if (last_move_to_index < pts.size()) move_to(pts[last_move_to_index].x, pts[last_move_to_index].y);
            else move_to(0.0f, 0.0f);
        }
    }
    SK_HD void line_to(float x, float y) {
        inject_move_to_if_needed();
        verbs.push_back(V_LINE);
        pts.push_back(P(x, y));
    }
    SK_HD void quad_to(float x1, float y1, float x, float y) {
        inject_move_to_if_needed();
        verbs.push_back(V_QUAD);
        pts.push_back(P(x1, y1));
        pts.push_back(P(x, y));
    }
    SK_HD void cubic_to(float x1, float y1, float x2, float y2, float x, float y) {
        inject_move_to_if_needed();
        verbs.push_back(V_CUBIC);
        pts.push_back(P(x1, y1));
        pts.push_back(P(x2, y2));
        pts.push_back(P(x, y));
    }
    SK_HD void close() {
        if (!verbs.empty() && verbs.back() != V_CLOSE) verbs.push_back(V_CLOSE);
        move_to_required = true;
    }
    SK_HD void set_last_point(Pt p) {
        if (pts.empty()) move_to(p.x, p.y);
        else pts.back() = p;
    }
    SK_HD bool zero_length_since_point(size_t start) const {
        size_t count = pts.size() - start;
        if (pts.size() < start || count < 2) return true;
        Pt first = pts[start];
        for (size_t i = 1; i < count; i++)
            if (first != pts[start + i]) return false;
        return true;
    }
    SK_HD void conic_points_to(Pt p1, Pt p2, float w);
    // appends `other`'s last contour reversed (PathBuilder::reverse_path_to)
    SK_HD void reverse_path_to(const BuilderT &other) {
        if (other.empty()) return;
        size_t off = other.pts.size() - 1;
        for (size_t i = other.verbs.size(); i-- > 0;) {
            switch (other.verbs[i]) {
            case V_MOVE: return;
            case V_LINE: {
                Pt a = other.pts[off - 1];
                off -= 1;
                line_to(a.x, a.y);
                break;
            }
            case V_QUAD: {
                Pt a = other.pts[off - 1], b = other.pts[off - 2];
                off -= 2;
                quad_to(a.x, a.y, b.x, b.y);
                break;
            }
            case V_CUBIC: {
                Pt a = other.pts[off - 1], b = other.pts[off - 2], c = other.pts[off - 3];
                off -= 3;
                cubic_to(a.x, a.y, b.x, b.y, c.x, c.y);
                break;
            }
            default: break;
            }
        }
    }
    SK_HD void push_builder(const BuilderT &o) {
        size_t base = pts.size();
        for (size_t i = 0; i < o.verbs.size(); i++) verbs.push_back(o.verbs[i]);
        for (size_t i = 0; i < o.pts.size(); i++) pts.push_back(o.pts[i]);
        if (!o.empty()) last_move_to_index = base + o.last_move_to_index;
    }
    SK_HD void push_circle(float x, float y, float r);
};

// ---------------------------------------------------------------- conics (path_geometry.rs Conic)
struct Conic {
    Pt p[3];
    float w = 0;
};

SK_HD inline bool between(float a, float b, float c) { return (a - b) * (c - b) <= 0.0f; }

SK_HD inline void conic_chop(const Conic &c, Conic out[2]) {
    float scale = 1.0f / (1.0f + c.w);
    float new_w = sk_sqrt(0.5f + c.w * 0.5f);
    Pt wp1 = P(c.w * c.p[1].x, c.w * c.p[1].y);
    Pt m = P((c.p[0].x + (wp1.x + wp1.x) + c.p[2].x) * scale * 0.5f,
             (c.p[0].y + (wp1.y + wp1.y) + c.p[2].y) * scale * 0.5f);
    if (!finite(m)) {
        double wd = c.w, w2 = wd * 2.0, sh = 1.0 / (1.0 + wd) * 0.5;
        m.x = (float)(((double)c.p[0].x + w2 * c.p[1].x + c.p[2].x) * sh);
        m.y = (float)(((double)c.p[0].y + w2 * c.p[1].y + c.p[2].y) * sh);
    }
    out[0].p[0] = c.p[0];
    out[0].p[1] = P((c.p[0].x + wp1.x) * scale, (c.p[0].y + wp1.y) * scale);
    out[0].p[2] = m;
    out[0].w = new_w;
    out[1].p[0] = m;
    out[1].p[1] = P((wp1.x + c.p[2].x) * scale, (wp1.y + c.p[2].y) * scale);
    out[1].p[2] = c.p[2];
    out[1].w = new_w;
}

// Depth-first halving to `level` (left half first), each chop's y-values
// pulled back between the parent's ends; iterative with an explicit stack.
SK_HD inline Pt *conic_subdivide(const Conic &src, Pt *pts, int level) {
    Conic stack[8];
    int lv[8];
    int sp = 0;
    stack[0] = src;
    lv[0] = level;
    sp = 1;
    while (sp > 0) {
        sp--;
        const Conic c = stack[sp];
        const int l = lv[sp];
        if (l == 0) {
            pts[0] = c.p[1];
            pts[1] = c.p[2];
            pts += 2;
            continue;
        }
        Conic dst[2];
        conic_chop(c, dst);
        float sy = c.p[0].y, ey = c.p[2].y;
        if (between(sy, c.p[1].y, ey)) {
            float my = dst[0].p[2].y;
            if (!between(sy, my, ey)) {
                float closer = sk_fabs(my - sy) < sk_fabs(my - ey) ? sy : ey;
                dst[0].p[2].y = closer;
                dst[1].p[0].y = closer;
            }
            if (!between(sy, dst[0].p[1].y, dst[0].p[2].y)) dst[0].p[1].y = sy;
            if (!between(dst[1].p[0].y, dst[1].p[1].y, ey)) dst[1].p[1].y = ey;
        }
        // right half below the left one: the left is taken first
        stack[sp] = dst[1];
        lv[sp] = l - 1;
        stack[sp + 1] = dst[0];
        lv[sp + 1] = l - 1;
        sp += 2;
    }
    return pts;
}

// AutoConicToQuads::compute with tolerance 0.25 (at least one split).
SK_HD inline int conic_to_quads(const Conic &c, Pt *out /* 1 + 2 * 16 */) {
    if (!finite(c.p[0]) || !finite(c.p[1]) || !finite(c.p[2])) return 0;
    float a = c.w - 1.0f;
    float k = a / (4.0f * (2.0f + a));
    float x = k * (c.p[0].x - 2.0f * c.p[1].x + c.p[2].x);
    float y = k * (c.p[0].y - 2.0f * c.p[1].y + c.p[2].y);
    float err = sk_sqrt(x * x + y * y);
    int pow2 = 0;
    for (int i = 0; i < 4; i++) {
        if (err <= 0.25f) break;
        err *= 0.25f;
        pow2++;
    }
    if (pow2 < 1) pow2 = 1;
    out[0] = c.p[0];
    conic_subdivide(c, out + 1, pow2);
    int quads = 1 << pow2;
    int npts = 2 * quads + 1;
    bool bad = false;
    for (int i = 0; i < npts; i++)
        if (!finite(out[i])) bad = true;
    if (bad)
        for (int i = 1; i < npts - 1; i++) out[i] = c.p[1];
    return quads;
}

template <class Tr> SK_HD inline void BuilderT<Tr>::conic_points_to(Pt p1, Pt p2, float w) {
    if (!(w > 0.0f)) {
        line_to(p2.x, p2.y);
    } else if (!sk_isfinite(w)) {
        line_to(p1.x, p1.y);
        line_to(p2.x, p2.y);
    } else if (w == 1.0f) {
        quad_to(p1.x, p1.y, p2.x, p2.y);
    } else {
        inject_move_to_if_needed();
        Pt last = pts.back();
        Pt q[33];
        Conic c;
        c.p[0] = last; c.p[1] = p1; c.p[2] = p2; c.w = w;
        int n = conic_to_quads(c, q);
        for (int i = 0; i < n; i++) quad_to(q[1 + 2 * i].x, q[1 + 2 * i].y, q[2 + 2 * i].x, q[2 + 2 * i].y);
    }
}

template <class Tr> SK_HD inline void BuilderT<Tr>::push_circle(float x, float y, float r) {
    float l = x - r, t = y - r, w = r + r, h = r + r;
    float rr = l + w, b = t + h;
    if (!(sk_isfinite(l) && sk_isfinite(t) && sk_isfinite(rr) && sk_isfinite(b) && l < rr && t < b)) return;
    float cx = l + (rr - l) * 0.5f, cy = t + (b - t) * 0.5f;
    move_to(rr, cy);
    conic_points_to(P(rr, b), P(cx, b), kRoot2Over2);
    conic_points_to(P(l, b), P(l, cy), kRoot2Over2);
    conic_points_to(P(l, t), P(cx, t), kRoot2Over2);
    conic_points_to(P(rr, t), P(rr, cy), kRoot2Over2);
    close();
}

// tiny-skia Transform::map_points for the unit-arc transform.
struct Ts {
    float sx = 1, ky = 0, kx = 0, sy = 1, tx = 0, ty = 0;
};
SK_HD inline bool ts_identity(const Ts &t) { return t.sx == 1 && t.ky == 0 && t.kx == 0 && t.sy == 1 && t.tx == 0 && t.ty == 0; }
SK_HD inline bool ts_skew(const Ts &t) { return t.kx != 0 || t.ky != 0; }
SK_HD inline float mam(float a, float b, float c, float d) { return (float)((double)a * b + (double)c * d); }
SK_HD inline Ts ts_concat(const Ts &a, const Ts &b) {
    if (ts_identity(a)) return b;
    if (ts_identity(b)) return a;
    Ts r;
    if (!ts_skew(a) && !ts_skew(b)) {
        r.sx = a.sx * b.sx; r.ky = 0; r.kx = 0; r.sy = a.sy * b.sy;
        r.tx = a.sx * b.tx + a.tx; r.ty = a.sy * b.ty + a.ty;
        return r;
    }
    r.sx = mam(a.sx, b.sx, a.kx, b.ky);
    r.ky = mam(a.ky, b.sx, a.sy, b.ky);
    r.kx = mam(a.sx, b.kx, a.kx, b.sy);
    r.sy = mam(a.ky, b.kx, a.sy, b.sy);
    r.tx = mam(a.sx, b.tx, a.kx, b.ty) + a.tx;
    r.ty = mam(a.ky, b.tx, a.sy, b.ty) + a.ty;
    return r;
}
SK_HD inline void ts_map(const Ts &t, Pt *p, int n) {
    if (ts_identity(t)) return;
    bool translate_only = !ts_skew(t) && t.sx == 1 && t.sy == 1;
    for (int i = 0; i < n; i++) {
        if (translate_only) { p[i].x += t.tx; p[i].y += t.ty; }
        else if (!ts_skew(t)) { p[i].x = p[i].x * t.sx + t.tx; p[i].y = p[i].y * t.sy + t.ty; }
        else {
            float x = p[i].x * t.sx + p[i].y * t.kx + t.tx;
            float y = p[i].x * t.ky + p[i].y * t.sy + t.ty;
            p[i].x = x; p[i].y = y;
        }
    }
}

// Conic::build_unit_arc; returns the number of conics (0 = none).
SK_HD inline int build_unit_arc(Pt u_start, Pt u_stop, bool ccw, const Ts &user, Conic dst[5]) {
    float x = dot(u_start, u_stop);
    float y = cross(u_start, u_stop);
    float abs_y = sk_fabs(y);
    if (abs_y <= kNearlyZero && x > 0.0f && ((y >= 0.0f && !ccw) || (y <= 0.0f && ccw))) return 0;
    if (ccw) y = -y;
    int quadrant = 0;
    if (y == 0.0f) {
        quadrant = 2;
    } else if (x == 0.0f) {
        quadrant = y > 0.0f ? 1 : 3;
    } else {
        if (y < 0.0f) quadrant += 2;
        if ((x < 0.0f) != (y < 0.0f)) quadrant += 1;
    }
    const float qx[9] = {1, 1, 0, -1, -1, -1, 0, 1, 1}, qy[9] = {0, 1, 1, 1, 0, -1, -1, -1, 0};
    auto qp = [&](int i) { return P(qx[i], qy[i]); };
    int count = quadrant;
    for (int i = 0; i < count; i++) {
        dst[i].p[0] = qp(i * 2);
        dst[i].p[1] = qp(i * 2 + 1);
        dst[i].p[2] = qp(i * 2 + 2);
        dst[i].w = kRoot2Over2;
    }
    Pt final_pt = P(x, y);
    Pt last_q = qp(quadrant * 2);
    float d = dot(last_q, final_pt);
    if (d < 1.0f) {
        Pt off = P(last_q.x + x, last_q.y + y);
        float cos_half = sk_sqrt((1.0f + d) / 2.0f);
        set_length(off, 1.0f / cos_half);
        if (can_normalize(last_q - off)) {
            dst[count].p[0] = last_q;
            dst[count].p[1] = off;
            dst[count].p[2] = final_pt;
            dst[count].w = cos_half;
            count++;
        }
    }
    // from_sin_cos(u_start.y, u_start.x), pre_scale(1, -1) when ccw, post_concat(user)
    Ts t;
    t.sx = u_start.x; t.ky = u_start.y; t.kx = -u_start.y; t.sy = u_start.x; t.tx = 0; t.ty = 0;
    if (!(sk_isfinite(t.sx) && sk_isfinite(t.ky))) return 0;
    if (ccw) {
        Ts s;
        s.sy = -1.0f;
        t = ts_concat(t, s);
    }
    t = ts_concat(user, t);
    for (int i = 0; i < count; i++) ts_map(t, dst[i].p, 3);
    return count;
}

// ---------------------------------------------------------------- curve helpers (path_geometry.rs)
SK_HD inline bool valid_unit_divide(float numer, float denom, float *r) {
    if (numer < 0.0f) { numer = -numer; denom = -denom; }
    if (denom == 0.0f || numer == 0.0f || numer >= denom) return false;
    float v = numer / denom;
    if (!(v > 0.0f && v < 1.0f)) return false;
    *r = v;
    return true;
}

SK_HD inline int find_unit_quad_roots(float a, float b, float c, float roots[3]) {
    if (a == 0.0f) return valid_unit_divide(-c, b, &roots[0]) ? 1 : 0;
    double dr = (double)b * b - 4.0 * (double)a * c;
    if (dr < 0.0) return 0;
    float r = (float)sk_sqrt(dr);
    if (!sk_isfinite(r)) return 0;
    float q = b < 0.0f ? -(b - r) / 2.0f : -(b + r) / 2.0f;
    int n = 0;
    if (valid_unit_divide(q, a, &roots[n])) n++;
    if (valid_unit_divide(c, q, &roots[n])) n++;
    if (n == 2) {
        if (roots[0] > roots[1]) sk_swap(roots[0], roots[1]);
        else if (roots[0] == roots[1]) n--;
    }
    return n;
}

SK_HD inline Pt eval_quad_at(const Pt q[3], float t) {
    float bx = (q[1].x - q[0].x) * 2.0f, by = (q[1].y - q[0].y) * 2.0f;
    float ax = q[2].x - (q[1].x + q[1].x) + q[0].x, ay = q[2].y - (q[1].y + q[1].y) + q[0].y;
    return P((ax * t + bx) * t + q[0].x, (ay * t + by) * t + q[0].y);
}

SK_HD inline Pt eval_quad_tangent_at(const Pt q[3], float t) {
    if ((t == 0.0f && q[0] == q[1]) || (t == 1.0f && q[1] == q[2])) return q[2] - q[0];
    float bx = q[1].x - q[0].x, by = q[1].y - q[0].y;
    float ax = q[2].x - q[1].x - bx, ay = q[2].y - q[1].y - by;
    float tx = ax * t + bx, ty = ay * t + by;
    return P(tx + tx, ty + ty);
}

SK_HD inline float find_quad_max_curvature(const Pt q[3]) {
    float ax = q[1].x - q[0].x, ay = q[1].y - q[0].y;
    float bx = q[0].x - q[1].x - q[1].x + q[2].x, by = q[0].y - q[1].y - q[1].y + q[2].y;
    float numer = -(ax * bx + ay * by);
    float denom = bx * bx + by * by;
    if (denom < 0.0f) { numer = -numer; denom = -denom; }
    if (numer <= 0.0f) return 0.0f;
    if (numer >= denom) return 1.0f;
    float t = numer / denom;
    return t;
}

SK_HD inline Pt eval_cubic_pos_at(const Pt c[4], float t) {
    float ax = c[3].x + 3.0f * (c[1].x - c[2].x) - c[0].x, ay = c[3].y + 3.0f * (c[1].y - c[2].y) - c[0].y;
    float bx = 3.0f * (c[2].x - (c[1].x + c[1].x) + c[0].x), by = 3.0f * (c[2].y - (c[1].y + c[1].y) + c[0].y);
    float cx = 3.0f * (c[1].x - c[0].x), cy = 3.0f * (c[1].y - c[0].y);
    return P(((ax * t + bx) * t + cx) * t + c[0].x, ((ay * t + by) * t + cy) * t + c[0].y);
}

SK_HD inline Pt eval_cubic_derivative(const Pt c[4], float t) {
    float ax = c[3].x + 3.0f * (c[1].x - c[2].x) - c[0].x, ay = c[3].y + 3.0f * (c[1].y - c[2].y) - c[0].y;
    float bx0 = c[2].x - (c[1].x + c[1].x) + c[0].x, by0 = c[2].y - (c[1].y + c[1].y) + c[0].y;
    float bx = bx0 + bx0, by = by0 + by0;
    float cx = c[1].x - c[0].x, cy = c[1].y - c[0].y;
    return P((ax * t + bx) * t + cx, (ay * t + by) * t + cy);
}

SK_HD inline Pt eval_cubic_tangent_at(const Pt c[4], float t) {
    if ((t == 0.0f && c[0] == c[1]) || (t == 1.0f && c[2] == c[3])) {
        Pt tan = t == 0.0f ? c[2] - c[0] : c[3] - c[1];
        if (tan.x == 0.0f && tan.y == 0.0f) tan = c[3] - c[0];
        return tan;
    }
    return eval_cubic_derivative(c, t);
}

SK_HD inline void chop_cubic_at2(const Pt s[4], float t, Pt d[7]) {
    auto interp = [t](Pt a, Pt b) { return P(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t); };
    Pt ab = interp(s[0], s[1]), bc = interp(s[1], s[2]), cd = interp(s[2], s[3]);
    Pt abc = interp(ab, bc), bcd = interp(bc, cd), abcd = interp(abc, bcd);
    d[0] = s[0]; d[1] = ab; d[2] = abc; d[3] = abcd; d[4] = bcd; d[5] = cd; d[6] = s[3];
}

SK_HD inline int find_cubic_inflections(const Pt s[4], float t[3]) {
    float ax = s[1].x - s[0].x, ay = s[1].y - s[0].y;
    float bx = s[2].x - 2.0f * s[1].x + s[0].x, by = s[2].y - 2.0f * s[1].y + s[0].y;
    float cx = s[3].x + 3.0f * (s[1].x - s[2].x) - s[0].x, cy = s[3].y + 3.0f * (s[1].y - s[2].y) - s[0].y;
    return find_unit_quad_roots(bx * cy - by * cx, ax * cy - ay * cx, ax * by - ay * bx, t);
}

SK_HD inline float clamp01(float v) {
    if (!sk_isfinite(v)) return 0.0f;
    return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
}

SK_HD inline void formulate_f1_dot_f2(const float s[4], float out[4]) {
    float a = s[1] - s[0];
    float b = s[2] - 2.0f * s[1] + s[0];
    float c = s[3] + 3.0f * (s[1] - s[2]) - s[0];
    out[0] = c * c;
    out[1] = 3.0f * b * c;
    out[2] = 2.0f * b * b + c * a;
    out[3] = a * b;
}

SK_HD inline int solve_cubic_poly(const float co[4], float t[3]) {
    if (nearly_zero(co[0])) {
        float tmp[3];
        int n = find_unit_quad_roots(co[1], co[2], co[3], tmp);
        for (int i = 0; i < n; i++) t[i] = tmp[i];
        return n;
    }
    float inva = 1.0f / co[0];
    float a = co[1] * inva, b = co[2] * inva, c = co[3] * inva;
    float q = (a * a - b * 3.0f) / 9.0f;
    float r = (2.0f * a * a * a - 9.0f * a * b + 27.0f * c) / 54.0f;
    float q3 = q * q * q;
    float r2_minus_q3 = r * r - q3;
    float adiv3 = a / 3.0f;
    if (r2_minus_q3 < 0.0f) {
        float v = r / sk_sqrt(q3);
        v = v < -1.0f ? -1.0f : (v > 1.0f ? 1.0f : v);
        float theta = sk_acos(v);
        float neg2_root_q = -2.0f * sk_sqrt(q);
        t[0] = clamp01(neg2_root_q * sk_cos(theta / 3.0f) - adiv3);
        t[1] = clamp01(neg2_root_q * sk_cos((theta + 2.0f * kPi) / 3.0f) - adiv3);
        t[2] = clamp01(neg2_root_q * sk_cos((theta - 2.0f * kPi) / 3.0f) - adiv3);
        if (t[0] > t[1]) sk_swap(t[0], t[1]);
        if (t[1] > t[2]) sk_swap(t[1], t[2]);
        if (t[0] > t[1]) sk_swap(t[0], t[1]);
        int len = 3;
        if (t[1] == t[2]) len = 2;
        if (t[0] == t[1]) {
            for (int i = 0; i < len - 1; i++) t[i] = t[i + 1];
            len--;
        }
        return len;
    }
    float aa = sk_fabs(r) + sk_sqrt(r2_minus_q3);
    aa = sk_pow(aa, 0.3333333f);
    if (r > 0.0f) aa = -aa;
    if (aa != 0.0f) aa += q / aa;
    t[0] = clamp01(aa - adiv3);
    return 1;
}

SK_HD inline int find_cubic_max_curvature(const Pt s[4], float t[3]) {
    float xs[4] = {s[0].x, s[1].x, s[2].x, s[3].x}, ys[4] = {s[0].y, s[1].y, s[2].y, s[3].y};
    float cx[4], cy[4];
    formulate_f1_dot_f2(xs, cx);
    formulate_f1_dot_f2(ys, cy);
    for (int i = 0; i < 4; i++) cx[i] += cy[i];
    return solve_cubic_poly(cx, t);
}

SK_HD inline bool on_same_side(const Pt s[4], int test, int line) {
    Pt origin = s[line];
    Pt l = s[line + 1] - origin;
    float c0 = cross(l, s[test] - origin), c1 = cross(l, s[test + 1] - origin);
    return c0 * c1 >= 0.0f;
}

SK_HD inline bool find_cubic_cusp(const Pt s[4], float *t_out) {
    if (s[0] == s[1] || s[2] == s[3]) return false;
    if (on_same_side(s, 0, 2) || on_same_side(s, 2, 0)) return false;
    float t[3];
    int n = find_cubic_max_curvature(s, t);
    for (int i = 0; i < n; i++) {
        if (0.0f >= t[i] || t[i] >= 1.0f) continue;
        Pt d = eval_cubic_derivative(s, t[i]);
        float mag = length_sqd(d);
        float precision = (dist_sqd(s[1], s[0]) + dist_sqd(s[2], s[1]) + dist_sqd(s[3], s[2])) * 1e-8f;
        if (mag < precision) {
            *t_out = t[i];
            return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------- stroker (stroker.rs)
enum class Reduction { Point, Line, Quad, Degenerate, Degenerate2, Degenerate3 };
enum class Result { Split, Degenerate, Quad };
enum class RayKind { CtrlPt, ResultType };
enum class Angle { NearlyLine, Shallow, Sharp, Nearly180 };
// recursion limits: tangent, cubic, conic, quad
SK_HD inline int recursive_limit(int i) { return i == 0 ? 5 * 3 : i == 1 ? 26 * 3 : 11 * 3; }

SK_HD inline bool degenerate_vector(Pt v) { return !can_normalize(v); }

SK_HD inline float pt_to_line(Pt pt, Pt a, Pt b) {
    Pt dxy = b - a;
    Pt ab0 = pt - a;
    float numer = dot(dxy, ab0);
    float denom = dot(dxy, dxy);
    float t = numer / denom;
    if (t >= 0.0f && t <= 1.0f) {
        Pt hit = P(a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t);
        return dist_sqd(hit, pt);
    }
    return length_sqd(ab0);
}

SK_HD inline bool quad_in_line(const Pt q[3]) {
    float pt_max = -1.0f;
    int o1 = 0, o2 = 0;
    for (int i = 0; i < 2; i++)
        for (int j = i + 1; j < 3; j++) {
            Pt d = q[j] - q[i];
            float m = sk_fmax(sk_fabs(d.x), sk_fabs(d.y));
            if (pt_max < m) { o1 = i; o2 = j; pt_max = m; }
        }
    int mid = o1 ^ o2 ^ 3;
    float slop = pt_max * pt_max * 0.000005f;
    return pt_to_line(q[mid], q[o1], q[o2]) <= slop;
}

SK_HD inline bool cubic_in_line(const Pt c[4]) {
    float pt_max = -1.0f;
    int o1 = 0, o2 = 0;
    for (int i = 0; i < 3; i++)
        for (int j = i + 1; j < 4; j++) {
            Pt d = c[j] - c[i];
            float m = sk_fmax(sk_fabs(d.x), sk_fabs(d.y));
            if (pt_max < m) { o1 = i; o2 = j; pt_max = m; }
        }
    int mid1 = (1 + (2 >> o2)) >> o1;
    int mid2 = o1 ^ o2 ^ mid1;
    float slop = pt_max * pt_max * 0.00001f;
    return pt_to_line(c[mid1], c[o1], c[o2]) <= slop && pt_to_line(c[mid2], c[o1], c[o2]) <= slop;
}

SK_HD inline Reduction check_quad_linear(const Pt q[3], Pt *reduction) {
    bool dab = degenerate_vector(q[1] - q[0]), dbc = degenerate_vector(q[2] - q[1]);
    if (dab && dbc) return Reduction::Point;
    if (dab || dbc) return Reduction::Line;
    if (!quad_in_line(q)) return Reduction::Quad;
    float t = find_quad_max_curvature(q);
    if (t == 0.0f || t == 1.0f) return Reduction::Line;
    *reduction = eval_quad_at(q, t);
    return Reduction::Degenerate;
}

SK_HD inline Reduction check_cubic_linear(const Pt c[4], Pt reduction[3], Pt *tangent_pt) {
    bool dab = degenerate_vector(c[1] - c[0]);
    bool dbc = degenerate_vector(c[2] - c[1]);
    bool dcd = degenerate_vector(c[3] - c[2]);
    if (dab && dbc && dcd) return Reduction::Point;
    if ((int)dab + (int)dbc + (int)dcd == 2) return Reduction::Line;
    if (!cubic_in_line(c)) {
        *tangent_pt = dab ? c[2] : c[1];
        return Reduction::Quad;
    }
    float t[3];
    int n = find_cubic_max_curvature(c, t);
    int r = 0;
    for (int i = 0; i < n; i++) {
        if (0.0f >= t[i] || t[i] >= 1.0f) continue;
        reduction[r] = eval_cubic_pos_at(c, t[i]);
        if (reduction[r] != c[0] && reduction[r] != c[3]) r++;
    }
    switch (r) {
    case 0: return Reduction::Line;
    case 1: return Reduction::Degenerate;
    case 2: return Reduction::Degenerate2;
    default: return Reduction::Degenerate3;
    }
}

SK_HD inline Angle dot_to_angle_type(float d) {
    if (d >= 0.0f) return nearly_zero(1.0f - d) ? Angle::NearlyLine : Angle::Shallow;
    return nearly_zero(1.0f + d) ? Angle::Nearly180 : Angle::Sharp;
}

SK_HD inline bool is_clockwise(Pt before, Pt after) { return before.x * after.y > before.y * after.x; }

SK_HD inline bool set_normal_unit_normal(Pt before, Pt after, float scale, float radius, Pt *normal, Pt *unit) {
    if (!set_length(*unit, (after.x - before.x) * scale, (after.y - before.y) * scale, 1.0f)) return false;
    rotate_ccw(*unit);
    *normal = scaled(*unit, radius);
    return true;
}

SK_HD inline bool set_normal_unit_normal2(Pt vec, float radius, Pt *normal, Pt *unit) {
    if (!set_length(*unit, vec.x, vec.y, 1.0f)) return false;
    rotate_ccw(*unit);
    *normal = scaled(*unit, radius);
    return true;
}

SK_HD inline bool points_within_dist(Pt a, Pt b, float limit) { return dist_sqd(a, b) <= limit * limit; }

SK_HD inline bool sharp_angle(const Pt q[3]) {
    Pt smaller = q[1] - q[0];
    Pt larger = q[1] - q[2];
    float smaller_len = length_sqd(smaller);
    float larger_len = length_sqd(larger);
    if (smaller_len > larger_len) {
        sk_swap(smaller, larger);
        larger_len = smaller_len;
    }
    if (!set_length(smaller, larger_len)) return false;
    return dot(smaller, larger) > 0.0f;
}

SK_HD inline int intersect_quad_ray(const Pt line[2], const Pt q[3], float roots[3]) {
    Pt vec = line[1] - line[0];
    float r[3];
    for (int n = 0; n < 3; n++) r[n] = (q[n].y - line[0].y) * vec.x - (q[n].x - line[0].x) * vec.y;
    float A = r[2], B = r[1], C = r[0];
    A += C - 2.0f * B;
    B -= C;
    return find_unit_quad_roots(A, 2.0f * B, C, roots);
}

struct QuadConstruct {
    Pt quad[3];
    Pt tangent_start, tangent_end;
    float start_t = 0, mid_t = 0, end_t = 0;
    bool start_set = false, end_set = false, opposite_tangents = false;

    SK_HD bool init(float start, float end) {
        start_t = start;
        mid_t = clamp01((start + end) * 0.5f);
        end_t = end;
        start_set = false;
        end_set = false;
        return start_t < mid_t && mid_t < end_t;
    }
    SK_HD bool init_with_start(const QuadConstruct &parent) {
        if (!init(parent.start_t, parent.mid_t)) return false;
        quad[0] = parent.quad[0];
        tangent_start = parent.tangent_start;
        start_set = true;
        return true;
    }
    SK_HD bool init_with_end(const QuadConstruct &parent) {
        if (!init(parent.mid_t, parent.end_t)) return false;
        quad[2] = parent.quad[2];
        tangent_end = parent.tangent_end;
        end_set = true;
        return true;
    }
};

enum class Join { Miter, MiterClip, Round, Bevel };
enum class Cap { Butt, Round, Square };

// Segments of the input path with auto-close (PathSegmentsIter).
struct Seg {
    uint8_t kind;  // V_*
    Pt p[3];
};

template <class Tr> struct StrokerT {
    using Builder = BuilderT<Tr>;
    float radius = 0, inv_miter_limit = 0, res_scale = 1, inv_res_scale = 1, inv_res_scale_squared = 1;
    Pt first_normal, prev_normal, first_unit_normal, prev_unit_normal;
    Pt first_pt, prev_pt, first_outer_pt;
    size_t first_outer_pt_index_in_contour = 0;
    int segment_count = -1;
    bool prev_is_line = false;
    Cap cap = Cap::Butt;
    Join join = Join::Miter;
    Builder inner, outer, cusper;
    float stroke_type = 1.0f;  // +1 outer, -1 inner
    int recursion_depth = 0;
    bool found_tangents = false, join_completed = false;

    // ---- joiners (the builders may swap for the rest of one join)
    SK_HD void handle_inner_join(Pt pivot, Pt after, Builder &in) {
        in.line_to(pivot.x, pivot.y);
        in.line_to(pivot.x - after.x, pivot.y - after.y);
    }
    SK_HD void bevel_joiner(Pt before_unit, Pt pivot, Pt after_unit, Builder *out, Builder *in) {
        Pt after = scaled(after_unit, radius);
        if (!is_clockwise(before_unit, after_unit)) {
            sk_swap(out, in);
            after = -after;
        }
        out->line_to(pivot.x + after.x, pivot.y + after.y);
        handle_inner_join(pivot, after, *in);
    }
    SK_HD void round_joiner(Pt before_unit, Pt pivot, Pt after_unit, Builder *out, Builder *in) {
        float d = dot(before_unit, after_unit);
        if (dot_to_angle_type(d) == Angle::NearlyLine) return;
        Pt before = before_unit, after = after_unit;
        bool ccw = false;
        if (!is_clockwise(before, after)) {
            sk_swap(out, in);
            before = -before;
            ccw = true;
        }
        Ts ts;
        ts.sx = radius; ts.sy = radius; ts.tx = pivot.x; ts.ty = pivot.y;
        Conic conics[5];
        int n = build_unit_arc(before, after, ccw, ts, conics);
        if (n > 0) {
            for (int i = 0; i < n; i++) out->conic_points_to(conics[i].p[1], conics[i].p[2], conics[i].w);
            after = scaled(after, radius);
            handle_inner_join(pivot, after, *in);
        }
    }
    SK_HD void miter_joiner(Pt before_unit, Pt pivot, Pt after_unit, bool clip, bool prev_line, bool curr_line,
                      Builder *out, Builder *in) {
        auto blunt_or_clipped = [&](Pt before, Pt mid, Pt after, bool curr) {
            after = scaled(after, radius);
            if (clip) {
                normalize(mid);
                float cos_beta = before.x * mid.x + before.y * mid.y;
                float sin_beta = cross(before, mid);
                float x = sk_fabs(sin_beta) <= kNearlyZero ? 1.0f / inv_miter_limit
                                                             : ((1.0f / inv_miter_limit) - cos_beta) / sin_beta;
                before = scaled(before, radius);
                Pt bt = before;
                rotate_cw(bt);
                Pt at = after;
                rotate_ccw(at);
                Pt c1 = pivot + before + scaled(bt, x);
                Pt c2 = pivot + after + scaled(at, x);
                if (prev_line) out->set_last_point(c1);
                else out->line_to(c1.x, c1.y);
                out->line_to(c2.x, c2.y);
            }
            if (!curr) out->line_to(pivot.x + after.x, pivot.y + after.y);
            handle_inner_join(pivot, after, *in);
        };
        auto do_miter = [&](Pt mid, Pt after, bool curr) {
            after = scaled(after, radius);
            if (prev_line) out->set_last_point(P(pivot.x + mid.x, pivot.y + mid.y));
            else out->line_to(pivot.x + mid.x, pivot.y + mid.y);
            if (!curr) out->line_to(pivot.x + after.x, pivot.y + after.y);
            handle_inner_join(pivot, after, *in);
        };
        float d = dot(before_unit, after_unit);
        Angle at = dot_to_angle_type(d);
        Pt before = before_unit, after = after_unit, mid;
        if (at == Angle::NearlyLine) return;
        if (at == Angle::Nearly180) {
            mid = scaled(after - before, radius / 2.0f);
            blunt_or_clipped(before, mid, after, false);
            return;
        }
        bool ccw = !is_clockwise(before, after);
        if (ccw) {
            sk_swap(out, in);
            before = -before;
            after = -after;
        }
        if (d == 0.0f && inv_miter_limit <= kRoot2Over2) {
            mid = scaled(before + after, radius);
            do_miter(mid, after, curr_line);
            return;
        }
        if (at == Angle::Sharp) {
            mid = P(after.y - before.y, before.x - after.x);
            if (ccw) mid = -mid;
        } else {
            mid = P(before.x + after.x, before.y + after.y);
        }
        float sin_half = sk_sqrt((1.0f + d) * 0.5f);
        if (sin_half < inv_miter_limit) {
            blunt_or_clipped(before, mid, after, false);
            return;
        }
        set_length(mid, radius / sin_half);
        do_miter(mid, after, curr_line);
    }
    SK_HD void joiner(Pt before_unit, Pt pivot, Pt after_unit, bool prev_line, bool curr_line, Join j) {
        switch (j) {
        case Join::Bevel: bevel_joiner(before_unit, pivot, after_unit, &outer, &inner); break;
        case Join::Round: round_joiner(before_unit, pivot, after_unit, &outer, &inner); break;
        case Join::Miter: miter_joiner(before_unit, pivot, after_unit, false, prev_line, curr_line, &outer, &inner); break;
        case Join::MiterClip: miter_joiner(before_unit, pivot, after_unit, true, prev_line, curr_line, &outer, &inner); break;
        }
    }

    // ---- cappers
    SK_HD void capper(Pt pivot, Pt normal, Pt stop, bool other_is_line, Builder &path) {
        switch (cap) {
        case Cap::Butt: path.line_to(stop.x, stop.y); break;
        case Cap::Round: {
            Pt parallel = normal;
            rotate_cw(parallel);
            Pt pc = pivot + parallel;
            path.conic_points_to(pc + normal, pc, kRoot2Over2);
            path.conic_points_to(pc - normal, stop, kRoot2Over2);
            break;
        }
        case Cap::Square: {
            Pt parallel = normal;
            rotate_cw(parallel);
            if (other_is_line) {
                path.set_last_point(P(pivot.x + normal.x + parallel.x, pivot.y + normal.y + parallel.y));
                path.line_to(pivot.x - normal.x + parallel.x, pivot.y - normal.y + parallel.y);
            } else {
                path.line_to(pivot.x + normal.x + parallel.x, pivot.y + normal.y + parallel.y);
                path.line_to(pivot.x - normal.x + parallel.x, pivot.y - normal.y + parallel.y);
                path.line_to(stop.x, stop.y);
            }
            break;
        }
        }
    }

    // ---- contour management
    SK_HD void move_to(Pt p) {
        if (segment_count > 0) finish_contour(false, false);
        segment_count = 0;
        first_pt = p;
        prev_pt = p;
        join_completed = false;
    }
    SK_HD void finish_contour(bool close, bool curr_is_line) {
        if (segment_count > 0) {
            if (close) {
                joiner(prev_unit_normal, prev_pt, first_unit_normal, prev_is_line, curr_is_line, join);
                outer.close();
                Pt pt;
                if (!inner.last_point(&pt)) pt = Pt{};
                outer.move_to(pt.x, pt.y);
                outer.reverse_path_to(inner);
                outer.close();
            } else {
                Pt pt;
                if (!inner.last_point(&pt)) pt = Pt{};
                capper(prev_pt, prev_normal, pt, curr_is_line, outer);
                outer.reverse_path_to(inner);
                capper(first_pt, -first_normal, first_outer_pt, prev_is_line, outer);
                outer.close();
            }
            if (!cusper.empty()) {
                outer.push_builder(cusper);
                cusper.clear();
            }
        }
        inner.clear();
        segment_count = -1;
        first_outer_pt_index_in_contour = outer.pts.size();
    }
    SK_HD bool pre_join_to(Pt p, bool curr_is_line, Pt *normal, Pt *unit) {
        float prev_x = prev_pt.x, prev_y = prev_pt.y;
        if (!set_normal_unit_normal(prev_pt, p, res_scale, radius, normal, unit)) {
            if (cap == Cap::Butt) return false;
            *normal = P(radius, 0.0f);
            *unit = P(1.0f, 0.0f);
        }
        if (segment_count == 0) {
            first_normal = *normal;
            first_unit_normal = *unit;
            first_outer_pt = P(prev_x + normal->x, prev_y + normal->y);
            outer.move_to(first_outer_pt.x, first_outer_pt.y);
            inner.move_to(prev_x - normal->x, prev_y - normal->y);
        } else {
            joiner(prev_unit_normal, prev_pt, *unit, prev_is_line, curr_is_line, join);
        }
        prev_is_line = curr_is_line;
        return true;
    }
    SK_HD void post_join_to(Pt p, Pt normal, Pt unit) {
        join_completed = true;
        prev_pt = p;
        prev_unit_normal = unit;
        prev_normal = normal;
        segment_count++;
    }

    // has_valid_tangent of the segment iterator positioned after the current line
    const Seg *segs = nullptr;
    size_t nsegs = 0;
    size_t seg_next = 0;
    SK_HD bool has_valid_tangent() const {
        for (size_t i = seg_next; i < nsegs; i++) {
            const Seg &s = segs[i];
            switch (s.kind) {
            case V_MOVE: return false;
            case V_LINE: continue;  // compared against itself after advancing: always skipped
            case V_QUAD:
                if (s.p[0] == s.p[1]) continue;
                return true;
            case V_CUBIC:
                if (s.p[0] == s.p[2] && s.p[1] == s.p[2]) continue;
                return true;
            default: return false;
            }
        }
        return false;
    }

    SK_HD void line_to(Pt p, bool with_iter) {
        bool teeny = sk_fabs(prev_pt.x - p.x) <= kNearlyZero * inv_res_scale &&
                     sk_fabs(prev_pt.y - p.y) <= kNearlyZero * inv_res_scale;
        if (cap == Cap::Butt && teeny) return;
        if (teeny && (join_completed || (with_iter && has_valid_tangent()))) return;
        Pt normal, unit;
        if (!pre_join_to(p, true, &normal, &unit)) return;
        outer.line_to(p.x + normal.x, p.y + normal.y);
        inner.line_to(p.x - normal.x, p.y - normal.y);
        post_join_to(p, normal, unit);
    }

    SK_HD void set_ray_points(Pt tp, Pt &dxy, Pt *on_p, Pt *tangent) {
        if (!set_length(dxy, radius)) dxy = P(radius, 0.0f);
        float flip = stroke_type;
        on_p->x = tp.x + flip * dxy.y;
        on_p->y = tp.y - flip * dxy.x;
        if (tangent) {
            tangent->x = on_p->x + dxy.x;
            tangent->y = on_p->y + dxy.y;
        }
    }
    SK_HD void quad_perp_ray(const Pt q[3], float t, Pt *t_pt, Pt *on_pt, Pt *tangent) {
        *t_pt = eval_quad_at(q, t);
        Pt dxy = eval_quad_tangent_at(q, t);
        if (dxy.x == 0.0f && dxy.y == 0.0f) dxy = q[2] - q[0];
        set_ray_points(*t_pt, dxy, on_pt, tangent);
    }
    SK_HD void cubic_perp_ray(const Pt c[4], float t, Pt *t_pt, Pt *on_pt, Pt *tangent) {
        *t_pt = eval_cubic_pos_at(c, t);
        Pt dxy = eval_cubic_tangent_at(c, t);
        Pt chopped[7];
        if (dxy.x == 0.0f && dxy.y == 0.0f) {
            const Pt *cp = c;
            if (nearly_zero(t)) {
                dxy = c[2] - c[0];
            } else if (nearly_zero(1.0f - t)) {
                dxy = c[3] - c[1];
            } else {
                chop_cubic_at2(c, t, chopped);
                dxy = chopped[3] - chopped[2];
                if (dxy.x == 0.0f && dxy.y == 0.0f) {
                    dxy = chopped[3] - chopped[1];
                    cp = chopped;
                }
            }
            if (dxy.x == 0.0f && dxy.y == 0.0f) dxy = cp[3] - cp[0];
        }
        set_ray_points(*t_pt, dxy, on_pt, tangent);
    }

    SK_HD Result intersect_ray(RayKind kind, QuadConstruct &qp) {
        Pt start = qp.quad[0], end = qp.quad[2];
        Pt a_len = qp.tangent_start - start;
        Pt b_len = qp.tangent_end - end;
        float denom = cross(a_len, b_len);
        if (denom == 0.0f || !sk_isfinite(denom)) {
            qp.opposite_tangents = dot(a_len, b_len) < 0.0f;
            return Result::Degenerate;
        }
        qp.opposite_tangents = false;
        Pt ab0 = start - end;
        float numer_a = cross(b_len, ab0);
        float numer_b = cross(a_len, ab0);
        if ((numer_a >= 0.0f) == (numer_b >= 0.0f)) {
            float d1 = pt_to_line(start, end, qp.tangent_end);
            float d2 = pt_to_line(end, start, qp.tangent_start);
            if (sk_fmax(d1, d2) <= inv_res_scale_squared) return Result::Degenerate;
            return Result::Split;
        }
        numer_a /= denom;
        bool valid = numer_a > numer_a - 1.0f;
        if (valid) {
            if (kind == RayKind::CtrlPt) {
                qp.quad[1].x = start.x * (1.0f - numer_a) + qp.tangent_start.x * numer_a;
                qp.quad[1].y = start.y * (1.0f - numer_a) + qp.tangent_start.y * numer_a;
            }
            return Result::Quad;
        }
        qp.opposite_tangents = dot(a_len, b_len) < 0.0f;
        return Result::Degenerate;
    }

    SK_HD bool pt_in_quad_bounds(const Pt q[3], Pt pt) {
        float xmin = sk_fmin(sk_fmin(q[0].x, q[1].x), q[2].x);
        if (pt.x + inv_res_scale < xmin) return false;
        float xmax = sk_fmax(sk_fmax(q[0].x, q[1].x), q[2].x);
        if (pt.x - inv_res_scale > xmax) return false;
        float ymin = sk_fmin(sk_fmin(q[0].y, q[1].y), q[2].y);
        if (pt.y + inv_res_scale < ymin) return false;
        float ymax = sk_fmax(sk_fmax(q[0].y, q[1].y), q[2].y);
        if (pt.y - inv_res_scale > ymax) return false;
        return true;
    }

    SK_HD Result stroke_close_enough(const Pt stroke[3], const Pt ray[2], QuadConstruct &qp) {
        Pt mid = eval_quad_at(stroke, 0.5f);
        if (points_within_dist(ray[0], mid, inv_res_scale)) {
            if (sharp_angle(qp.quad)) return Result::Split;
            return Result::Quad;
        }
        if (!pt_in_quad_bounds(stroke, ray[0])) return Result::Split;
        float roots[3];
        int n = intersect_quad_ray(ray, stroke, roots);
        if (n != 1) return Result::Split;
        Pt qpt = eval_quad_at(stroke, roots[0]);
        float error = inv_res_scale * (1.0f - sk_fabs(roots[0] - 0.5f) * 2.0f);
        if (points_within_dist(ray[0], qpt, error)) {
            if (sharp_angle(qp.quad)) return Result::Split;
            return Result::Quad;
        }
        return Result::Split;
    }

    SK_HD Result compare_quad_quad(const Pt q[3], QuadConstruct &qp) {
        if (!qp.start_set) {
            Pt s;
            quad_perp_ray(q, qp.start_t, &s, &qp.quad[0], &qp.tangent_start);
            qp.start_set = true;
        }
        if (!qp.end_set) {
            Pt e;
            quad_perp_ray(q, qp.end_t, &e, &qp.quad[2], &qp.tangent_end);
            qp.end_set = true;
        }
        Result r = intersect_ray(RayKind::CtrlPt, qp);
        if (r != Result::Quad) return r;
        Pt ray[2];
        quad_perp_ray(q, qp.mid_t, &ray[1], &ray[0], nullptr);
        Pt stroke[3] = {qp.quad[0], qp.quad[1], qp.quad[2]};
        return stroke_close_enough(stroke, ray, qp);
    }

    SK_HD void cubic_quad_ends(const Pt c[4], QuadConstruct &qp) {
        if (!qp.start_set) {
            Pt s;
            cubic_perp_ray(c, qp.start_t, &s, &qp.quad[0], &qp.tangent_start);
            qp.start_set = true;
        }
        if (!qp.end_set) {
            Pt e;
            cubic_perp_ray(c, qp.end_t, &e, &qp.quad[2], &qp.tangent_end);
            qp.end_set = true;
        }
    }

    SK_HD Result compare_quad_cubic(const Pt c[4], QuadConstruct &qp) {
        cubic_quad_ends(c, qp);
        Result r = intersect_ray(RayKind::CtrlPt, qp);
        if (r != Result::Quad) return r;
        Pt ray[2];
        cubic_perp_ray(c, qp.mid_t, &ray[1], &ray[0], nullptr);
        Pt stroke[3] = {qp.quad[0], qp.quad[1], qp.quad[2]};
        return stroke_close_enough(stroke, ray, qp);
    }

    SK_HD Builder &cur() { return stroke_type > 0 ? outer : inner; }
    SK_HD void add_degenerate_line(const QuadConstruct &qp) { cur().line_to(qp.quad[2].x, qp.quad[2].y); }

    SK_HD bool cubic_mid_on_line(const Pt c[4], const QuadConstruct &qp) {
        Pt mid, on;
        cubic_perp_ray(c, qp.mid_t, &on, &mid, nullptr);
        float dist = pt_to_line(mid, qp.quad[0], qp.quad[2]);
        return dist < inv_res_scale_squared;
    }

    SK_HD void init_quad(float type, float start, float end, QuadConstruct &qp) {
        stroke_type = type;
        found_tangents = false;
        qp.init(start, end);
    }

    // quad_stroke and cubic_stroke halve a span until its offset is close to a
    // quad: recursive in stroker.rs, here a depth-first walk over an explicit
    // stack that keeps the recursion's order, its `half` objects (the second
    // half reuses the first one's record) and its depth bookkeeping (a failed
    // span leaves recursion_depth raised, as an early return does).
    static constexpr int kMaxFrames = 26 * 3 + 2;
    QuadConstruct frames[kMaxFrames];
    uint8_t stage[kMaxFrames];

    SK_HD bool quad_stroke(const Pt q[3], QuadConstruct &top) {
        int k = 0;
        stage[0] = 0;
        for (;;) {
            QuadConstruct &qp = k == 0 ? top : frames[k];
            bool done = false;
            if (stage[k] == 0) {
                Result r = compare_quad_quad(q, qp);
                if (r == Result::Quad) {
                    cur().quad_to(qp.quad[1].x, qp.quad[1].y, qp.quad[2].x, qp.quad[2].y);
                    done = true;
                } else if (r == Result::Degenerate) {
                    add_degenerate_line(qp);
                    done = true;
                } else {
                    recursion_depth++;
                    if (recursion_depth > recursive_limit(3) || k + 1 >= kMaxFrames) return false;
                    frames[k + 1] = QuadConstruct{};
                    frames[k + 1].init_with_start(qp);
                    stage[k] = 1;
                    stage[++k] = 0;
                    continue;
                }
            } else if (stage[k] == 1) {
                frames[k + 1].init_with_end(qp);
                stage[k] = 2;
                stage[++k] = 0;
                continue;
            } else {
                recursion_depth--;
                done = true;
            }
            if (done) {
                if (k == 0) return true;
                k--;
            }
        }
    }

    SK_HD bool cubic_stroke(const Pt c[4], QuadConstruct &top) {
        int k = 0;
        stage[0] = 0;
        for (;;) {
            QuadConstruct &qp = k == 0 ? top : frames[k];
            bool done = false;
            if (stage[k] == 0) {
                if (!found_tangents) {
                    cubic_quad_ends(c, qp);
                    Result r = intersect_ray(RayKind::ResultType, qp);
                    if (r != Result::Quad) {
                        bool ok = points_within_dist(qp.quad[0], qp.quad[2], inv_res_scale);
                        if ((r == Result::Degenerate || ok) && cubic_mid_on_line(c, qp)) {
                            add_degenerate_line(qp);
                            done = true;
                        }
                    } else {
                        found_tangents = true;
                    }
                }
                if (!done && found_tangents) {
                    Result r = compare_quad_cubic(c, qp);
                    if (r == Result::Quad) {
                        cur().quad_to(qp.quad[1].x, qp.quad[1].y, qp.quad[2].x, qp.quad[2].y);
                        done = true;
                    } else if (r == Result::Degenerate && !qp.opposite_tangents) {
                        add_degenerate_line(qp);
                        done = true;
                    }
                }
                if (!done) {
                    if (!sk_isfinite(qp.quad[2].x) || !sk_isfinite(qp.quad[2].y)) return false;
                    recursion_depth++;
                    if (recursion_depth > recursive_limit(found_tangents ? 1 : 0) || k + 1 >= kMaxFrames) return false;
                    frames[k + 1] = QuadConstruct{};
                    if (!frames[k + 1].init_with_start(qp)) {
                        add_degenerate_line(qp);
                        recursion_depth--;
                        done = true;
                    } else {
                        stage[k] = 1;
                        stage[++k] = 0;
                        continue;
                    }
                }
            } else if (stage[k] == 1) {
                if (!frames[k + 1].init_with_end(qp)) {
                    add_degenerate_line(qp);
                    recursion_depth--;
                    done = true;
                } else {
                    stage[k] = 2;
                    stage[++k] = 0;
                    continue;
                }
            } else {
                recursion_depth--;
                done = true;
            }
            if (done) {
                if (k == 0) return true;
                k--;
            }
        }
    }

    SK_HD void quad_to(Pt p1, Pt p2) {
        Pt q[3] = {prev_pt, p1, p2};
        Pt reduction;
        Reduction rt = check_quad_linear(q, &reduction);
        if (rt == Reduction::Point || rt == Reduction::Line) {
            line_to(p2, false);
            return;
        }
        if (rt == Reduction::Degenerate) {
            line_to(reduction, false);
            Join save = join;
            join = Join::Round;
            line_to(p2, false);
            join = save;
            return;
        }
        Pt normal_ab, unit_ab, normal_bc, unit_bc;
        if (!pre_join_to(p1, false, &normal_ab, &unit_ab)) {
            line_to(p2, false);
            return;
        }
        QuadConstruct qp;
        init_quad(1.0f, 0.0f, 1.0f, qp);
        quad_stroke(q, qp);
        init_quad(-1.0f, 0.0f, 1.0f, qp);
        quad_stroke(q, qp);
        set_normal_unit_normal(q[1], q[2], res_scale, radius, &normal_bc, &unit_bc);
        post_join_to(p2, normal_bc, unit_bc);
    }

    SK_HD void set_cubic_end_normal(const Pt c[4], Pt normal_ab, Pt unit_ab, Pt *normal_cd, Pt *unit_cd) {
        Pt ab = c[1] - c[0], cd = c[3] - c[2];
        bool dab = degenerate_vector(ab), dcb = degenerate_vector(cd);
        if (dab && dcb) {
            *normal_cd = normal_ab;
            *unit_cd = unit_ab;
            return;
        }
        if (dab) {
            ab = c[2] - c[0];
            dab = degenerate_vector(ab);
        }
        if (dcb) {
            cd = c[3] - c[1];
            dcb = degenerate_vector(cd);
        }
        if (dab || dcb) {
            *normal_cd = normal_ab;
            *unit_cd = unit_ab;
            return;
        }
        set_normal_unit_normal2(cd, radius, normal_cd, unit_cd);
    }

    SK_HD void cubic_to(Pt p1, Pt p2, Pt p3) {
        Pt c[4] = {prev_pt, p1, p2, p3};
        Pt reduction[3];
        Pt tangent_pt;
        Reduction rt = check_cubic_linear(c, reduction, &tangent_pt);
        if (rt == Reduction::Point || rt == Reduction::Line) {
            line_to(p3, false);
            return;
        }
        if (rt == Reduction::Degenerate || rt == Reduction::Degenerate2 || rt == Reduction::Degenerate3) {
            line_to(reduction[0], false);
            Join save = join;
            join = Join::Round;
            if (rt == Reduction::Degenerate2 || rt == Reduction::Degenerate3) line_to(reduction[1], false);
            if (rt == Reduction::Degenerate3) line_to(reduction[2], false);
            line_to(p3, false);
            join = save;
            return;
        }
        Pt normal_ab, unit_ab, normal_cd, unit_cd;
        if (!pre_join_to(tangent_pt, false, &normal_ab, &unit_ab)) {
            line_to(p3, false);
            return;
        }
        float tv[3];
        int n = find_cubic_inflections(c, tv);
        float last_t = 0.0f;
        for (int i = 0; i <= n; i++) {
            float next_t = i < n ? tv[i] : 1.0f;
            QuadConstruct qp;
            init_quad(1.0f, last_t, next_t, qp);
            cubic_stroke(c, qp);
            init_quad(-1.0f, last_t, next_t, qp);
            cubic_stroke(c, qp);
            last_t = next_t;
        }
        float cusp;
        if (find_cubic_cusp(c, &cusp)) {
            Pt loc = eval_cubic_pos_at(c, cusp);
            cusper.push_circle(loc.x, loc.y, radius);
        }
        set_cubic_end_normal(c, normal_ab, unit_ab, &normal_cd, &unit_cd);
        post_join_to(p3, normal_cd, unit_cd);
    }

    SK_HD bool current_contour_empty() const {
        return inner.zero_length_since_point(0) && outer.zero_length_since_point(first_outer_pt_index_in_contour);
    }
};

struct StrokeParams {
    float width = 1.0f;
    float miter_limit = 4.0f;
    uint32_t cap = 0;   // rgpu_cap
    uint32_t join = 0;  // rgpu_join
    float res_scale = 1.0f;
};

// PathSegmentsIter with auto-close: a close whose last point differs from the
// contour start first yields the closing line.  `segs` holds at least
// 2 * nv entries; returns the count, or -1 for a verb that is not a path verb.
SK_HD inline long build_segments(const uint8_t *verbs, size_t nv, const float *pts, Seg *segs) {
    long n = 0;
    size_t pi = 0;
    Pt last_move, last_pt;
    for (size_t i = 0; i < nv; i++) {
        Seg s{};
        s.kind = verbs[i];
        switch (verbs[i]) {
        case V_MOVE:
            last_move = last_pt = P(pts[2 * pi], pts[2 * pi + 1]);
            pi += 1;
            s.p[0] = last_move;
            segs[n++] = s;
            break;
        case V_LINE:
            last_pt = P(pts[2 * pi], pts[2 * pi + 1]);
            pi += 1;
            s.p[0] = last_pt;
            segs[n++] = s;
            break;
        case V_QUAD:
            s.p[0] = P(pts[2 * pi], pts[2 * pi + 1]);
            s.p[1] = P(pts[2 * pi + 2], pts[2 * pi + 3]);
            pi += 2;
            last_pt = s.p[1];
            segs[n++] = s;
            break;
        case V_CUBIC:
            s.p[0] = P(pts[2 * pi], pts[2 * pi + 1]);
            s.p[1] = P(pts[2 * pi + 2], pts[2 * pi + 3]);
            s.p[2] = P(pts[2 * pi + 4], pts[2 * pi + 5]);
            pi += 3;
            last_pt = s.p[2];
            segs[n++] = s;
            break;
        case V_CLOSE:
            if (last_pt != last_move) {
                Seg l{};
                l.kind = V_LINE;
                l.p[0] = last_move;
                segs[n++] = l;
            }
            last_pt = last_move;
            segs[n++] = s;
            break;
        default: return -1;
        }
    }
    return n;
}

// Path::stroke over prepared segments into sk.outer (whose storage, like the
// inner and cusp builders', the caller has set up).  False when nothing is
// produced.
template <class Tr>
SK_HD inline bool stroke_segments(StrokerT<Tr> &sk, const Seg *segs, size_t nsegs, const StrokeParams &st) {
    if (!(st.width > 0.0f) || !sk_isfinite(st.width)) return false;
    Join join = st.join == 1 ? Join::MiterClip : st.join == 2 ? Join::Round : st.join == 3 ? Join::Bevel : Join::Miter;
    float inv_miter = 0.0f;
    if (join == Join::Miter) {
        if (st.miter_limit <= 1.0f) join = Join::Bevel;
        else inv_miter = 1.0f / st.miter_limit;
    }
    if (join == Join::MiterClip) inv_miter = 1.0f / st.miter_limit;
    sk.res_scale = st.res_scale;
    sk.inv_res_scale = 1.0f / (st.res_scale * 4.0f);
    sk.inv_res_scale_squared = sk.inv_res_scale * sk.inv_res_scale;
    sk.radius = st.width * 0.5f;
    sk.inv_miter_limit = inv_miter;
    sk.cap = st.cap == 1 ? Cap::Round : st.cap == 2 ? Cap::Square : Cap::Butt;
    sk.join = join;
    sk.segs = segs;
    sk.nsegs = nsegs;
    bool last_is_line = false;
    for (size_t i = 0; i < nsegs; i++) {
        const Seg &s = segs[i];
        sk.seg_next = i + 1;
        switch (s.kind) {
        case V_MOVE: sk.move_to(s.p[0]); break;
        case V_LINE:
            sk.line_to(s.p[0], true);
            last_is_line = true;
            break;
        case V_QUAD:
            sk.quad_to(s.p[0], s.p[1]);
            last_is_line = false;
            break;
        case V_CUBIC:
            sk.cubic_to(s.p[0], s.p[1], s.p[2]);
            last_is_line = false;
            break;
        case V_CLOSE:
            if (sk.cap != Cap::Butt) {
                if (sk.segment_count == 0) {
                    sk.line_to(sk.first_pt, false);
                    last_is_line = true;
                    continue;
                }
                if (sk.current_contour_empty()) {
                    last_is_line = true;
                    continue;
                }
            }
            sk.finish_contour(true, last_is_line);
            break;
        }
    }
    sk.finish_contour(false, last_is_line);
    return sk.outer.verbs.size() > 1;
}

}  // namespace sk
}  // namespace rgpu
