// Device edge builder: per path segment, the fixed-point edges Skia's edge
// builder produces (tiny-skia 0.12.0 edge.rs / edge_builder.rs / edge_clipper.rs /
// path_geometry.rs).  Each thread owns one segment and runs the same f32/f64
// and 16.16 fixed-point arithmetic serially; curve edges are expanded into their
// forward-differenced line pieces up front instead of lazily inside the scan
// loop, which yields the identical sequence of line edges.
#pragma once
#include <stdint.h>
#include "../device_types.h"

namespace rgpu {
namespace dev {

struct Pt { float x, y; };

__device__ __forceinline__ int32_t sat_i32(float v) {
    if (isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
__device__ __forceinline__ bool valid_unit_divide(float numer, float denom, float *ratio) {
    if (numer < 0) { numer = -numer; denom = -denom; }
    if (denom == 0 || numer == 0 || numer >= denom) return false;
    float r = __fdiv_rn(numer, denom);
    if (isnan(r)) return false;
    if (r == 0) return false;
    *ratio = r;
    return true;
}
__device__ __forceinline__ int find_unit_quad_roots(float a, float b, float c, float roots[2]) {
    if (a == 0) return valid_unit_divide(-c, b, &roots[0]) ? 1 : 0;
    double dr = __dsub_rn(__dmul_rn((double)b, (double)b), __dmul_rn(__dmul_rn(4.0, (double)a), (double)c));
    if (dr < 0) return 0;
    dr = __dsqrt_rn(dr);
    float r = (float)dr;
    if (isinf(r) || isnan(r)) return 0;
    float q = (b < 0) ? __fdiv_rn(-(b - r), 2.0f) : __fdiv_rn(-(b + r), 2.0f);
    int n = 0;
    if (valid_unit_divide(q, a, &roots[n])) n++;
    if (valid_unit_divide(c, q, &roots[n])) n++;
    if (n == 2) {
        if (roots[0] > roots[1]) { float t = roots[0]; roots[0] = roots[1]; roots[1] = t; }
        else if (roots[0] == roots[1]) n--;
    }
    return n;
}
__device__ __forceinline__ Pt interp(Pt a, Pt b, float t) {
    return Pt{__fadd_rn(a.x, __fmul_rn(__fsub_rn(b.x, a.x), t)), __fadd_rn(a.y, __fmul_rn(__fsub_rn(b.y, a.y), t))};
}
__device__ __forceinline__ void chop_cubic_at2(const Pt *src, float t, Pt *dst) {
    Pt ab = interp(src[0], src[1], t), bc = interp(src[1], src[2], t), cd = interp(src[2], src[3], t);
    Pt abc = interp(ab, bc, t), bcd = interp(bc, cd, t), abcd = interp(abc, bcd, t);
    dst[0] = src[0]; dst[1] = ab; dst[2] = abc; dst[3] = abcd; dst[4] = bcd; dst[5] = cd; dst[6] = src[3];
}
__device__ __forceinline__ void chop_cubic_at(const Pt *src, const float *ts, int n, Pt *dst) {
    if (n == 0) { for (int i = 0; i < 4; i++) dst[i] = src[i]; return; }
    float t = ts[0];
    Pt tmp[4];
    Pt cur[4] = {src[0], src[1], src[2], src[3]};
    int off = 0;
    for (int i = 0; i < n; i++) {
        chop_cubic_at2(cur, t, dst + off);
        if (i == n - 1) break;
        off += 3;
        for (int k = 0; k < 4; k++) tmp[k] = dst[off + k];
        for (int k = 0; k < 4; k++) cur[k] = tmp[k];
        float nt;
        if (!valid_unit_divide(ts[i + 1] - ts[i], 1.0f - ts[i], &nt)) {
            dst[off + 4] = cur[3]; dst[off + 5] = cur[3]; dst[off + 6] = cur[3];
            break;
        }
        t = nt;
    }
}
__device__ __forceinline__ int find_cubic_extrema(float a, float b, float c, float d, float ts[2]) {
    float A = d - a + 3.0f * (b - c);
    float B = 2.0f * (a - b - b + c);
    float C = b - a;
    return find_unit_quad_roots(A, B, C, ts);
}
__device__ __forceinline__ int chop_cubic_at_y_extrema(const Pt *src, Pt *dst) {
    float ts[2];
    int n = find_cubic_extrema(src[0].y, src[1].y, src[2].y, src[3].y, ts);
    chop_cubic_at(src, ts, n, dst);
    if (n > 0) {
        dst[2].y = dst[3].y; dst[4].y = dst[3].y;
        if (n == 2) { dst[5].y = dst[6].y; dst[7].y = dst[6].y; }
    }
    return n;
}
__device__ __forceinline__ int chop_cubic_at_x_extrema(const Pt *src, Pt *dst) {
    float ts[2];
    int n = find_cubic_extrema(src[0].x, src[1].x, src[2].x, src[3].x, ts);
    chop_cubic_at(src, ts, n, dst);
    if (n > 0) {
        dst[2].x = dst[3].x; dst[4].x = dst[3].x;
        if (n == 2) { dst[5].x = dst[6].x; dst[7].x = dst[6].x; }
    }
    return n;
}
__device__ __forceinline__ void chop_quad_at(const Pt *src, float t, Pt *dst) {
    Pt p01 = interp(src[0], src[1], t), p12 = interp(src[1], src[2], t);
    dst[0] = src[0]; dst[1] = p01; dst[2] = interp(p01, p12, t); dst[3] = p12; dst[4] = src[2];
}
__device__ __forceinline__ bool is_not_monotonic(float a, float b, float c) {
    float ab = a - b, bc = b - c;
    if (ab < 0) bc = -bc;
    return ab == 0 || bc < 0;
}
__device__ __forceinline__ int chop_quad_at_y_extrema(const Pt *src, Pt *dst) {
    float a = src[0].y, b = src[1].y, c = src[2].y;
    if (is_not_monotonic(a, b, c)) {
        float t;
        if (valid_unit_divide(a - b, a - b - b + c, &t)) {
            chop_quad_at(src, t, dst);
            dst[1].y = dst[2].y; dst[3].y = dst[2].y;
            return 1;
        }
        b = (fabsf(a - b) < fabsf(b - c)) ? a : c;
    }
    dst[0] = Pt{src[0].x, a}; dst[1] = Pt{src[1].x, b}; dst[2] = Pt{src[2].x, c};
    return 0;
}
__device__ __forceinline__ int chop_quad_at_x_extrema(const Pt *src, Pt *dst) {
    float a = src[0].x, b = src[1].x, c = src[2].x;
    if (is_not_monotonic(a, b, c)) {
        float t;
        if (valid_unit_divide(a - b, a - b - b + c, &t)) {
            chop_quad_at(src, t, dst);
            dst[1].x = dst[2].x; dst[3].x = dst[2].x;
            return 1;
        }
        b = (fabsf(a - b) < fabsf(b - c)) ? a : c;
    }
    dst[0] = Pt{a, src[0].y}; dst[1] = Pt{b, src[1].y}; dst[2] = Pt{c, src[2].y};
    return 0;
}

// ---- fixed point
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t lsh(int32_t v, int s) { return (int32_t)((uint32_t)v << s); }
__device__ __forceinline__ int32_t fdot6_round(int32_t n) { return (n + 32) >> 6; }
__device__ __forceinline__ int32_t fdot6_to_fdot16(int32_t v) { return lsh(v, 10); }
__device__ __forceinline__ int32_t fdot16_mul(int32_t a, int32_t b) { return (int32_t)(((int64_t)a * (int64_t)b) >> 16); }
__device__ __forceinline__ int32_t fdot6_div(int32_t a, int32_t b) {
    if (a >= -32768 && a <= 32767) return lsh(a, 16) / b;
    int64_t v = ((int64_t)a * 65536) / (int64_t)b;
    if (v < INT32_MIN) v = INT32_MIN;
    if (v > INT32_MAX) v = INT32_MAX;
    return (int32_t)v;
}
__device__ __forceinline__ int32_t compute_dy(int32_t top, int32_t y0) { return lsh(top, 6) + 32 - y0; }

struct LineE { int32_t x, dx, first_y, last_y; };

__device__ __forceinline__ bool line_update(LineE &e, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
    y0 >>= 10; y1 >>= 10;
    int32_t top = fdot6_round(y0), bot = fdot6_round(y1);
    if (top == bot) return false;
    x0 >>= 10; x1 >>= 10;
    int32_t slope = fdot6_div(x1 - x0, y1 - y0);
    int32_t dy = compute_dy(top, y0);
    e.x = fdot6_to_fdot16(x0 + fdot16_mul(slope, dy));
    e.dx = slope;
    e.first_y = top;
    e.last_y = bot - 1;
    return true;
}
__device__ __forceinline__ int32_t cheap_distance(int32_t dx, int32_t dy) {
    dx = abs(dx); dy = abs(dy);
    return dx > dy ? dx + (dy >> 1) : dy + (dx >> 1);
}
__device__ __forceinline__ int diff_to_shift(int32_t dx, int32_t dy, int shift_aa) {
    int32_t dist = cheap_distance(dx, dy);
    dist = (dist + (1 << 4)) >> (3 + shift_aa);
    return (32 - __clz(dist)) >> 1;
}
__device__ __forceinline__ int32_t cubic_delta_from_line(int32_t a, int32_t b, int32_t c, int32_t d) {
    int32_t one_third = ((a * 8 - b * 15 + 6 * c + d) * 19) >> 9;
    int32_t two_third = ((a + 6 * b - c * 15 + d * 8) * 19) >> 9;
    return max(abs(one_third), abs(two_third));
}

// Sink receiving the line edges of one segment (counting or writing).
struct EdgeSink {
    EdgeRec *out;    // null: count only
    uint32_t n;
    uint32_t cap;
    __device__ __forceinline__ void put(const LineE &e, int winding) {
        if (out && n < cap) {
            EdgeRec r;
            r.x = e.x; r.dx = e.dx; r.first_y = e.first_y;
            r.hw = ((e.last_y - e.first_y) << 8) | (winding & 0xff);
            out[n] = r;
        }
        n++;
    }
};

__device__ __forceinline__ void push_line(EdgeSink &s, Pt p0, Pt p1, int shift) {
    float scale = (float)(1 << (shift + 6));
    int32_t x0 = sat_i32(p0.x * scale), y0 = sat_i32(p0.y * scale);
    int32_t x1 = sat_i32(p1.x * scale), y1 = sat_i32(p1.y * scale);
    int w = 1;
    if (y0 > y1) { int32_t t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; w = -1; }
    int32_t top = fdot6_round(y0), bottom = fdot6_round(y1);
    if (top == bottom) return;
    int32_t slope = fdot6_div(x1 - x0, y1 - y0);
    int32_t dy = compute_dy(top, y0);
    LineE e;
    e.x = fdot6_to_fdot16(x0 + fdot16_mul(slope, dy));
    e.dx = slope;
    e.first_y = top;
    e.last_y = bottom - 1;
    s.put(e, w);
}

__device__ __noinline__ void push_quad(EdgeSink &s, const Pt *pts, int shift) {
    float scale = (float)(1 << (shift + 6));
    int32_t x0 = sat_i32(pts[0].x * scale), y0 = sat_i32(pts[0].y * scale);
    int32_t x1 = sat_i32(pts[1].x * scale), y1 = sat_i32(pts[1].y * scale);
    int32_t x2 = sat_i32(pts[2].x * scale), y2 = sat_i32(pts[2].y * scale);
    int w = 1;
    if (y0 > y2) { int32_t t = x0; x0 = x2; x2 = t; t = y0; y0 = y2; y2 = t; w = -1; }
    int32_t top = fdot6_round(y0), bot = fdot6_round(y2);
    if (top == bot) return;
    {
        int32_t dx = (lsh(x1, 1) - x0 - x2) >> 2;
        int32_t dy = (lsh(y1, 1) - y0 - y2) >> 2;
        shift = diff_to_shift(dx, dy, shift);
    }
    if (shift == 0) shift = 1;
    else if (shift > 6) shift = 6;
    int count = 1 << shift;
    int cshift = shift - 1;
    int32_t A = lsh(x0 - x1 - x1 + x2, 9);
    int32_t B = fdot6_to_fdot16(x1 - x0);
    int32_t qx = fdot6_to_fdot16(x0), qdx = B + (A >> shift), qddx = A >> (shift - 1);
    A = lsh(y0 - y1 - y1 + y2, 9);
    B = fdot6_to_fdot16(y1 - y0);
    int32_t qy = fdot6_to_fdot16(y0), qdy = B + (A >> shift), qddy = A >> (shift - 1);
    int32_t lastx = fdot6_to_fdot16(x2), lasty = fdot6_to_fdot16(y2);
    int32_t oldx = qx, oldy = qy;
    // expand every forward-difference step; zero-height pieces are skipped as
    // the lazy updater would skip them
    while (count > 0) {
        int32_t newx, newy;
        count--;
        if (count > 0) {
            newx = oldx + (qdx >> cshift); qdx += qddx;
            newy = oldy + (qdy >> cshift); qdy += qddy;
        } else {
            newx = lastx; newy = lasty;
        }
        LineE e;
        if (line_update(e, oldx, oldy, newx, newy)) s.put(e, w);
        oldx = newx; oldy = newy;
    }
}

__device__ __noinline__ void push_cubic(EdgeSink &s, const Pt *pts, int shift) {
    float scale = (float)(1 << (shift + 6));
    int32_t x0 = sat_i32(pts[0].x * scale), y0 = sat_i32(pts[0].y * scale);
    int32_t x1 = sat_i32(pts[1].x * scale), y1 = sat_i32(pts[1].y * scale);
    int32_t x2 = sat_i32(pts[2].x * scale), y2 = sat_i32(pts[2].y * scale);
    int32_t x3 = sat_i32(pts[3].x * scale), y3 = sat_i32(pts[3].y * scale);
    int w = 1;
    if (y0 > y3) {
        int32_t t;
        t = x0; x0 = x3; x3 = t; t = x1; x1 = x2; x2 = t;
        t = y0; y0 = y3; y3 = t; t = y1; y1 = y2; y2 = t;
        w = -1;
    }
    int32_t top = fdot6_round(y0), bot = fdot6_round(y3);
    if (top == bot) return;
    {
        int32_t dx = cubic_delta_from_line(x0, x1, x2, x3);
        int32_t dy = cubic_delta_from_line(y0, y1, y2, y3);
        shift = diff_to_shift(dx, dy, 2) + 1;
    }
    if (shift > 6) shift = 6;
    int up_shift = 6;
    int down_shift = shift + up_shift - 10;
    if (down_shift < 0) { down_shift = 0; up_shift = 10 - shift; }
    int32_t B = lsh(3 * (x1 - x0), up_shift);
    int32_t C = lsh(3 * (x0 - x1 - x1 + x2), up_shift);
    int32_t D = lsh(x3 + 3 * (x1 - x2) - x0, up_shift);
    int32_t cx = fdot6_to_fdot16(x0);
    int32_t cdx = B + (C >> shift) + (D >> (2 * shift));
    int32_t cddx = 2 * C + ((3 * D) >> (shift - 1));
    int32_t cdddx = (3 * D) >> (shift - 1);
    B = lsh(3 * (y1 - y0), up_shift);
    C = lsh(3 * (y0 - y1 - y1 + y2), up_shift);
    D = lsh(y3 + 3 * (y1 - y2) - y0, up_shift);
    int32_t cy = fdot6_to_fdot16(y0);
    int32_t cdy = B + (C >> shift) + (D >> (2 * shift));
    int32_t cddy = 2 * C + ((3 * D) >> (shift - 1));
    int32_t cdddy = (3 * D) >> (shift - 1);
    int32_t lastx = fdot6_to_fdot16(x3), lasty = fdot6_to_fdot16(y3);
    int count = -(1 << shift);
    int32_t oldx = cx, oldy = cy;
    while (count < 0) {
        int32_t newx, newy;
        count++;
        if (count < 0) {
            newx = oldx + (cdx >> down_shift); cdx += cddx >> shift; cddx += cdddx;
            newy = oldy + (cdy >> down_shift); cdy += cddy >> shift; cddy += cdddy;
        } else {
            newx = lastx; newy = lasty;
        }
        if (newy < oldy) newy = oldy;
        LineE e;
        if (line_update(e, oldx, oldy, newx, newy)) s.put(e, w);
        oldx = newx; oldy = newy;
    }
}

// ---- edge clipper (edge_clipper.rs / line_clipper.rs)
struct ClipR { float l, t, r, b; };

__device__ __forceinline__ float pin_unsorted(double v, double a, double b) {
    if (a > b) { double t = a; a = b; b = t; }
    if (v < a) v = a;
    if (v > b) v = b;
    return (float)v;
}
__device__ __forceinline__ float sect_with_horizontal(const Pt *src, float Y) {
    float dy = src[1].y - src[0].y;
    if (fabsf(dy) <= (1.0f / 4096.0f)) return __fmul_rn(__fadd_rn(src[0].x, src[1].x), 0.5f);
    double X0 = src[0].x, Y0 = src[0].y, X1 = src[1].x, Y1 = src[1].y;
    double r = __dadd_rn(X0, __ddiv_rn(__dmul_rn(__dsub_rn((double)Y, Y0), __dsub_rn(X1, X0)), __dsub_rn(Y1, Y0)));
    return pin_unsorted(r, X0, X1);
}
__device__ __forceinline__ float sect_with_vertical(const Pt *src, float X) {
    float dx = src[1].x - src[0].x;
    if (fabsf(dx) <= (1.0f / 4096.0f)) return __fmul_rn(__fadd_rn(src[0].y, src[1].y), 0.5f);
    double X0 = src[0].x, Y0 = src[0].y, X1 = src[1].x, Y1 = src[1].y;
    return (float)__dadd_rn(Y0, __ddiv_rn(__dmul_rn(__dsub_rn((double)X, X0), __dsub_rn(Y1, Y0)), __dsub_rn(X1, X0)));
}
__device__ __forceinline__ float sect_clamp_with_vertical(const Pt *src, float x) {
    float y = sect_with_vertical(src, x);
    float a = src[0].y, b = src[1].y;
    if (a > b) { float t = a; a = b; b = t; }
    return fminf(fmaxf(y, a), b);
}
__device__ __noinline__ void clip_line(EdgeSink &s, Pt p0, Pt p1, const ClipR &clip, int shift) {
    Pt pts[2] = {p0, p1};
    int i0, i1;
    if (pts[0].y < pts[1].y) { i0 = 0; i1 = 1; } else { i0 = 1; i1 = 0; }
    if (pts[i1].y <= clip.t) return;
    if (pts[i0].y >= clip.b) return;
    Pt tmp[2] = {pts[0], pts[1]};
    if (pts[i0].y < clip.t) tmp[i0] = Pt{sect_with_horizontal(pts, clip.t), clip.t};
    if (tmp[i1].y > clip.b) tmp[i1] = Pt{sect_with_horizontal(pts, clip.b), clip.b};
    Pt res[4];
    int n = 1;
    bool reverse;
    if (pts[0].x < pts[1].x) { i0 = 0; i1 = 1; reverse = false; } else { i0 = 1; i1 = 0; reverse = true; }
    if (tmp[i1].x <= clip.l) {
        tmp[0].x = tmp[1].x = clip.l;
        res[0] = tmp[0]; res[1] = tmp[1];
        reverse = false;
    } else if (tmp[i0].x >= clip.r) {
        tmp[0].x = tmp[1].x = clip.r;
        res[0] = tmp[0]; res[1] = tmp[1];
        reverse = false;
    } else {
        int k = 0;
        if (tmp[i0].x < clip.l) {
            res[k++] = Pt{clip.l, tmp[i0].y};
            res[k] = Pt{clip.l, sect_clamp_with_vertical(tmp, clip.l)};
        } else {
            res[k] = tmp[i0];
        }
        k++;
        if (tmp[i1].x > clip.r) {
            res[k++] = Pt{clip.r, sect_clamp_with_vertical(tmp, clip.r)};
            res[k] = Pt{clip.r, tmp[i1].y};
        } else {
            res[k] = tmp[i1];
        }
        n = k;
    }
    if (reverse) {
        for (int i = n - 1; i >= 0; i--) push_line(s, res[i + 1], res[i], shift);
        // emitted in the reversed point order: lines[n-i] = res[i]
    } else {
        for (int i = 0; i < n; i++) push_line(s, res[i], res[i + 1], shift);
    }
}
__device__ __forceinline__ void append_vline(EdgeSink &s, float x, float y0, float y1, bool reverse, int shift) {
    if (reverse) { float t = y0; y0 = y1; y1 = t; }
    push_line(s, Pt{x, y0}, Pt{x, y1}, shift);
}
__device__ __forceinline__ bool chop_mono_quad_at(const Pt *src, float v, bool is_y, float *t) {
    float c0 = is_y ? src[0].y : src[0].x, c1 = is_y ? src[1].y : src[1].x, c2 = is_y ? src[2].y : src[2].x;
    float a = c0 - c1 - c1 + c2, b = 2.0f * (c1 - c0), c = c0 - v;
    float roots[2];
    int n = find_unit_quad_roots(a, b, c, roots);
    if (n) { *t = roots[0]; return true; }
    return false;
}
__device__ __noinline__ void clip_mono_quad(EdgeSink &s, const Pt *src, const ClipR &clip, int shift) {
    Pt pts[3];
    bool reverse;
    if (src[0].y > src[2].y) { pts[0] = src[2]; pts[1] = src[1]; pts[2] = src[0]; reverse = true; }
    else { pts[0] = src[0]; pts[1] = src[1]; pts[2] = src[2]; reverse = false; }
    if (pts[2].y <= clip.t || pts[0].y >= clip.b) return;
    float t;
    Pt tmp[5];
    if (pts[0].y < clip.t) {
        if (chop_mono_quad_at(pts, clip.t, true, &t)) {
            chop_quad_at(pts, t, tmp);
            tmp[2].y = clip.t;
            tmp[3].y = fmaxf(tmp[3].y, clip.t);
            pts[0] = tmp[2]; pts[1] = tmp[3];
        } else {
            for (int i = 0; i < 3; i++) if (pts[i].y < clip.t) pts[i].y = clip.t;
        }
    }
    if (pts[2].y > clip.b) {
        if (chop_mono_quad_at(pts, clip.b, true, &t)) {
            chop_quad_at(pts, t, tmp);
            tmp[1].y = fminf(tmp[1].y, clip.b);
            tmp[2].y = clip.b;
            pts[1] = tmp[1]; pts[2] = tmp[2];
        } else {
            for (int i = 0; i < 3; i++) if (pts[i].y > clip.b) pts[i].y = clip.b;
        }
    }
    if (pts[0].x > pts[2].x) { Pt q = pts[0]; pts[0] = pts[2]; pts[2] = q; reverse = !reverse; }
    if (pts[2].x <= clip.l) { append_vline(s, clip.l, pts[0].y, pts[2].y, reverse, shift); return; }
    if (pts[0].x >= clip.r) { append_vline(s, clip.r, pts[0].y, pts[2].y, reverse, shift); return; }
    if (pts[0].x < clip.l) {
        if (chop_mono_quad_at(pts, clip.l, false, &t)) {
            chop_quad_at(pts, t, tmp);
            append_vline(s, clip.l, tmp[0].y, tmp[2].y, reverse, shift);
            tmp[2].x = clip.l;
            tmp[3].x = fmaxf(tmp[3].x, clip.l);
            pts[0] = tmp[2]; pts[1] = tmp[3];
        } else {
            append_vline(s, clip.l, pts[0].y, pts[2].y, reverse, shift);
            return;
        }
    }
    Pt q[3];
    if (pts[2].x > clip.r) {
        if (chop_mono_quad_at(pts, clip.r, false, &t)) {
            chop_quad_at(pts, t, tmp);
            tmp[1].x = fminf(tmp[1].x, clip.r);
            tmp[2].x = clip.r;
            if (reverse) { q[0] = tmp[2]; q[1] = tmp[1]; q[2] = tmp[0]; } else { q[0] = tmp[0]; q[1] = tmp[1]; q[2] = tmp[2]; }
            push_quad(s, q, shift);
            append_vline(s, clip.r, tmp[2].y, tmp[4].y, reverse, shift);
        } else {
            pts[1].x = fminf(pts[1].x, clip.r);
            pts[2].x = fminf(pts[2].x, clip.r);
            if (reverse) { q[0] = pts[2]; q[1] = pts[1]; q[2] = pts[0]; } else { q[0] = pts[0]; q[1] = pts[1]; q[2] = pts[2]; }
            push_quad(s, q, shift);
        }
    } else {
        if (reverse) { q[0] = pts[2]; q[1] = pts[1]; q[2] = pts[0]; } else { q[0] = pts[0]; q[1] = pts[1]; q[2] = pts[2]; }
        push_quad(s, q, shift);
    }
}
__device__ __noinline__ void clip_quad(EdgeSink &s, const Pt *p, const ClipR &clip, int shift) {
    float t = fminf(fminf(p[0].y, p[1].y), p[2].y), b = fmaxf(fmaxf(p[0].y, p[1].y), p[2].y);
    if (!(b > clip.t && t < clip.b)) return;
    Pt mono_y[5];
    int ny = chop_quad_at_y_extrema(p, mono_y);
    for (int y = 0; y <= ny; y++) {
        Pt mono_x[5];
        int nx = chop_quad_at_x_extrema(&mono_y[y * 2], mono_x);
        for (int x = 0; x <= nx; x++) clip_mono_quad(s, &mono_x[x * 2], clip, shift);
    }
}
// root of a monotonic cubic coordinate in double (bisection to convergence)
__device__ __forceinline__ bool mono_cubic_root(const Pt *src, float v, bool is_y, double *t_out) {
    double c[4];
    for (int i = 0; i < 4; i++) c[i] = is_y ? src[i].y : src[i].x;
    double A = __dsub_rn(__dadd_rn(c[3], __dmul_rn(3.0, __dsub_rn(c[1], c[2]))), c[0]);
    double B = __dmul_rn(3.0, __dadd_rn(__dsub_rn(c[2], __dmul_rn(2.0, c[1])), c[0]));
    double C = __dmul_rn(3.0, __dsub_rn(c[1], c[0]));
    double D = __dsub_rn(c[0], (double)v);
    auto f = [&](double t) {
        return __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(A, t), B), t), C), t), D);
    };
    double f0 = f(0.0), f1 = f(1.0);
    if (f0 == 0.0) { *t_out = 0.0; return true; }
    if (f1 == 0.0) { *t_out = 1.0; return true; }
    if ((f0 < 0) == (f1 < 0)) return false;
    double lo = 0.0, hi = 1.0;
    bool inc = f0 < 0;
    for (int it = 0; it < 100; it++) {
        double mid = __dmul_rn(0.5, __dadd_rn(lo, hi));
        if (mid <= lo || mid >= hi) break;
        double fm = f(mid);
        if (fm == 0.0) { lo = hi = mid; break; }
        if ((fm < 0) == inc) lo = mid; else hi = mid;
    }
    *t_out = __dmul_rn(0.5, __dadd_rn(lo, hi));
    return true;
}
__device__ __forceinline__ void chop_cubic_at_d(const Pt *src, double t, Pt *dst) {
    double x[4], y[4];
    for (int i = 0; i < 4; i++) { x[i] = src[i].x; y[i] = src[i].y; }
    auto lerp = [](double a, double b, double t) { return __dadd_rn(a, __dmul_rn(__dsub_rn(b, a), t)); };
    double abx = lerp(x[0], x[1], t), aby = lerp(y[0], y[1], t);
    double bcx = lerp(x[1], x[2], t), bcy = lerp(y[1], y[2], t);
    double cdx = lerp(x[2], x[3], t), cdy = lerp(y[2], y[3], t);
    double abcx = lerp(abx, bcx, t), abcy = lerp(aby, bcy, t);
    double bcdx = lerp(bcx, cdx, t), bcdy = lerp(bcy, cdy, t);
    double ax = lerp(abcx, bcdx, t), ay = lerp(abcy, bcdy, t);
    dst[0] = src[0];
    dst[1] = Pt{(float)abx, (float)aby};
    dst[2] = Pt{(float)abcx, (float)abcy};
    dst[3] = Pt{(float)ax, (float)ay};
    dst[4] = Pt{(float)bcdx, (float)bcdy};
    dst[5] = Pt{(float)cdx, (float)cdy};
    dst[6] = src[3];
}
__device__ __forceinline__ float mono_cubic_closest_t(const float *src, float x) {
    float t = 0.5f, last_t, best_t = 0.5f, step = 0.25f;
    float D = src[0];
    float A = src[6] + 3.0f * (src[2] - src[4]) - D;
    float B = 3.0f * (src[4] - src[2] - src[2] + D);
    float C = 3.0f * (src[2] - D);
    x -= D;
    float closest = 3.4028235e38f;
    do {
        float loc = ((A * t + B) * t + C) * t;
        float dist = fabsf(loc - x);
        if (closest > dist) { closest = dist; best_t = t; }
        last_t = t;
        t += loc < x ? step : -step;
        step *= 0.5f;
    } while (closest > 0.25f && last_t != t);
    return best_t;
}
__device__ __forceinline__ void chop_mono_cubic_at(const Pt *src, float v, bool is_y, Pt *dst) {
    double t;
    if (mono_cubic_root(src, v, is_y, &t)) { chop_cubic_at_d(src, t, dst); return; }
    float tmp[8];
    for (int i = 0; i < 4; i++) { tmp[i * 2] = src[i].x; tmp[i * 2 + 1] = src[i].y; }
    float tt = mono_cubic_closest_t(is_y ? tmp + 1 : tmp, v);
    chop_cubic_at2(src, tt, dst);
}
__device__ __forceinline__ void emit_cubic(EdgeSink &s, const Pt *p, bool reverse, int shift) {
    Pt q[4];
    if (reverse) { q[0] = p[3]; q[1] = p[2]; q[2] = p[1]; q[3] = p[0]; }
    else { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; q[3] = p[3]; }
    push_cubic(s, q, shift);
}
__device__ __noinline__ void clip_mono_cubic(EdgeSink &s, const Pt *src, const ClipR &clip, int shift) {
    Pt pts[4];
    bool reverse;
    if (src[0].y > src[3].y) { for (int i = 0; i < 4; i++) pts[i] = src[3 - i]; reverse = true; }
    else { for (int i = 0; i < 4; i++) pts[i] = src[i]; reverse = false; }
    if (pts[3].y <= clip.t || pts[0].y >= clip.b) return;
    // chop in y
    if (pts[0].y < clip.t) {
        Pt tmp[7];
        chop_mono_cubic_at(pts, clip.t, true, tmp);
        if (tmp[3].y < clip.t && tmp[4].y < clip.t && tmp[5].y < clip.t) {
            Pt tmp2[4] = {tmp[3], tmp[4], tmp[5], tmp[6]};
            chop_mono_cubic_at(tmp2, clip.t, true, tmp);
        }
        tmp[3].y = clip.t;
        tmp[4].y = fmaxf(tmp[4].y, clip.t);
        pts[0] = tmp[3]; pts[1] = tmp[4]; pts[2] = tmp[5];
    }
    if (pts[3].y > clip.b) {
        Pt tmp[7];
        chop_mono_cubic_at(pts, clip.b, true, tmp);
        tmp[3].y = clip.b;
        tmp[2].y = fminf(tmp[2].y, clip.b);
        pts[1] = tmp[1]; pts[2] = tmp[2]; pts[3] = tmp[3];
    }
    if (pts[0].x > pts[3].x) {
        Pt q = pts[0]; pts[0] = pts[3]; pts[3] = q;
        q = pts[1]; pts[1] = pts[2]; pts[2] = q;
        reverse = !reverse;
    }
    if (pts[3].x <= clip.l) { append_vline(s, clip.l, pts[0].y, pts[3].y, reverse, shift); return; }
    if (pts[0].x >= clip.r) { append_vline(s, clip.r, pts[0].y, pts[3].y, reverse, shift); return; }
    if (pts[0].x < clip.l) {
        Pt tmp[7];
        chop_mono_cubic_at(pts, clip.l, false, tmp);
        append_vline(s, clip.l, tmp[0].y, tmp[3].y, reverse, shift);
        tmp[3].x = clip.l;
        tmp[4].x = fmaxf(tmp[4].x, clip.l);
        pts[0] = tmp[3]; pts[1] = tmp[4]; pts[2] = tmp[5];
    }
    if (pts[3].x > clip.r) {
        Pt tmp[7];
        chop_mono_cubic_at(pts, clip.r, false, tmp);
        tmp[3].x = clip.r;
        tmp[2].x = fminf(tmp[2].x, clip.r);
        emit_cubic(s, tmp, reverse, shift);
        append_vline(s, clip.r, tmp[3].y, tmp[6].y, reverse, shift);
    } else {
        emit_cubic(s, pts, reverse, shift);
    }
}
__device__ __noinline__ void clip_cubic(EdgeSink &s, const Pt *p, const ClipR &clip, int shift) {
    float l = fminf(fminf(p[0].x, p[1].x), fminf(p[2].x, p[3].x)), r = fmaxf(fmaxf(p[0].x, p[1].x), fmaxf(p[2].x, p[3].x));
    float t = fminf(fminf(p[0].y, p[1].y), fminf(p[2].y, p[3].y)), b = fmaxf(fmaxf(p[0].y, p[1].y), fmaxf(p[2].y, p[3].y));
    if (!(b > clip.t && t < clip.b)) return;
    const float lim = (float)(1 << 22);
    if (l < -lim || t < -lim || r > lim || b > lim) { clip_line(s, p[0], p[3], clip, shift); return; }
    Pt mono_y[10];
    int ny = chop_cubic_at_y_extrema(p, mono_y);
    for (int y = 0; y <= ny; y++) {
        Pt mono_x[10];
        int nx = chop_cubic_at_x_extrema(&mono_y[y * 3], mono_x);
        for (int x = 0; x <= nx; x++) clip_mono_cubic(s, &mono_x[x * 3], clip, shift);
    }
}

// One path segment -> line edges (EdgeBuilder::build for one PathEdge).
__device__ __forceinline__ void build_segment(EdgeSink &s, int kind, const Pt *p, bool contained, const ClipR &clip,
                                              int shift) {
    if (kind == 1) {
        if (contained) push_line(s, p[0], p[1], shift);
        else clip_line(s, p[0], p[1], clip, shift);
    } else if (kind == 2) {
        if (contained) {
            Pt mono[5];
            int n = chop_quad_at_y_extrema(p, mono);
            for (int i = 0; i <= n; i++) push_quad(s, &mono[i * 2], shift);
        } else {
            clip_quad(s, p, clip, shift);
        }
    } else if (kind == 3) {
        if (contained) {
            Pt mono[10];
            int n = chop_cubic_at_y_extrema(p, mono);
            for (int i = 0; i <= n; i++) push_cubic(s, &mono[i * 3], shift);
        } else {
            clip_cubic(s, p, clip, shift);
        }
    }
}

}  // namespace dev
}  // namespace rgpu
