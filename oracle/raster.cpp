// CPU oracle — test infrastructure only (see raster.h).
//
// Restatement of tiny-skia 0.12.0's raster path (itself Skia's algorithms):
//   * tiny-skia-path transform.rs  (Transform concat/invert/map_points)
//   * path_geometry.rs             (unit quad roots, cubic/quad chopping at extrema)
//   * edge.rs                      (SkEdge: fixed-point line/quad/cubic edges)
//   * edge_clipper.rs, line_clipper.rs (SkEdgeClipper / SkLineClipper)
//   * edge_builder.rs              (SkBasicEdgeBuilder incl. vertical-edge combining)
//   * scan/path.rs                 (walk_edges), scan/path_aa.rs (SuperBlitter, 4x4 SS)
//   * alpha_runs.rs                (SkAlphaRuns::add with catch-overflow)
//   * pipeline/{lowp,highp}.rs     (raster pipeline stage arithmetic)
//   * painter.rs / pixmap.rs / mask.rs (fill_path, fill_rect, draw_pixmap, masks)
// Compiled with -ffp-contract=off so that every a*b+c rounds twice, as in Rust.
#include "raster.h"
#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <type_traits>

namespace ora {

// ---------------------------------------------------------------- numerics
int32_t sat_i32(float v) {            // Rust `f32 as i32`
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
int32_t sat_i32d(double v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483647.0) return INT32_MAX;
    if (v <= -2147483648.0) return INT32_MIN;
    return (int32_t)v;
}
static inline uint8_t sat_u8(float v) {  // Rust `f32 as u8`
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}
static inline uint16_t sat_u16(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 65535.0f) return 65535;
    return (uint16_t)v;
}
uint8_t to_u8_norm(float v) {  // strict-num NormalizedF32::to_u8: (v*255 + 0.5) as u8
    return sat_u8(v * 255.0f + 0.5f);
}
ColorF color_from_rgba8(uint8_t r, uint8_t g, uint8_t b, uint8_t a) {
    return ColorF{r / 255.0f, g / 255.0f, b / 255.0f, a / 255.0f};
}
static const float SCALAR_NEARLY_ZERO = 1.0f / (1 << 12);
static bool is_nearly_zero(float v) { return std::fabs(v) <= SCALAR_NEARLY_ZERO; }
static bool is_nearly_zero_tol(float v, float tol) { return std::fabs(v) <= tol; }

// ---------------------------------------------------------------- transform
static float mul_add_mul(float a, float b, float c, float d) {
    return (float)((double)a * (double)b + (double)c * (double)d);
}
static Transform concat(const Transform &a, const Transform &b) {
    if (a.is_identity()) return b;
    if (b.is_identity()) return a;
    if (!a.has_skew() && !b.has_skew()) {
        return Transform::from_row(a.sx * b.sx, 0, 0, a.sy * b.sy, a.sx * b.tx + a.tx, a.sy * b.ty + a.ty);
    }
    return Transform::from_row(mul_add_mul(a.sx, b.sx, a.kx, b.ky), mul_add_mul(a.ky, b.sx, a.sy, b.ky),
                               mul_add_mul(a.sx, b.kx, a.kx, b.sy), mul_add_mul(a.ky, b.kx, a.sy, b.sy),
                               mul_add_mul(a.sx, b.tx, a.kx, b.ty) + a.tx,
                               mul_add_mul(a.ky, b.tx, a.sy, b.ty) + a.ty);
}
Transform Transform::pre_concat(const Transform &o) const { return concat(*this, o); }
Transform Transform::post_concat(const Transform &o) const { return concat(o, *this); }
bool Transform::is_finite() const {
    return std::isfinite(sx) && std::isfinite(ky) && std::isfinite(kx) && std::isfinite(sy) &&
           std::isfinite(tx) && std::isfinite(ty);
}
bool Transform::invert(Transform *out) const {
    if (is_identity()) { *out = *this; return true; }
    if (is_scale_translate()) {
        if (has_scale()) {
            float ix = 1.0f / sx, iy = 1.0f / sy;
            *out = from_row(ix, 0, 0, iy, -tx * ix, -ty * iy);
        } else {
            *out = translate(-tx, -ty);
        }
        return true;
    }
    double det = (double)sx * (double)sy - (double)kx * (double)ky;
    float tol = SCALAR_NEARLY_ZERO * SCALAR_NEARLY_ZERO * SCALAR_NEARLY_ZERO;
    if (is_nearly_zero_tol((float)det, tol)) return false;
    double inv = 1.0 / det;
    Transform t = from_row((float)(sy * inv), (float)(-ky * inv), (float)(-kx * inv), (float)(sx * inv),
                           (float)(((double)kx * ty - (double)sy * tx) * inv),
                           (float)(((double)ky * tx - (double)sx * ty) * inv));
    if (!t.is_finite()) return false;
    *out = t;
    return true;
}
void Transform::map_points(Point *p, size_t n) const {
    if (is_identity()) return;
    if (is_translate()) {
        for (size_t i = 0; i < n; i++) { p[i].x += tx; p[i].y += ty; }
    } else if (is_scale_translate()) {
        for (size_t i = 0; i < n; i++) { p[i].x = p[i].x * sx + tx; p[i].y = p[i].y * sy + ty; }
    } else {
        for (size_t i = 0; i < n; i++) {
            float x = p[i].x * sx + p[i].y * kx + tx;
            float y = p[i].x * ky + p[i].y * sy + ty;
            p[i].x = x; p[i].y = y;
        }
    }
}
void Transform::get_scale(float *x, float *y) const {
    *x = std::sqrt(sx * sx + kx * kx);
    *y = std::sqrt(ky * ky + sy * sy);
}

// ---------------------------------------------------------------- path
void Path::compute_bounds() {
    if (pts.empty()) { bounds = Rect{0, 0, 0, 0}; return; }
    float l = pts[0].x, r = pts[0].x, t = pts[0].y, b = pts[0].y;
    for (auto &p : pts) {
        l = std::min(l, p.x); r = std::max(r, p.x);
        t = std::min(t, p.y); b = std::max(b, p.y);
    }
    bounds = Rect{l, t, r, b};
}
bool Path::transform(const Transform &ts) {
    ts.map_points(pts.data(), pts.size());
    for (auto &p : pts)
        if (!std::isfinite(p.x) || !std::isfinite(p.y)) return false;
    compute_bounds();
    return true;
}

Rect rect_transform(const Rect &r, const Transform &ts, bool *ok) {
    Point p[4] = {{r.l, r.t}, {r.r, r.t}, {r.r, r.b}, {r.l, r.b}};
    ts.map_points(p, 4);
    Rect o{p[0].x, p[0].y, p[0].x, p[0].y};
    for (int i = 1; i < 4; i++) {
        o.l = std::min(o.l, p[i].x); o.r = std::max(o.r, p[i].x);
        o.t = std::min(o.t, p[i].y); o.b = std::max(o.b, p[i].y);
    }
    *ok = std::isfinite(o.l) && std::isfinite(o.t) && std::isfinite(o.r) && std::isfinite(o.b) && o.r > o.l &&
          o.b > o.t;
    return o;
}
// NonZeroRect::to_int_rect: floor origin, ceil size, size >= 1.
bool rect_to_int_rect(const Rect &r, IntRect *out) {
    int32_t x = sat_i32(std::floor(r.l)), y = sat_i32(std::floor(r.t));
    int64_t w = std::max<int64_t>(1, (int64_t)std::ceil(r.w()));
    int64_t h = std::max<int64_t>(1, (int64_t)std::ceil(r.h()));
    if ((int64_t)x + w > INT32_MAX || (int64_t)y + h > INT32_MAX) return false;
    *out = IntRect{x, y, (int32_t)w, (int32_t)h};
    return true;
}

// ---------------------------------------------------------------- geometry
// path_geometry.rs: valid_unit_divide / find_unit_quad_roots
static bool valid_unit_divide(float numer, float denom, float *ratio) {
    if (numer < 0) { numer = -numer; denom = -denom; }
    if (denom == 0 || numer == 0 || numer >= denom) return false;
    float r = numer / denom;
    if (std::isnan(r)) return false;
    if (r == 0) return false;
    *ratio = r;
    return true;
}
static int find_unit_quad_roots(float a, float b, float c, float roots[2]) {
    if (a == 0) return valid_unit_divide(-c, b, &roots[0]) ? 1 : 0;
    double dr = (double)b * (double)b - 4.0 * (double)a * (double)c;
    if (dr < 0) return 0;
    dr = std::sqrt(dr);
    float r = (float)dr;
    if (!std::isfinite(r)) return 0;
    float q = (b < 0) ? -(b - r) / 2.0f : -(b + r) / 2.0f;
    int n = 0;
    if (valid_unit_divide(q, a, &roots[n])) n++;
    if (valid_unit_divide(c, q, &roots[n])) n++;
    if (n == 2) {
        if (roots[0] > roots[1]) std::swap(roots[0], roots[1]);
        else if (roots[0] == roots[1]) n--;
    }
    return n;
}
static inline Point interp(Point a, Point b, float t) { return Point{a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t}; }
static void chop_cubic_at2(const Point *src, float t, Point *dst) {
    Point ab = interp(src[0], src[1], t), bc = interp(src[1], src[2], t), cd = interp(src[2], src[3], t);
    Point abc = interp(ab, bc, t), bcd = interp(bc, cd, t), abcd = interp(abc, bcd, t);
    dst[0] = src[0]; dst[1] = ab; dst[2] = abc; dst[3] = abcd; dst[4] = bcd; dst[5] = cd; dst[6] = src[3];
}
static void chop_cubic_at(const Point *src, const float *ts, int n, Point *dst) {
    if (n == 0) { for (int i = 0; i < 4; i++) dst[i] = src[i]; return; }
    float t = ts[0];
    Point tmp[4];
    int off = 0;
    for (int i = 0; i < n; i++) {
        chop_cubic_at2(src, t, dst + off);
        if (i == n - 1) break;
        off += 3;
        for (int k = 0; k < 4; k++) tmp[k] = dst[off + k];
        src = tmp;
        float nt;
        if (!valid_unit_divide(ts[i + 1] - ts[i], 1.0f - ts[i], &nt)) {
            dst[off + 4] = src[3]; dst[off + 5] = src[3]; dst[off + 6] = src[3];
            break;
        }
        t = nt;
    }
}
static int find_cubic_extrema(float a, float b, float c, float d, float ts[2]) {
    float A = d - a + 3.0f * (b - c);
    float B = 2.0f * (a - b - b + c);
    float C = b - a;
    return find_unit_quad_roots(A, B, C, ts);
}
// chop_cubic_at_y_extrema: dst holds 1 + 3n points' worth (up to 10)
static int chop_cubic_at_y_extrema(const Point *src, Point *dst) {
    float ts[2];
    int n = find_cubic_extrema(src[0].y, src[1].y, src[2].y, src[3].y, ts);
    chop_cubic_at(src, ts, n, dst);
    if (n > 0) {
        dst[2].y = dst[3].y; dst[4].y = dst[3].y;
        if (n == 2) { dst[5].y = dst[6].y; dst[7].y = dst[6].y; }
    }
    return n;
}
static int chop_cubic_at_x_extrema(const Point *src, Point *dst) {
    float ts[2];
    int n = find_cubic_extrema(src[0].x, src[1].x, src[2].x, src[3].x, ts);
    chop_cubic_at(src, ts, n, dst);
    if (n > 0) {
        dst[2].x = dst[3].x; dst[4].x = dst[3].x;
        if (n == 2) { dst[5].x = dst[6].x; dst[7].x = dst[6].x; }
    }
    return n;
}
static void chop_quad_at(const Point *src, float t, Point *dst) {
    Point p01 = interp(src[0], src[1], t), p12 = interp(src[1], src[2], t);
    dst[0] = src[0]; dst[1] = p01; dst[2] = interp(p01, p12, t); dst[3] = p12; dst[4] = src[2];
}
static bool is_not_monotonic(float a, float b, float c) {
    float ab = a - b, bc = b - c;
    if (ab < 0) bc = -bc;
    return ab == 0 || bc < 0;
}
static int chop_quad_at_y_extrema(const Point *src, Point *dst) {
    float a = src[0].y, b = src[1].y, c = src[2].y;
    if (is_not_monotonic(a, b, c)) {
        float t;
        if (valid_unit_divide(a - b, a - b - b + c, &t)) {
            chop_quad_at(src, t, dst);
            dst[1].y = dst[2].y; dst[3].y = dst[2].y;
            return 1;
        }
        b = (std::fabs(a - b) < std::fabs(b - c)) ? a : c;
    }
    dst[0] = Point{src[0].x, a}; dst[1] = Point{src[1].x, b}; dst[2] = Point{src[2].x, c};
    return 0;
}
static int chop_quad_at_x_extrema(const Point *src, Point *dst) {
    float a = src[0].x, b = src[1].x, c = src[2].x;
    if (is_not_monotonic(a, b, c)) {
        float t;
        if (valid_unit_divide(a - b, a - b - b + c, &t)) {
            chop_quad_at(src, t, dst);
            dst[1].x = dst[2].x; dst[3].x = dst[2].x;
            return 1;
        }
        b = (std::fabs(a - b) < std::fabs(b - c)) ? a : c;
    }
    dst[0] = Point{a, src[0].y}; dst[1] = Point{b, src[1].y}; dst[2] = Point{c, src[2].y};
    return 0;
}

// ---------------------------------------------------------------- fixed point (fdot6 / fdot16)
typedef int32_t FDot6;
typedef int32_t FDot16;
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t lshift(int32_t v, int s) { return (int32_t)((uint32_t)v << s); }
static inline FDot6 fdot6_round(FDot6 n) { return (n + 32) >> 6; }
static inline FDot16 fdot6_to_fdot16(FDot6 v) { return lshift(v, 10); }
static inline FDot16 fdot16_mul(FDot16 a, FDot16 b) { return (int32_t)(((int64_t)a * (int64_t)b) >> 16); }
static inline FDot16 fdot16_div(FDot6 numer, FDot6 denom) {
    int64_t v = ((int64_t)numer * 65536) / (int64_t)denom;
    if (v < INT32_MIN) v = INT32_MIN;
    if (v > INT32_MAX) v = INT32_MAX;
    return (int32_t)v;
}
static inline FDot16 fdot6_div(FDot6 a, FDot6 b) {
    if (a >= -32768 && a <= 32767) return lshift(a, 16) / b;
    return fdot16_div(a, b);
}
static inline int32_t fdot16_round_to_i32(FDot16 x) { return wadd(x, 0x8000) >> 16; }
static inline FDot6 compute_dy(FDot6 top, FDot6 y0) { return lshift(top, 6) + 32 - y0; }

// ---------------------------------------------------------------- edges (edge.rs)
enum EdgeType { EDGE_LINE, EDGE_QUAD, EDGE_CUBIC };
struct Edge {
    EdgeType type = EDGE_LINE;
    // LineEdge
    FDot16 x = 0, dx = 0;
    int32_t first_y = 0, last_y = 0;
    int8_t winding = 1;
    // curve state
    int8_t curve_count = 0;
    uint8_t curve_shift = 0, cubic_dshift = 0;
    FDot16 qx, qy, qdx, qdy, qddx, qddy, qlast_x, qlast_y;        // quad
    FDot16 cx, cy, cdx, cdy, cddx, cddy, cdddx, cdddy, clast_x, clast_y;  // cubic
    // list links (indices into the edge vector)
    int prev = -1, next = -1;
};

static bool line_update(Edge &e, FDot16 x0, FDot16 y0, FDot16 x1, FDot16 y1) {
    y0 >>= 10; y1 >>= 10;
    int32_t top = fdot6_round(y0), bot = fdot6_round(y1);
    if (top == bot) return false;
    x0 >>= 10; x1 >>= 10;
    FDot16 slope = fdot6_div(x1 - x0, y1 - y0);
    FDot6 dy = compute_dy(top, y0);
    e.x = fdot6_to_fdot16(x0 + fdot16_mul(slope, dy));
    e.dx = slope;
    e.first_y = top;
    e.last_y = bot - 1;
    return true;
}
static bool line_new(const Point &p0, const Point &p1, int shift, Edge &e) {
    float scale = (float)(1 << (shift + 6));
    FDot6 x0 = sat_i32(p0.x * scale), y0 = sat_i32(p0.y * scale);
    FDot6 x1 = sat_i32(p1.x * scale), y1 = sat_i32(p1.y * scale);
    int8_t winding = 1;
    if (y0 > y1) { std::swap(x0, x1); std::swap(y0, y1); winding = -1; }
    int32_t top = fdot6_round(y0), bottom = fdot6_round(y1);
    if (top == bottom) return false;
    FDot16 slope = fdot6_div(x1 - x0, y1 - y0);
    FDot6 dy = compute_dy(top, y0);
    e = Edge();
    e.type = EDGE_LINE;
    e.x = fdot6_to_fdot16(x0 + fdot16_mul(slope, dy));
    e.dx = slope;
    e.first_y = top;
    e.last_y = bottom - 1;
    e.winding = winding;
    return true;
}
static FDot6 cheap_distance(FDot6 dx, FDot6 dy) {
    dx = std::abs(dx); dy = std::abs(dy);
    return dx > dy ? dx + (dy >> 1) : dy + (dx >> 1);
}
static int diff_to_shift(FDot6 dx, FDot6 dy, int shift_aa) {
    FDot6 dist = cheap_distance(dx, dy);
    dist = (dist + (1 << 4)) >> (3 + shift_aa);
    int lz = dist == 0 ? 32 : __builtin_clz((uint32_t)dist);
    return (32 - lz) >> 1;
}
static const int MAX_COEFF_SHIFT = 6;

static bool quad_update(Edge &e) {
    bool success;
    int count = e.curve_count;
    FDot16 oldx = e.qx, oldy = e.qy, dx = e.qdx, dy = e.qdy, newx, newy;
    int shift = e.curve_shift;
    do {
        count--;
        if (count > 0) {
            newx = oldx + (dx >> shift); dx += e.qddx;
            newy = oldy + (dy >> shift); dy += e.qddy;
        } else {
            newx = e.qlast_x; newy = e.qlast_y;
        }
        success = line_update(e, oldx, oldy, newx, newy);
        oldx = newx; oldy = newy;
    } while (count > 0 && !success);
    e.qx = newx; e.qy = newy; e.qdx = dx; e.qdy = dy;
    e.curve_count = (int8_t)count;
    return success;
}
static bool quad_new(const Point *pts, int shift, Edge &e) {
    float scale = (float)(1 << (shift + 6));
    FDot6 x0 = sat_i32(pts[0].x * scale), y0 = sat_i32(pts[0].y * scale);
    FDot6 x1 = sat_i32(pts[1].x * scale), y1 = sat_i32(pts[1].y * scale);
    FDot6 x2 = sat_i32(pts[2].x * scale), y2 = sat_i32(pts[2].y * scale);
    int8_t winding = 1;
    if (y0 > y2) { std::swap(x0, x2); std::swap(y0, y2); winding = -1; }
    int32_t top = fdot6_round(y0), bot = fdot6_round(y2);
    if (top == bot) return false;
    {
        FDot6 dx = (lshift(x1, 1) - x0 - x2) >> 2;
        FDot6 dy = (lshift(y1, 1) - y0 - y2) >> 2;
        shift = diff_to_shift(dx, dy, shift);
    }
    if (shift == 0) shift = 1;
    else if (shift > MAX_COEFF_SHIFT) shift = MAX_COEFF_SHIFT;
    e = Edge();
    e.type = EDGE_QUAD;
    e.winding = winding;
    e.curve_count = (int8_t)(1 << shift);
    e.curve_shift = (uint8_t)(shift - 1);
    FDot16 A = lshift(x0 - x1 - x1 + x2, 9);
    FDot16 B = fdot6_to_fdot16(x1 - x0);
    e.qx = fdot6_to_fdot16(x0);
    e.qdx = B + (A >> shift);
    e.qddx = A >> (shift - 1);
    A = lshift(y0 - y1 - y1 + y2, 9);
    B = fdot6_to_fdot16(y1 - y0);
    e.qy = fdot6_to_fdot16(y0);
    e.qdy = B + (A >> shift);
    e.qddy = A >> (shift - 1);
    e.qlast_x = fdot6_to_fdot16(x2);
    e.qlast_y = fdot6_to_fdot16(y2);
    return quad_update(e);
}
static FDot6 cubic_delta_from_line(FDot6 a, FDot6 b, FDot6 c, FDot6 d) {
    FDot6 one_third = ((a * 8 - b * 15 + 6 * c + d) * 19) >> 9;
    FDot6 two_third = ((a + 6 * b - c * 15 + d * 8) * 19) >> 9;
    return std::max(std::abs(one_third), std::abs(two_third));
}
static bool cubic_update(Edge &e) {
    bool success;
    int count = e.curve_count;
    FDot16 oldx = e.cx, oldy = e.cy, newx, newy;
    int ddshift = e.curve_shift, dshift = e.cubic_dshift;
    do {
        count++;
        if (count < 0) {
            newx = oldx + (e.cdx >> dshift); e.cdx += e.cddx >> ddshift; e.cddx += e.cdddx;
            newy = oldy + (e.cdy >> dshift); e.cdy += e.cddy >> ddshift; e.cddy += e.cdddy;
        } else {
            newx = e.clast_x; newy = e.clast_y;
        }
        if (newy < oldy) newy = oldy;
        success = line_update(e, oldx, oldy, newx, newy);
        oldx = newx; oldy = newy;
    } while (count < 0 && !success);
    e.cx = newx; e.cy = newy;
    e.curve_count = (int8_t)count;
    return success;
}
static bool cubic_new(const Point *pts, int shift, Edge &e) {
    float scale = (float)(1 << (shift + 6));
    FDot6 x0 = sat_i32(pts[0].x * scale), y0 = sat_i32(pts[0].y * scale);
    FDot6 x1 = sat_i32(pts[1].x * scale), y1 = sat_i32(pts[1].y * scale);
    FDot6 x2 = sat_i32(pts[2].x * scale), y2 = sat_i32(pts[2].y * scale);
    FDot6 x3 = sat_i32(pts[3].x * scale), y3 = sat_i32(pts[3].y * scale);
    int8_t winding = 1;
    if (y0 > y3) {
        std::swap(x0, x3); std::swap(x1, x2); std::swap(y0, y3); std::swap(y1, y2);
        winding = -1;
    }
    int32_t top = fdot6_round(y0), bot = fdot6_round(y3);
    if (top == bot) return false;
    {
        FDot6 dx = cubic_delta_from_line(x0, x1, x2, x3);
        FDot6 dy = cubic_delta_from_line(y0, y1, y2, y3);
        shift = diff_to_shift(dx, dy, 2) + 1;
    }
    if (shift > MAX_COEFF_SHIFT) shift = MAX_COEFF_SHIFT;
    int up_shift = 6;
    int down_shift = shift + up_shift - 10;
    if (down_shift < 0) { down_shift = 0; up_shift = 10 - shift; }
    e = Edge();
    e.type = EDGE_CUBIC;
    e.winding = winding;
    e.curve_count = (int8_t)(-(1 << shift));
    e.curve_shift = (uint8_t)shift;
    e.cubic_dshift = (uint8_t)down_shift;
    FDot16 B = lshift(3 * (x1 - x0), up_shift);
    FDot16 C = lshift(3 * (x0 - x1 - x1 + x2), up_shift);
    FDot16 D = lshift(x3 + 3 * (x1 - x2) - x0, up_shift);
    e.cx = fdot6_to_fdot16(x0);
    e.cdx = B + (C >> shift) + (D >> (2 * shift));
    e.cddx = 2 * C + ((3 * D) >> (shift - 1));
    e.cdddx = (3 * D) >> (shift - 1);
    B = lshift(3 * (y1 - y0), up_shift);
    C = lshift(3 * (y0 - y1 - y1 + y2), up_shift);
    D = lshift(y3 + 3 * (y1 - y2) - y0, up_shift);
    e.cy = fdot6_to_fdot16(y0);
    e.cdy = B + (C >> shift) + (D >> (2 * shift));
    e.cddy = 2 * C + ((3 * D) >> (shift - 1));
    e.cdddy = (3 * D) >> (shift - 1);
    e.clast_x = fdot6_to_fdot16(x3);
    e.clast_y = fdot6_to_fdot16(y3);
    return cubic_update(e);
}

// ---------------------------------------------------------------- line clipper (line_clipper.rs)
static float pin_unsorted_f(double v, double a, double b) {
    if (a > b) std::swap(a, b);
    if (v < a) v = a;
    if (v > b) v = b;
    return (float)v;
}
static float sect_with_horizontal(const Point src[2], float Y) {
    float dy = src[1].y - src[0].y;
    if (is_nearly_zero(dy)) return (src[0].x + src[1].x) * 0.5f;
    double X0 = src[0].x, Y0 = src[0].y, X1 = src[1].x, Y1 = src[1].y;
    double r = X0 + ((double)Y - Y0) * (X1 - X0) / (Y1 - Y0);
    return pin_unsorted_f(r, X0, X1);
}
static float sect_with_vertical(const Point src[2], float X) {
    float dx = src[1].x - src[0].x;
    if (is_nearly_zero(dx)) return (src[0].y + src[1].y) * 0.5f;
    double X0 = src[0].x, Y0 = src[0].y, X1 = src[1].x, Y1 = src[1].y;
    return (float)(Y0 + ((double)X - X0) * (Y1 - Y0) / (X1 - X0));
}
static float sect_clamp_with_vertical(const Point src[2], float x) {
    float y = sect_with_vertical(src, x);
    float a = src[0].y, b = src[1].y;
    if (a > b) std::swap(a, b);
    return std::min(std::max(y, a), b);
}
// returns number of lines (points = n+1) into lines[0..4]
static int clip_line_pts(const Point pts[2], const Rect &clip, Point lines[4], bool can_cull_right) {
    int i0, i1;
    if (pts[0].y < pts[1].y) { i0 = 0; i1 = 1; } else { i0 = 1; i1 = 0; }
    if (pts[i1].y <= clip.t) return 0;
    if (pts[i0].y >= clip.b) return 0;
    Point tmp[2] = {pts[0], pts[1]};
    if (pts[i0].y < clip.t) tmp[i0] = Point{sect_with_horizontal(pts, clip.t), clip.t};
    if (tmp[i1].y > clip.b) tmp[i1] = Point{sect_with_horizontal(pts, clip.b), clip.b};
    Point storage[4];
    Point *result;
    int line_count = 1;
    bool reverse;
    if (pts[0].x < pts[1].x) { i0 = 0; i1 = 1; reverse = false; } else { i0 = 1; i1 = 0; reverse = true; }
    if (tmp[i1].x <= clip.l) {
        tmp[0].x = tmp[1].x = clip.l;
        result = tmp; reverse = false;
    } else if (tmp[i0].x >= clip.r) {
        if (can_cull_right) return 0;
        tmp[0].x = tmp[1].x = clip.r;
        result = tmp; reverse = false;
    } else {
        result = storage;
        Point *r = result;
        if (tmp[i0].x < clip.l) {
            *r = Point{clip.l, tmp[i0].y}; r++;
            *r = Point{clip.l, sect_clamp_with_vertical(tmp, clip.l)};
        } else {
            *r = tmp[i0];
        }
        r++;
        if (tmp[i1].x > clip.r) {
            *r = Point{clip.r, sect_clamp_with_vertical(tmp, clip.r)}; r++;
            *r = Point{clip.r, tmp[i1].y};
        } else {
            *r = tmp[i1];
        }
        line_count = (int)(r - result);
    }
    if (reverse) {
        for (int i = 0; i <= line_count; i++) lines[line_count - i] = result[i];
    } else {
        for (int i = 0; i <= line_count; i++) lines[i] = result[i];
    }
    return line_count;
}

// ---------------------------------------------------------------- edge clipper (edge_clipper.rs)
enum SegKind { SEG_LINE = 1, SEG_QUAD = 2, SEG_CUBIC = 3 };
struct Seg { int kind; Point p[4]; };

struct EdgeClipper {
    Rect clip;
    bool can_cull_right;
    std::vector<Seg> out;

    void append_line(Point a, Point b) { out.push_back(Seg{SEG_LINE, {a, b}}); }
    void append_vline(float x, float y0, float y1, bool reverse) {
        if (reverse) std::swap(y0, y1);
        append_line(Point{x, y0}, Point{x, y1});
    }
    void clip_line(Point p0, Point p1) {
        Point pts[2] = {p0, p1}, lines[4];
        int n = clip_line_pts(pts, clip, lines, can_cull_right);
        for (int i = 0; i < n; i++) append_line(lines[i], lines[i + 1]);
    }
    // ---- quads
    static bool chop_mono_quad_at(const Point *src, float y, bool is_y, float *t) {
        float c0 = is_y ? src[0].y : src[0].x, c1 = is_y ? src[1].y : src[1].x, c2 = is_y ? src[2].y : src[2].x;
        float a = c0 - c1 - c1 + c2, b = 2.0f * (c1 - c0), c = c0 - y;
        float roots[2];
        int n = find_unit_quad_roots(a, b, c, roots);
        if (n) { *t = roots[0]; return true; }
        return false;
    }
    static void chop_quad_in_y(Point pts[3], const Rect &clip) {
        float t;
        Point tmp[5];
        if (pts[0].y < clip.t) {
            if (chop_mono_quad_at(pts, clip.t, true, &t)) {
                chop_quad_at(pts, t, tmp);
                tmp[2].y = clip.t;
                tmp[3].y = std::max(tmp[3].y, clip.t);
                pts[0] = tmp[2]; pts[1] = tmp[3];
            } else {
                for (int i = 0; i < 3; i++)
                    if (pts[i].y < clip.t) pts[i].y = clip.t;
            }
        }
        if (pts[2].y > clip.b) {
            if (chop_mono_quad_at(pts, clip.b, true, &t)) {
                chop_quad_at(pts, t, tmp);
                tmp[1].y = std::min(tmp[1].y, clip.b);
                tmp[2].y = clip.b;
                pts[1] = tmp[1]; pts[2] = tmp[2];
            } else {
                for (int i = 0; i < 3; i++)
                    if (pts[i].y > clip.b) pts[i].y = clip.b;
            }
        }
    }
    void append_quad(const Point *p, bool reverse) {
        Seg s{SEG_QUAD, {}};
        if (reverse) { s.p[0] = p[2]; s.p[1] = p[1]; s.p[2] = p[0]; }
        else { s.p[0] = p[0]; s.p[1] = p[1]; s.p[2] = p[2]; }
        out.push_back(s);
    }
    void clip_mono_quad(const Point src[3]) {
        Point pts[3];
        bool reverse;
        if (src[0].y > src[2].y) { pts[0] = src[2]; pts[1] = src[1]; pts[2] = src[0]; reverse = true; }
        else { pts[0] = src[0]; pts[1] = src[1]; pts[2] = src[2]; reverse = false; }
        if (pts[2].y <= clip.t || pts[0].y >= clip.b) return;
        chop_quad_in_y(pts, clip);
        if (pts[0].x > pts[2].x) { std::swap(pts[0], pts[2]); reverse = !reverse; }
        if (pts[2].x <= clip.l) { append_vline(clip.l, pts[0].y, pts[2].y, reverse); return; }
        if (pts[0].x >= clip.r) {
            if (!can_cull_right) append_vline(clip.r, pts[0].y, pts[2].y, reverse);
            return;
        }
        float t;
        Point tmp[5];
        if (pts[0].x < clip.l) {
            if (chop_mono_quad_at(pts, clip.l, false, &t)) {
                chop_quad_at(pts, t, tmp);
                append_vline(clip.l, tmp[0].y, tmp[2].y, reverse);
                tmp[2].x = clip.l;
                tmp[3].x = std::max(tmp[3].x, clip.l);
                pts[0] = tmp[2]; pts[1] = tmp[3];
            } else {
                append_vline(clip.l, pts[0].y, pts[2].y, reverse);
                return;
            }
        }
        if (pts[2].x > clip.r) {
            if (chop_mono_quad_at(pts, clip.r, false, &t)) {
                chop_quad_at(pts, t, tmp);
                tmp[1].x = std::min(tmp[1].x, clip.r);
                tmp[2].x = clip.r;
                append_quad(tmp, reverse);
                append_vline(clip.r, tmp[2].y, tmp[4].y, reverse);
            } else {
                pts[1].x = std::min(pts[1].x, clip.r);
                pts[2].x = std::min(pts[2].x, clip.r);
                append_quad(pts, reverse);
            }
        } else {
            append_quad(pts, reverse);
        }
    }
    void clip_quad(const Point *p) {
        float l = std::min({p[0].x, p[1].x, p[2].x}), r = std::max({p[0].x, p[1].x, p[2].x});
        float t = std::min({p[0].y, p[1].y, p[2].y}), b = std::max({p[0].y, p[1].y, p[2].y});
        (void)l; (void)r;
        if (!(b > clip.t && t < clip.b)) return;
        Point mono_y[5];
        int ny = chop_quad_at_y_extrema(p, mono_y);
        for (int y = 0; y <= ny; y++) {
            Point mono_x[5];
            int nx = chop_quad_at_x_extrema(&mono_y[y * 2], mono_x);
            for (int x = 0; x <= nx; x++) clip_mono_quad(&mono_x[x * 2]);
        }
    }
    // ---- cubics
    // Root of a monotonic cubic coordinate = v, in double: bisection refined to full
    // precision, then the curve is split in double and rounded to f32 (tiny-skia's
    // cubic_dchop_at_intercept works in f64 as well).
    static bool mono_cubic_root(const Point *src, float v, bool is_y, double *t_out) {
        double c[4];
        for (int i = 0; i < 4; i++) c[i] = is_y ? src[i].y : src[i].x;
        double A = c[3] + 3.0 * (c[1] - c[2]) - c[0];
        double B = 3.0 * (c[2] - 2.0 * c[1] + c[0]);
        double C = 3.0 * (c[1] - c[0]);
        double D = c[0] - v;
        auto f = [&](double t) { return ((A * t + B) * t + C) * t + D; };
        double f0 = f(0.0), f1 = f(1.0);
        if (f0 == 0.0) { *t_out = 0.0; return true; }
        if (f1 == 0.0) { *t_out = 1.0; return true; }
        if ((f0 < 0) == (f1 < 0)) return false;
        double lo = 0.0, hi = 1.0;
        bool inc = f0 < 0;
        for (int it = 0; it < 100; it++) {
            double mid = 0.5 * (lo + hi);
            if (mid <= lo || mid >= hi) break;
            double fm = f(mid);
            if (fm == 0.0) { lo = hi = mid; break; }
            if ((fm < 0) == inc) lo = mid; else hi = mid;
        }
        *t_out = 0.5 * (lo + hi);
        return true;
    }
    static void chop_cubic_at_d(const Point *src, double t, Point *dst) {
        double x[4], y[4];
        for (int i = 0; i < 4; i++) { x[i] = src[i].x; y[i] = src[i].y; }
        auto lerp = [](double a, double b, double t) { return a + (b - a) * t; };
        double abx = lerp(x[0], x[1], t), aby = lerp(y[0], y[1], t);
        double bcx = lerp(x[1], x[2], t), bcy = lerp(y[1], y[2], t);
        double cdx = lerp(x[2], x[3], t), cdy = lerp(y[2], y[3], t);
        double abcx = lerp(abx, bcx, t), abcy = lerp(aby, bcy, t);
        double bcdx = lerp(bcx, cdx, t), bcdy = lerp(bcy, cdy, t);
        double ax = lerp(abcx, bcdx, t), ay = lerp(abcy, bcdy, t);
        dst[0] = src[0];
        dst[1] = Point{(float)abx, (float)aby};
        dst[2] = Point{(float)abcx, (float)abcy};
        dst[3] = Point{(float)ax, (float)ay};
        dst[4] = Point{(float)bcdx, (float)bcdy};
        dst[5] = Point{(float)cdx, (float)cdy};
        dst[6] = src[3];
    }
    static float mono_cubic_closest_t(const float *src /*stride 2*/, float x) {
        float t = 0.5f, last_t, best_t = 0.5f, step = 0.25f;
        float D = src[0];
        float A = src[6] + 3.0f * (src[2] - src[4]) - D;
        float B = 3.0f * (src[4] - src[2] - src[2] + D);
        float C = 3.0f * (src[2] - D);
        x -= D;
        float closest = FLT_MAX;
        do {
            float loc = ((A * t + B) * t + C) * t;
            float dist = std::fabs(loc - x);
            if (closest > dist) { closest = dist; best_t = t; }
            last_t = t;
            t += loc < x ? step : -step;
            step *= 0.5f;
        } while (closest > 0.25f && last_t != t);
        return best_t;
    }
    static void chop_mono_cubic_at(const Point *src, float v, bool is_y, Point *dst) {
        double t;
        if (mono_cubic_root(src, v, is_y, &t)) { chop_cubic_at_d(src, t, dst); return; }
        float tmp[8];
        for (int i = 0; i < 4; i++) { tmp[i * 2] = src[i].x; tmp[i * 2 + 1] = src[i].y; }
        float tt = mono_cubic_closest_t(is_y ? tmp + 1 : tmp, v);
        chop_cubic_at2(src, tt, dst);
    }
    static void chop_cubic_in_y(Point pts[4], const Rect &clip) {
        if (pts[0].y < clip.t) {
            Point tmp[7];
            chop_mono_cubic_at(pts, clip.t, true, tmp);
            if (tmp[3].y < clip.t && tmp[4].y < clip.t && tmp[5].y < clip.t) {
                Point tmp2[4] = {tmp[3], tmp[4], tmp[5], tmp[6]};
                chop_mono_cubic_at(tmp2, clip.t, true, tmp);
            }
            tmp[3].y = clip.t;
            tmp[4].y = std::max(tmp[4].y, clip.t);
            pts[0] = tmp[3]; pts[1] = tmp[4]; pts[2] = tmp[5];
        }
        if (pts[3].y > clip.b) {
            Point tmp[7];
            chop_mono_cubic_at(pts, clip.b, true, tmp);
            tmp[3].y = clip.b;
            tmp[2].y = std::min(tmp[2].y, clip.b);
            pts[1] = tmp[1]; pts[2] = tmp[2]; pts[3] = tmp[3];
        }
    }
    void append_cubic(const Point *p, bool reverse) {
        Seg s{SEG_CUBIC, {}};
        if (reverse) { s.p[0] = p[3]; s.p[1] = p[2]; s.p[2] = p[1]; s.p[3] = p[0]; }
        else { for (int i = 0; i < 4; i++) s.p[i] = p[i]; }
        out.push_back(s);
    }
    void clip_mono_cubic(const Point src[4]) {
        Point pts[4];
        bool reverse;
        if (src[0].y > src[3].y) { for (int i = 0; i < 4; i++) pts[i] = src[3 - i]; reverse = true; }
        else { for (int i = 0; i < 4; i++) pts[i] = src[i]; reverse = false; }
        if (pts[3].y <= clip.t || pts[0].y >= clip.b) return;
        chop_cubic_in_y(pts, clip);
        if (pts[0].x > pts[3].x) { std::swap(pts[0], pts[3]); std::swap(pts[1], pts[2]); reverse = !reverse; }
        if (pts[3].x <= clip.l) { append_vline(clip.l, pts[0].y, pts[3].y, reverse); return; }
        if (pts[0].x >= clip.r) {
            if (!can_cull_right) append_vline(clip.r, pts[0].y, pts[3].y, reverse);
            return;
        }
        if (pts[0].x < clip.l) {
            Point tmp[7];
            chop_mono_cubic_at(pts, clip.l, false, tmp);
            append_vline(clip.l, tmp[0].y, tmp[3].y, reverse);
            tmp[3].x = clip.l;
            tmp[4].x = std::max(tmp[4].x, clip.l);
            pts[0] = tmp[3]; pts[1] = tmp[4]; pts[2] = tmp[5];
        }
        if (pts[3].x > clip.r) {
            Point tmp[7];
            chop_mono_cubic_at(pts, clip.r, false, tmp);
            tmp[3].x = clip.r;
            tmp[2].x = std::min(tmp[2].x, clip.r);
            append_cubic(tmp, reverse);
            append_vline(clip.r, tmp[3].y, tmp[6].y, reverse);
        } else {
            append_cubic(pts, reverse);
        }
    }
    static bool too_big_for_reliable_float_math(float l, float t, float r, float b) {
        const float limit = (float)(1 << 22);
        return l < -limit || t < -limit || r > limit || b > limit;
    }
    void clip_cubic(const Point *p) {
        float l = std::min({p[0].x, p[1].x, p[2].x, p[3].x}), r = std::max({p[0].x, p[1].x, p[2].x, p[3].x});
        float t = std::min({p[0].y, p[1].y, p[2].y, p[3].y}), b = std::max({p[0].y, p[1].y, p[2].y, p[3].y});
        if (!(b > clip.t && t < clip.b)) return;
        if (too_big_for_reliable_float_math(l, t, r, b)) { clip_line(p[0], p[3]); return; }
        Point mono_y[10];
        int ny = chop_cubic_at_y_extrema(p, mono_y);
        for (int y = 0; y <= ny; y++) {
            Point mono_x[10];
            int nx = chop_cubic_at_x_extrema(&mono_y[y * 3], mono_x);
            for (int x = 0; x <= nx; x++) clip_mono_cubic(&mono_x[x * 3]);
        }
    }
};

// ---------------------------------------------------------------- path edge iterator (path.rs PathEdgeIter)
template <class F>
static void for_each_path_edge(const Path &path, F &&f) {
    size_t pi = 0;
    Point move_to{0, 0};
    bool needs_close = false;
    for (size_t vi = 0; vi < path.verbs.size(); vi++) {
        uint8_t v = path.verbs[vi];
        switch (v) {
        case RGPU_MOVE:
            if (needs_close) { Point s[2] = {path.pts[pi - 1], move_to}; f(SEG_LINE, s); needs_close = false; }
            move_to = path.pts[pi]; pi += 1;
            break;
        case RGPU_CLOSE:
            if (needs_close) { Point s[2] = {path.pts[pi - 1], move_to}; f(SEG_LINE, s); needs_close = false; }
            break;
        case RGPU_LINE: { needs_close = true; Point s[2] = {path.pts[pi - 1], path.pts[pi]}; pi += 1; f(SEG_LINE, s); break; }
        case RGPU_QUAD: { needs_close = true; Point s[3] = {path.pts[pi - 1], path.pts[pi], path.pts[pi + 1]}; pi += 2; f(SEG_QUAD, s); break; }
        case RGPU_CUBIC: { needs_close = true; Point s[4] = {path.pts[pi - 1], path.pts[pi], path.pts[pi + 1], path.pts[pi + 2]}; pi += 3; f(SEG_CUBIC, s); break; }
        }
    }
    if (needs_close) { Point s[2] = {path.pts[pi - 1], move_to}; f(SEG_LINE, s); }
}

// ---------------------------------------------------------------- edge builder (edge_builder.rs)
enum Combine { COMBINE_NO, COMBINE_PARTIAL, COMBINE_TOTAL };
static Combine combine_vertical(const Edge &edge, Edge &last) {
    if (last.dx != 0 || edge.x != last.x) return COMBINE_NO;
    if (edge.winding == last.winding) {
        if (edge.last_y + 1 == last.first_y) { last.first_y = edge.first_y; return COMBINE_PARTIAL; }
        if (edge.first_y == last.last_y + 1) { last.last_y = edge.last_y; return COMBINE_PARTIAL; }
        return COMBINE_NO;
    }
    if (edge.first_y == last.first_y) {
        if (edge.last_y == last.last_y) return COMBINE_TOTAL;
        if (edge.last_y < last.last_y) { last.first_y = edge.last_y + 1; return COMBINE_PARTIAL; }
        last.first_y = last.last_y + 1;
        last.last_y = edge.last_y;
        last.winding = edge.winding;
        return COMBINE_PARTIAL;
    }
    if (edge.last_y == last.last_y) {
        if (edge.first_y > last.first_y) {
            last.last_y = edge.first_y - 1;
        } else {
            last.last_y = last.first_y - 1;
            last.first_y = edge.first_y;
            last.winding = edge.winding;
        }
        return COMBINE_PARTIAL;
    }
    return COMBINE_NO;
}
struct EdgeBuilder {
    int shift;
    std::vector<Edge> edges;
    void push_line(const Point *p) {
        Edge e;
        if (!line_new(p[0], p[1], shift, e)) return;
        Combine c = COMBINE_NO;
        if (e.dx == 0 && !edges.empty() && edges.back().type == EDGE_LINE) c = combine_vertical(e, edges.back());
        if (c == COMBINE_TOTAL) edges.pop_back();
        else if (c == COMBINE_NO) edges.push_back(e);
    }
    void push_quad(const Point *p) { Edge e; if (quad_new(p, shift, e)) edges.push_back(e); }
    void push_cubic(const Point *p) { Edge e; if (cubic_new(p, shift, e)) edges.push_back(e); }
    bool build(const Path &path, const Rect *clip) {
        bool ok = true;
        if (clip) {
            EdgeClipper clipper{*clip, false, {}};
            for_each_path_edge(path, [&](int kind, const Point *p) {
                clipper.out.clear();
                if (kind == SEG_LINE) clipper.clip_line(p[0], p[1]);
                else if (kind == SEG_QUAD) clipper.clip_quad(p);
                else clipper.clip_cubic(p);
                for (auto &s : clipper.out) {
                    for (int i = 0; i <= s.kind; i++)
                        if (!std::isfinite(s.p[i].x) || !std::isfinite(s.p[i].y)) ok = false;
                    if (!ok) return;
                    if (s.kind == SEG_LINE) push_line(s.p);
                    else if (s.kind == SEG_QUAD) push_quad(s.p);
                    else push_cubic(s.p);
                }
            });
        } else {
            for_each_path_edge(path, [&](int kind, const Point *p) {
                if (kind == SEG_LINE) {
                    push_line(p);
                } else if (kind == SEG_QUAD) {
                    Point mono[5];
                    int n = chop_quad_at_y_extrema(p, mono);
                    for (int i = 0; i <= n; i++) push_quad(&mono[i * 2]);
                } else {
                    Point mono[10];
                    int n = chop_cubic_at_y_extrema(p, mono);
                    for (int i = 0; i <= n; i++) push_cubic(&mono[i * 3]);
                }
            });
        }
        return ok;
    }
};

// ---------------------------------------------------------------- scan conversion (scan/path.rs)
struct SpanSink {
    virtual void blit_h(int32_t x, int32_t y, int32_t width) = 0;
    virtual ~SpanSink() {}
};

static void backward_insert_edge_based_on_x(std::vector<Edge> &E, int edge) {
    FDot16 x = E[edge].x;
    int prev = E[edge].prev;
    while (E[prev].prev != -1 && E[prev].x > x) prev = E[prev].prev;
    if (E[prev].next != edge) {
        // remove edge
        E[E[edge].prev].next = E[edge].next;
        E[E[edge].next].prev = E[edge].prev;
        // insert after prev
        E[edge].prev = prev;
        E[edge].next = E[prev].next;
        E[E[prev].next].prev = edge;
        E[prev].next = edge;
    }
}
static void insert_edge_after(std::vector<Edge> &E, int edge, int after) {
    E[edge].prev = after;
    E[edge].next = E[after].next;
    E[E[after].next].prev = edge;
    E[after].next = edge;
}
static void backward_insert_start(std::vector<Edge> &E, int prev, FDot16 x, int *out) {
    while (E[prev].prev != -1 && E[prev].x > x) prev = E[prev].prev;
    *out = prev;
}
static void insert_new_edges(std::vector<Edge> &E, int new_edge, int32_t curr_y) {
    if (E[new_edge].first_y != curr_y) return;
    int prev = E[new_edge].prev;
    if (E[prev].x <= E[new_edge].x) return;
    // find first x pos to insert
    int start;
    backward_insert_start(E, prev, E[new_edge].x, &start);
    // insert the lot, fixing up the links as we go
    do {
        int next = E[new_edge].next;
        bool keep = false;
        for (;;) {
            if (E[start].next == new_edge) { keep = true; break; }
            int after = E[start].next;
            if (E[after].x >= E[new_edge].x) break;
            start = after;
        }
        if (!keep) {
            // remove new_edge
            E[E[new_edge].prev].next = E[new_edge].next;
            E[E[new_edge].next].prev = E[new_edge].prev;
            insert_edge_after(E, new_edge, start);
        }
        start = new_edge;
        new_edge = next;
    } while (E[new_edge].first_y == curr_y);
}
static void remove_edge(std::vector<Edge> &E, int e) {
    E[E[e].prev].next = E[e].next;
    E[E[e].next].prev = E[e].prev;
}
static void walk_edges(uint32_t rule, int32_t start_y, int32_t stop_y, int32_t right_clip, std::vector<Edge> &E,
                       SpanSink &blitter) {
    int32_t curr_y = start_y;
    int32_t winding_mask = rule == RGPU_EVENODD ? 1 : -1;
    for (;;) {
        int32_t w = 0;
        int32_t left = 0;
        int prev_x_e = 0;  // head
        FDot16 prev_x = E[prev_x_e].x;
        int curr_e = E[0].next;
        while (E[curr_e].first_y <= curr_y) {
            int32_t x = fdot16_round_to_i32(E[curr_e].x);
            if ((w & winding_mask) == 0) left = x;
            w += E[curr_e].winding;
            if ((w & winding_mask) == 0) {
                int32_t width = x - left;
                if (width > 0) blitter.blit_h(left, curr_y, width);
            }
            int next = E[curr_e].next;
            FDot16 new_x;
            bool advance = false;
            if (E[curr_e].last_y == curr_y) {
                bool updated = false;
                if (E[curr_e].type == EDGE_QUAD && E[curr_e].curve_count > 0) updated = quad_update(E[curr_e]);
                else if (E[curr_e].type == EDGE_CUBIC && E[curr_e].curve_count < 0) updated = cubic_update(E[curr_e]);
                if (updated) { new_x = E[curr_e].x; advance = true; }
                else remove_edge(E, curr_e);
            } else {
                new_x = wadd(E[curr_e].x, E[curr_e].dx);
                E[curr_e].x = new_x;
                advance = true;
            }
            if (advance) {
                if (new_x < prev_x) backward_insert_edge_based_on_x(E, curr_e);
                else prev_x = new_x;
            }
            curr_e = next;
        }
        if ((w & winding_mask) != 0) {
            int32_t width = right_clip - left;
            if (width > 0) blitter.blit_h(left, curr_y, width);
        }
        curr_y += 1;
        if (curr_y >= stop_y) break;
        insert_new_edges(E, curr_e, curr_y);
    }
}

// Shared setup of scan/path.rs fill_path_impl: edges sorted and linked.
static bool prepare_edges(const Path &path, const IntRect &clip, int shift, bool contained,
                          std::vector<Edge> &E) {
    EdgeBuilder b{shift, {}};
    Rect shifted{(float)(clip.x << shift), (float)(clip.y << shift), (float)(clip.right() << shift),
                 (float)(clip.bottom() << shift)};
    // tiny-skia passes the shifted clip recovered to a float rect; the path is
    // built with points scaled by 2^shift inside the edge constructors, so the
    // clip is applied in unshifted space.
    Rect unshifted{(float)clip.x, (float)clip.y, (float)clip.right(), (float)clip.bottom()};
    (void)shifted;
    if (!b.build(path, contained ? nullptr : &unshifted)) return false;
    if (b.edges.size() < 2) return false;
    std::stable_sort(b.edges.begin(), b.edges.end(), [](const Edge &a, const Edge &c) {
        if (a.first_y != c.first_y) return a.first_y < c.first_y;
        return a.x < c.x;
    });
    E.clear();
    E.reserve(b.edges.size() + 2);
    Edge head; head.first_y = INT32_MIN; head.x = INT32_MIN; head.prev = -1; head.next = 1;
    E.push_back(head);
    for (size_t i = 0; i < b.edges.size(); i++) {
        Edge e = b.edges[i];
        e.prev = (int)i;
        e.next = (int)i + 2;
        E.push_back(e);
    }
    Edge tail; tail.first_y = INT32_MAX; tail.x = INT32_MAX; tail.prev = (int)b.edges.size(); tail.next = -1;
    E.push_back(tail);
    return true;
}

// ---------------------------------------------------------------- AA: SuperBlitter (scan/path_aa.rs)
static const int SHIFT = 2;
static const int SCALE = 1 << SHIFT;
static const int MASK = SCALE - 1;

template <class F>
struct SuperBlitter : SpanSink {
    int32_t left, width, super_left;
    int32_t curr_iy;
    std::vector<uint8_t> row;
    F *pixel;
    void flush() {
        if (curr_iy < 0) return;
        for (int32_t x = 0; x < width; x++) {
            uint8_t c = row[x];
            if (c) (*pixel)(left + x, curr_iy, c);
            row[x] = 0;
        }
    }
    void blit_h(int32_t x, int32_t y, int32_t w) override {
        int32_t iy = y >> SHIFT;
        x -= super_left;
        if (x < 0) { w += x; x = 0; }
        if (w <= 0) return;
        if (iy != curr_iy) { flush(); curr_iy = iy; }
        int32_t start = x, stop = x + w;
        int32_t fb = start & MASK, fe = stop & MASK;
        int32_t n = (stop >> SHIFT) - (start >> SHIFT) - 1;
        if (n < 0) { fb = fe - fb; n = 0; fe = 0; }
        else if (fb == 0) n += 1;
        else fb = SCALE - fb;
        int32_t max_value = (1 << (8 - SHIFT)) - (((y & MASK) + 1) >> SHIFT);
        int32_t px = start >> SHIFT;
        int32_t start_alpha = fb << (8 - 2 * SHIFT), stop_alpha = fe << (8 - 2 * SHIFT);
        if (start_alpha) {
            if (px < width) { uint32_t tmp = row[px] + start_alpha; row[px] = (uint8_t)(tmp - (tmp >> 8)); }
            px += 1;
        }
        for (int32_t i = 0; i < n; i++, px++) {
            if (px < width) { uint32_t tmp = row[px] + max_value; row[px] = (uint8_t)(tmp - (tmp >> 8)); }
        }
        if (stop_alpha) {
            if (px < width) row[px] = (uint8_t)(row[px] + stop_alpha);
        }
    }
};

struct NonAABlitter : SpanSink {
    std::vector<std::pair<int32_t, std::pair<int32_t, int32_t>>> spans;  // y, (x, w)
    void blit_h(int32_t x, int32_t y, int32_t w) override { spans.push_back({y, {x, w}}); }
};

// Pixel callback: coverage in 1..255 (255 = full).
typedef void (*PixelFn)(void *ctx, int32_t x, int32_t y, uint8_t cov);

// Path scan (AA or not) -> per-pixel coverage callbacks, following
// scan/path_aa.rs::fill_path and scan/path.rs::fill_path.
template <class F>
static void scan_path(const Path &path, uint32_t rule, bool aa, const IntRect &clip, F &&pixel) {
    if (aa) {
        Rect rb{std::floor(path.bounds.l), std::floor(path.bounds.t), std::ceil(path.bounds.r),
                std::ceil(path.bounds.b)};
        IntRect ir{sat_i32(rb.l), sat_i32(rb.t), std::max(1, sat_i32(rb.r - rb.l)), std::max(1, sat_i32(rb.b - rb.t))};
        // intersect with clip
        int32_t l = std::max(ir.x, clip.x), t = std::max(ir.y, clip.y);
        int32_t r = std::min(ir.right(), clip.right()), b = std::min(ir.bottom(), clip.bottom());
        if (r <= l || b <= t) return;
        {
            // rect_overflows_short_shift: supersampled coords must fit in i16
            auto ovf = [](int32_t v) { return v > (32767 >> SHIFT) || v < -(32768 >> SHIFT); };
            if (ovf(l) || ovf(t) || ovf(r) || ovf(b)) { scan_path(path, rule, false, clip, pixel); return; }
        }
        if (clip.right() > 32767 || clip.bottom() > 32767) return;
        bool contained = ir.x >= 0 && ir.y >= 0 && ir.x >= clip.x && ir.y >= clip.y &&
                         ir.right() <= clip.right() && ir.bottom() <= clip.bottom();
        std::vector<Edge> E;
        if (!prepare_edges(path, clip, SHIFT, contained, E)) return;
        SuperBlitter<typename std::remove_reference<F>::type> sb;
        sb.left = l; sb.width = r - l; sb.super_left = l << SHIFT; sb.curr_iy = -1;
        sb.row.assign((size_t)sb.width, 0);
        sb.pixel = &pixel;
        int32_t start_y = ir.y << SHIFT, stop_y = ir.bottom() << SHIFT;
        if (!contained) {
            start_y = std::max(start_y, clip.y << SHIFT);
            stop_y = std::min(stop_y, clip.bottom() << SHIFT);
        }
        walk_edges(rule, start_y, stop_y, clip.right() << SHIFT, E, sb);
        sb.flush();
    } else {
        const double bias = 0.5 + 1.5 / 64.0;
        int32_t l = sat_i32d(std::ceil((double)path.bounds.l - bias));
        int32_t t = sat_i32d(std::ceil((double)path.bounds.t - bias));
        int32_t r = sat_i32d(std::floor((double)path.bounds.r + bias));
        int32_t b = sat_i32d(std::floor((double)path.bounds.b + bias));
        if (r <= l || b <= t) return;
        bool contained = l >= 0 && t >= 0 && l >= clip.x && t >= clip.y && r <= clip.right() && b <= clip.bottom();
        std::vector<Edge> E;
        if (!prepare_edges(path, clip, 0, contained, E)) return;
        int32_t start_y = t, stop_y = b;
        if (!contained) { start_y = std::max(start_y, clip.y); stop_y = std::min(stop_y, clip.bottom()); }
        if (start_y >= stop_y) return;
        NonAABlitter nb;
        walk_edges(rule, start_y, stop_y, clip.right(), E, nb);
        for (auto &s : nb.spans) {
            int32_t y = s.first, x = s.second.first, w = s.second.second;
            if (y < clip.y || y >= clip.bottom()) continue;
            for (int32_t i = 0; i < w; i++) {
                int32_t xx = x + i;
                if (xx < clip.x || xx >= clip.right()) continue;
                pixel(xx, y, (uint8_t)255);
            }
        }
    }
}

// ---------------------------------------------------------------- shaders & pipelines
bool Shader::is_opaque() const {
    switch (kind) {
    case SHADER_SOLID: return color.a == 1.0f;
    case SHADER_LINEAR:
    case SHADER_RADIAL:
        for (auto &s : stops) if (s.color.a != 1.0f) return false;
        return true;
    default: return false;
    }
}
static ColorF premultiply(ColorF c) {
    if (c.a == 1.0f) return c;
    auto cl = [](float v) { return std::min(std::max(v, 0.0f), 1.0f); };
    return ColorF{cl(c.r * c.a), cl(c.g * c.a), cl(c.b * c.a), c.a};
}
static inline uint8_t f32_to_u8_round(float v) { return sat_u8(v * 255.0f + 0.5f); }

// lowp helpers (u16 lanes, wrapping)
static inline uint16_t div255(uint16_t v) { return (uint16_t)((uint16_t)(v + 255) >> 8); }
static inline uint16_t inv(uint16_t v) { return (uint16_t)(255 - v); }
static inline uint16_t lerp16(uint16_t from, uint16_t to, uint16_t t) {
    return div255((uint16_t)(from * inv(t) + to * t));
}
// highp store: clamp to [0,1], * 255, round to nearest even.
static inline uint8_t unnorm(float v) {
    v = std::max(v, 0.0f);
    v = std::min(v, 1.0f);
    return (uint8_t)std::nearbyint(v * 255.0f);
}
static const float INV255 = 1.0f / 255.0f;

// --- gradient (gradient.rs / linear_gradient.rs / radial_gradient.rs)
struct GradientCtx {
    std::vector<ColorF> factors, biases;
    std::vector<float> t_values;
    bool two_stop = false;
    ColorF f2{0, 0, 0, 0}, b2{0, 0, 0, 0};
    bool pad_clamp = false;
    bool premul = false;
    Transform ts;  // device -> unit space
    bool radial_simple = false;
    bool radial_conical = false;
    // conical in unit space where the focal circle centre is at origin
    float fr0 = 0, fr1 = 0, cdx = 0, cdy = 0;  // radii and centre delta
    bool valid = true;
};

static bool build_gradient(const Shader &sh, GradientCtx &g) {
    std::vector<GradientStop> stops = sh.stops;
    if (stops.size() < 2) return false;
    bool dummy_first = stops[0].pos != 0.0f;
    bool dummy_last = stops.back().pos != 1.0f;
    if (dummy_first) stops.insert(stops.begin(), GradientStop{0.0f, stops[0].color});
    if (dummy_last) stops.push_back(GradientStop{1.0f, stops.back().color});
    bool opaque = true;
    for (auto &s : stops) if (s.color.a != 1.0f) opaque = false;
    size_t start_index = dummy_first ? 0 : 1;
    float prev = 0.0f;
    bool uniform = true;
    float uniform_step = stops[start_index].pos - prev;
    for (size_t i = start_index; i < stops.size(); i++) {
        float curr;
        if (i + 1 == stops.size()) curr = 1.0f;
        else {
            float v = stops[i].pos;
            curr = v > 1.0f ? 1.0f : (v >= prev ? v : prev);
        }
        uniform = uniform && std::fabs(uniform_step - (curr - prev)) <= SCALAR_NEARLY_ZERO;
        stops[i].pos = std::min(std::max(curr, 0.0f), 1.0f);
        prev = curr;
    }
    g.premul = !opaque;
    if (sh.spread == RGPU_SPREAD_PAD && uniform) g.pad_clamp = true;
    if (stops.size() == 2) {
        ColorF c0 = stops[0].color, c1 = stops[1].color;
        g.two_stop = true;
        g.f2 = ColorF{c1.r - c0.r, c1.g - c0.g, c1.b - c0.b, c1.a - c0.a};
        g.b2 = c0;
    } else {
        size_t first_stop = 0, last_stop = 1;
        if (stops.size() > 2) {
            auto eq = [](ColorF a, ColorF b) { return a.r == b.r && a.g == b.g && a.b == b.b && a.a == b.a; };
            first_stop = eq(stops[0].color, stops[1].color) ? 1 : 0;
            last_stop = eq(stops.back().color, stops[stops.size() - 2].color) ? stops.size() - 2 : stops.size() - 1;
        }
        float t_l = stops[first_stop].pos;
        ColorF c_l = stops[first_stop].color;
        g.factors.push_back(ColorF{0, 0, 0, 0}); g.biases.push_back(c_l); g.t_values.push_back(0.0f);
        for (size_t i = first_stop; i < last_stop; i++) {
            float t_r = stops[i + 1].pos;
            ColorF c_r = stops[i + 1].color;
            if (t_l < t_r) {
                float d = t_r - t_l;
                ColorF f{(c_r.r - c_l.r) / d, (c_r.g - c_l.g) / d, (c_r.b - c_l.b) / d, (c_r.a - c_l.a) / d};
                g.factors.push_back(f);
                g.biases.push_back(ColorF{c_l.r - f.r * t_l, c_l.g - f.g * t_l, c_l.b - f.b * t_l, c_l.a - f.a * t_l});
                g.t_values.push_back(std::min(std::max(t_l, 0.0f), 1.0f));
            }
            t_l = t_r;
            c_l = c_r;
        }
        g.factors.push_back(ColorF{0, 0, 0, 0}); g.biases.push_back(c_l);
        g.t_values.push_back(std::min(std::max(t_l, 0.0f), 1.0f));
    }
    return true;
}

// Build the shader context for a gradient; `paint_ts` is the transform the
// shader was given by fill_path (gradientTransform already concatenated).
static bool gradient_setup(const Shader &sh, GradientCtx &g) {
    if (!build_gradient(sh, g)) return false;
    Transform inv;
    if (!sh.transform.invert(&inv)) return false;
    Transform unit;
    if (sh.kind == SHADER_LINEAR) {
        float vx = sh.p1.x - sh.p0.x, vy = sh.p1.y - sh.p0.y;
        float mag = std::sqrt(vx * vx + vy * vy);
        float invm = mag != 0.0f ? 1.0f / mag : 0.0f;
        vx *= invm; vy *= invm;
        float sinv = -vy, cosv = vx;
        float cos_inv = 1.0f - cosv;
        float px = sh.p0.x, py = sh.p0.y;
        unit = Transform::from_row(cosv, sinv, -sinv, cosv, sinv * py + cos_inv * px, -sinv * px + cos_inv * py);
        unit = unit.post_concat(Transform::translate(-sh.p0.x, -sh.p0.y));
        unit = unit.post_concat(Transform::scale(invm, invm));
    } else {
        // radial: unit space centred on the focal point, scaled by the end radius
        float r1 = sh.r1;
        if (!(r1 > 0)) return false;
        float inv_r = 1.0f / r1;
        unit = Transform::translate(-sh.p0.x, -sh.p0.y).post_concat(Transform::scale(inv_r, inv_r));
        bool concentric = sh.p0.x == sh.p1.x && sh.p0.y == sh.p1.y;
        if (concentric && sh.r0 == 0.0f) {
            g.radial_simple = true;
        } else {
            g.radial_conical = true;
            g.fr0 = sh.r0 * inv_r;
            g.fr1 = 1.0f;
            g.cdx = (sh.p1.x - sh.p0.x) * inv_r;
            g.cdy = (sh.p1.y - sh.p0.y) * inv_r;
        }
    }
    g.ts = inv.post_concat(unit);
    return true;
}

// Evaluate a gradient at device pixel (x, y): premultiplied f32 colour.
// Returns false when the pixel is masked out (degenerate conical region).
static bool gradient_eval(const GradientCtx &g, uint32_t spread, int32_t px, int32_t py, ColorF *out,
                          bool premul_stage = true) {
    float x = (float)px + 0.5f, y = (float)py + 0.5f;
    const Transform &ts = g.ts;
    float tx = x * ts.sx + y * ts.kx + ts.tx;
    float ty = x * ts.ky + y * ts.sy + ts.ty;
    float t;
    if (g.radial_simple) {
        t = std::sqrt(tx * tx + ty * ty);
    } else if (g.radial_conical) {
        // largest t with |p - t*cd| = r0 + t*(r1 - r0), r(t) >= 0
        float dr = g.fr1 - g.fr0;
        float a = g.cdx * g.cdx + g.cdy * g.cdy - dr * dr;
        float b = tx * g.cdx + ty * g.cdy + g.fr0 * dr;
        float c = tx * tx + ty * ty - g.fr0 * g.fr0;
        if (a == 0.0f) {
            if (b == 0.0f) return false;
            t = c / (2.0f * b);
            if (g.fr0 + t * dr < 0.0f) return false;
        } else {
            float disc = b * b - a * c;
            if (disc < 0.0f) return false;
            float s = std::sqrt(disc);
            float t1 = (b + s) / a, t2 = (b - s) / a;
            float hi = std::max(t1, t2), lo = std::min(t1, t2);
            if (g.fr0 + hi * dr >= 0.0f) t = hi;
            else if (g.fr0 + lo * dr >= 0.0f) t = lo;
            else return false;
        }
    } else {
        t = tx;
    }
    if (spread == RGPU_SPREAD_REFLECT) {
        float u = t - 1.0f;
        t = std::fabs(u - 2.0f * std::floor(u * 0.5f) - 1.0f);
        t = std::min(std::max(t, 0.0f), 1.0f);
    } else if (spread == RGPU_SPREAD_REPEAT) {
        t = t - std::floor(t);
        t = std::min(std::max(t, 0.0f), 1.0f);
    } else if (g.pad_clamp) {
        t = std::min(std::max(t, 0.0f), 1.0f);
    }
    ColorF c;
    if (g.two_stop) {
        c = ColorF{t * g.f2.r + g.b2.r, t * g.f2.g + g.b2.g, t * g.f2.b + g.b2.b, t * g.f2.a + g.b2.a};
    } else {
        size_t idx = 0;
        for (size_t i = 1; i < g.t_values.size(); i++)
            if (t >= g.t_values[i]) idx++;
        const ColorF &f = g.factors[idx], &b = g.biases[idx];
        c = ColorF{t * f.r + b.r, t * f.g + b.g, t * f.b + b.b, t * f.a + b.a};
    }
    if (g.premul && premul_stage) { c.r *= c.a; c.g *= c.a; c.b *= c.a; }
    *out = c;
    return true;
}

// lowp gradient colour (pipeline/lowp.rs): the f32 stop interpolation is
// clamped, rounded to u16 by truncating v * 255 + 0.5, and premultiplied
// with div255 when the stops are not opaque.  Linear and simple radial
// gradients only (the two-point conical stages exist in highp alone).
static void gradient_eval_lowp(const GradientCtx &g, uint32_t spread, int32_t px, int32_t py, uint16_t out[4]) {
    ColorF c;
    gradient_eval(g, spread, px, py, &c, false);
    float v[4] = {c.r, c.g, c.b, c.a};
    for (int i = 0; i < 4; i++) {
        float x = std::min(std::max(v[i], 0.0f), 1.0f) * 255.0f + 0.5f;
        out[i] = (uint16_t)x;
    }
    if (g.premul)
        for (int i = 0; i < 3; i++) out[i] = (uint16_t)(((uint32_t)out[i] * out[3] + 255) >> 8);
}

// highp blend (pipeline/highp.rs).  s/d are premultiplied f32.
static inline float hinv(float v) { return 1.0f - v; }
static void blend_sep(uint32_t mode, const float s[4], const float d[4], float o[4]) {
    float sa = s[3], da = d[3];
    auto all = [&](auto f) { for (int i = 0; i < 4; i++) o[i] = f(s[i], d[i]); };
    auto rgb = [&](auto f) {
        for (int i = 0; i < 3; i++) o[i] = f(s[i], d[i]);
        o[3] = sa + da * hinv(sa);
    };
    switch (mode) {
    case RGPU_BLEND_CLEAR: all([](float, float) { return 0.0f; }); break;
    case RGPU_BLEND_SOURCE: all([](float s_, float) { return s_; }); break;
    case RGPU_BLEND_DESTINATION: all([](float, float d_) { return d_; }); break;
    case RGPU_BLEND_SOURCE_OVER: all([&](float s_, float d_) { return d_ * hinv(sa) + s_; }); break;
    case RGPU_BLEND_DESTINATION_OVER: all([&](float s_, float d_) { return s_ * hinv(da) + d_; }); break;
    case RGPU_BLEND_SOURCE_IN: all([&](float s_, float) { return s_ * da; }); break;
    case RGPU_BLEND_DESTINATION_IN: all([&](float, float d_) { return d_ * sa; }); break;
    case RGPU_BLEND_SOURCE_OUT: all([&](float s_, float) { return s_ * hinv(da); }); break;
    case RGPU_BLEND_DESTINATION_OUT: all([&](float, float d_) { return d_ * hinv(sa); }); break;
    case RGPU_BLEND_SOURCE_ATOP: all([&](float s_, float d_) { return s_ * da + d_ * hinv(sa); }); break;
    case RGPU_BLEND_DESTINATION_ATOP: all([&](float s_, float d_) { return d_ * sa + s_ * hinv(da); }); break;
    case RGPU_BLEND_XOR: all([&](float s_, float d_) { return s_ * hinv(da) + d_ * hinv(sa); }); break;
    case RGPU_BLEND_PLUS: all([](float s_, float d_) { return std::min(s_ + d_, 1.0f); }); break;
    case RGPU_BLEND_MODULATE: all([](float s_, float d_) { return s_ * d_; }); break;
    case RGPU_BLEND_SCREEN: all([](float s_, float d_) { return s_ + d_ - s_ * d_; }); break;
    case RGPU_BLEND_MULTIPLY: all([&](float s_, float d_) { return s_ * hinv(da) + d_ * hinv(sa) + s_ * d_; }); break;
    case RGPU_BLEND_DARKEN: rgb([&](float s_, float d_) { return s_ + d_ - std::max(s_ * da, d_ * sa); }); break;
    case RGPU_BLEND_LIGHTEN: rgb([&](float s_, float d_) { return s_ + d_ - std::min(s_ * da, d_ * sa); }); break;
    case RGPU_BLEND_DIFFERENCE:
        rgb([&](float s_, float d_) { float m = std::min(s_ * da, d_ * sa); return s_ + d_ - (m + m); }); break;
    case RGPU_BLEND_EXCLUSION: rgb([&](float s_, float d_) { float m = s_ * d_; return s_ + d_ - (m + m); }); break;
    case RGPU_BLEND_COLOR_BURN:
        rgb([&](float s_, float d_) {
            if (d_ == da) return d_ + s_ * hinv(da);
            if (s_ == 0.0f) return d_ * hinv(sa);
            return sa * (da - std::min(da, (da - d_) * sa * (1.0f / s_))) + s_ * hinv(da) + d_ * hinv(sa);
        });
        break;
    case RGPU_BLEND_COLOR_DODGE:
        rgb([&](float s_, float d_) {
            if (d_ == 0.0f) return s_ * hinv(da);
            if (s_ == sa) return s_ + d_ * hinv(sa);
            return sa * std::min(da, (d_ * sa) * (1.0f / (sa - s_))) + s_ * hinv(da) + d_ * hinv(sa);
        });
        break;
    case RGPU_BLEND_HARD_LIGHT:
        rgb([&](float s_, float d_) {
            float x = (s_ + s_ <= sa) ? (s_ * d_) + (s_ * d_) : sa * da - 2.0f * ((da - d_) * (sa - s_));
            return s_ * hinv(da) + d_ * hinv(sa) + x;
        });
        break;
    case RGPU_BLEND_OVERLAY:
        rgb([&](float s_, float d_) {
            float x = (d_ + d_ <= da) ? (s_ * d_) + (s_ * d_) : sa * da - 2.0f * ((da - d_) * (sa - s_));
            return s_ * hinv(da) + d_ * hinv(sa) + x;
        });
        break;
    case RGPU_BLEND_SOFT_LIGHT:
        rgb([&](float s_, float d_) {
            float m = da > 0.0f ? d_ / da : 0.0f;
            float s2 = s_ + s_;
            float m4 = (m + m) + (m + m);
            float dark_src = d_ * (sa + (s2 - sa) * (1.0f - m));
            float dark_dst = (m4 * m4 + m4) * (m - 1.0f) + 7.0f * m;
            float lite_dst = std::sqrt(m) - m;
            float lite_src = d_ * sa + da * (s2 - sa) * ((d_ + d_) + (d_ + d_) <= da ? dark_dst : lite_dst);
            return s_ * hinv(da) + d_ * hinv(sa) + (s2 <= sa ? dark_src : lite_src);
        });
        break;
    default: {
        // non-separable: hue, saturation, color, luminosity (highp.rs)
        auto lum = [](float r, float g, float b) { return r * 0.30f + g * 0.59f + b * 0.11f; };
        auto sat = [](float r, float g, float b) { return std::max({r, g, b}) - std::min({r, g, b}); };
        auto set_sat = [&](float &r, float &g, float &b, float s_) {
            float mn = std::min({r, g, b}), mx = std::max({r, g, b});
            float sat_ = mx - mn;
            auto scale = [&](float c) { return sat_ == 0.0f ? 0.0f : (c - mn) * s_ / sat_; };
            r = scale(r); g = scale(g); b = scale(b);
        };
        auto set_lum = [&](float &r, float &g, float &b, float l) {
            float diff = l - lum(r, g, b);
            r += diff; g += diff; b += diff;
        };
        // pulls channels above `a` towards the luminance and clamps negatives
        // to zero; there is no separate pull-up of a negative minimum (pinned
        // against resvg's mix-blend-mode goldens).
        auto clip_color = [&](float &r, float &g, float &b, float a) {
            float mx = std::max({r, g, b});
            float l = lum(r, g, b);
            auto clip = [&](float c) {
                if (mx > a && mx - l != 0.0f) c = l + (c - l) * (a - l) / (mx - l);
                return std::max(c, 0.0f);
            };
            r = clip(r); g = clip(g); b = clip(b);
        };
        float r, g, b;
        if (mode == RGPU_BLEND_HUE) {
            r = s[0] * sa; g = s[1] * sa; b = s[2] * sa;
            set_sat(r, g, b, sat(d[0], d[1], d[2]) * sa);
            set_lum(r, g, b, lum(d[0], d[1], d[2]) * sa);
            clip_color(r, g, b, sa * da);
        } else if (mode == RGPU_BLEND_SATURATION) {
            r = d[0] * sa; g = d[1] * sa; b = d[2] * sa;
            set_sat(r, g, b, sat(s[0], s[1], s[2]) * da);
            set_lum(r, g, b, lum(d[0], d[1], d[2]) * sa);
            clip_color(r, g, b, sa * da);
        } else if (mode == RGPU_BLEND_COLOR) {
            r = s[0] * da; g = s[1] * da; b = s[2] * da;
            set_lum(r, g, b, lum(d[0], d[1], d[2]) * sa);
            clip_color(r, g, b, sa * da);
        } else {  // luminosity
            r = d[0] * sa; g = d[1] * sa; b = d[2] * sa;
            set_lum(r, g, b, lum(s[0], s[1], s[2]) * da);
            clip_color(r, g, b, sa * da);
        }
        o[0] = r + d[0] * hinv(sa) + s[0] * hinv(da);
        o[1] = g + d[1] * hinv(sa) + s[1] * hinv(da);
        o[2] = b + d[2] * hinv(sa) + s[2] * hinv(da);
        o[3] = sa + da - sa * da;
    }
    }
}

// The blitter restated: RasterPipelineBlitter::new + blit_h / blit_anti_h.
// tiny-skia's Pattern shader (shaders/pattern.rs) in the highp pipeline:
// seed_shader (pixel centre), the inverse transform, then either nearest
// (repeat, gather) or bicubic (4x4 taps, each tiled with repeat and gathered,
// weights 1/18 * (1 + 9t + 27t^2 - 21t^3) and t^2 (7t - 6) / 18), clamp_0,
// clamp_a, and the opacity scale.
static inline float ulp_below(float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    b -= 1;
    std::memcpy(&v, &b, 4);
    return v;
}
static void pattern_gather(const Pixmap &pm, bool repeat, float x, float y, float c[4]) {
    const float w = (float)pm.width, h = (float)pm.height;
    if (repeat) {
        x = x - std::floor(x * (1.0f / w)) * w;
        y = y - std::floor(y * (1.0f / h)) * h;
    }
    x = std::min(std::max(x, 0.0f), ulp_below(w));
    y = std::min(std::max(y, 0.0f), ulp_below(h));
    const uint8_t *p = pm.px((uint32_t)x, (uint32_t)y);
    for (int i = 0; i < 4; i++) c[i] = (float)p[i] * (1.0f / 255.0f);
}
static inline float bicubic_near(float t) {
    return t * (t * ((-21.0f / 18.0f) * t + 27.0f / 18.0f) + 9.0f / 18.0f) + 1.0f / 18.0f;
}
static inline float bicubic_far(float t) { return (t * t) * ((7.0f / 18.0f) * t + (-6.0f / 18.0f)); }
static void pattern_eval(const Shader &sh, const Transform &inv, int quality, int32_t x, int32_t y, float out[4]) {
    const bool rep = sh.spread == RGPU_SPREAD_REPEAT;
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    const float u = px * inv.sx + (py * inv.kx + inv.tx);
    const float v = px * inv.ky + (py * inv.sy + inv.ty);
    if (quality == 0) {
        pattern_gather(*sh.pattern, rep, u, v, out);
    } else if (quality == 1) {
        // bilinear: 2x2 taps at -0.5 / +0.5, weights 1 - f and f
        const float fx = (u + 0.5f) - std::floor(u + 0.5f), fy = (v + 0.5f) - std::floor(v + 0.5f);
        const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy};
        float acc[4] = {0, 0, 0, 0};
        float sy = v - 0.5f;
        for (int j = 0; j < 2; j++) {
            float sx = u - 0.5f;
            for (int i = 0; i < 2; i++) {
                float c[4];
                pattern_gather(*sh.pattern, rep, sx, sy, c);
                const float wgt = wx[i] * wy[j];
                for (int k = 0; k < 4; k++) acc[k] = wgt * c[k] + acc[k];
                sx += 1.0f;
            }
            sy += 1.0f;
        }
        for (int k = 0; k < 4; k++) out[k] = acc[k];
    } else {
        const float fx = (u + 0.5f) - std::floor(u + 0.5f), fy = (v + 0.5f) - std::floor(v + 0.5f);
        const float wx[4] = {bicubic_far(1.0f - fx), bicubic_near(1.0f - fx), bicubic_near(fx), bicubic_far(fx)};
        const float wy[4] = {bicubic_far(1.0f - fy), bicubic_near(1.0f - fy), bicubic_near(fy), bicubic_far(fy)};
        float acc[4] = {0, 0, 0, 0};
        float sy = v - 1.5f;
        for (int j = 0; j < 4; j++) {
            float sx = u - 1.5f;
            for (int i = 0; i < 4; i++) {
                float c[4];
                pattern_gather(*sh.pattern, rep, sx, sy, c);
                const float wgt = wx[i] * wy[j];
                for (int k = 0; k < 4; k++) acc[k] = wgt * c[k] + acc[k];
                sx += 1.0f;
            }
            sy += 1.0f;
        }
        for (int k = 0; k < 4; k++) acc[k] = std::max(acc[k], 0.0f);
        for (int k = 0; k < 3; k++) acc[k] = std::min(acc[k], acc[3]);
        for (int k = 0; k < 4; k++) out[k] = acc[k];
    }
    if (sh.opacity != 1.0f)
        for (int k = 0; k < 4; k++) out[k] = out[k] * sh.opacity;
}

struct PipelineBlitter {
    Pixmap *pm = nullptr;
    uint32_t blend;
    bool lowp;
    bool memset_ok = false;
    uint8_t memset_color[4];
    uint16_t rgba16[4];          // lowp uniform colour
    float colorf[4];             // highp uniform colour (premultiplied)
    const Shader *shader = nullptr;
    GradientCtx grad;
    Transform pinv;
    int pquality = 2;
    bool skip = false;

    bool setup(Pixmap &p, const Paint &paint) {
        pm = &p;
        blend = paint.blend;
        bool opaque = paint.shader.is_opaque();
        if (blend == RGPU_BLEND_DESTINATION) { skip = true; return false; }
        if (blend == RGPU_BLEND_DESTINATION_IN && opaque && paint.shader.kind == SHADER_SOLID) { skip = true; return false; }
        if (opaque && blend == RGPU_BLEND_SOURCE_OVER) blend = RGPU_BLEND_SOURCE;
        shader = &paint.shader;
        if (paint.shader.kind == SHADER_SOLID) {
            ColorF c = premultiply(paint.shader.color);
            float cf[4] = {c.r, c.g, c.b, c.a};
            for (int i = 0; i < 4; i++) {
                colorf[i] = cf[i];
                rgba16[i] = sat_u16(cf[i] * 255.0f + 0.5f);
                memset_color[i] = f32_to_u8_round(cf[i]);
            }
            if (blend == RGPU_BLEND_SOURCE) memset_ok = true;
        } else if (paint.shader.kind == SHADER_LINEAR || paint.shader.kind == SHADER_RADIAL) {
            if (!gradient_setup(paint.shader, grad)) { skip = true; return false; }
        } else if (paint.shader.kind == SHADER_PATTERN) {
            if (!paint.shader.pattern || !paint.shader.transform.invert(&pinv)) { skip = true; return false; }
            // a translation-only transform samples nearest (tiny-skia's quality downgrade)
            const bool translate = pinv.sx == 1.0f && pinv.sy == 1.0f && pinv.kx == 0.0f && pinv.ky == 0.0f;
            pquality = translate ? 0 : paint.shader.quality;
        }
        if (blend == RGPU_BLEND_CLEAR && !paint.anti_alias) {
            blend = RGPU_BLEND_SOURCE;
            memset_ok = true;
            memset_color[0] = memset_color[1] = memset_color[2] = memset_color[3] = 0;
        }
        // lowp is possible for a solid colour, a linear or a simple radial
        // gradient, with the blend modes resvg fills with.
        bool lowp_shader = paint.shader.kind == SHADER_SOLID || paint.shader.kind == SHADER_LINEAR ||
                           (paint.shader.kind == SHADER_RADIAL && grad.radial_simple);
        lowp = lowp_shader &&
               (blend == RGPU_BLEND_SOURCE || blend == RGPU_BLEND_SOURCE_OVER || blend == RGPU_BLEND_CLEAR ||
                blend == RGPU_BLEND_DESTINATION_OUT || blend == RGPU_BLEND_XOR || blend == RGPU_BLEND_SOURCE_ATOP ||
                blend == RGPU_BLEND_PLUS || blend == RGPU_BLEND_MODULATE || blend == RGPU_BLEND_SCREEN);
        return true;
    }
    bool pre_scale() const {
        return blend == RGPU_BLEND_DESTINATION || blend == RGPU_BLEND_DESTINATION_OVER || blend == RGPU_BLEND_PLUS ||
               blend == RGPU_BLEND_DESTINATION_OUT || blend == RGPU_BLEND_SOURCE_ATOP ||
               blend == RGPU_BLEND_SOURCE_OVER || blend == RGPU_BLEND_XOR;
    }
    void lowp_blend(uint16_t s[4], uint16_t d[4], uint16_t o[4]) {
        uint16_t sa = s[3];
        for (int i = 0; i < 4; i++) {
            switch (blend) {
            case RGPU_BLEND_CLEAR: o[i] = 0; break;
            case RGPU_BLEND_SOURCE_OVER: o[i] = (uint16_t)(s[i] + div255((uint16_t)(d[i] * inv(sa)))); break;
            case RGPU_BLEND_DESTINATION_OUT: o[i] = div255((uint16_t)(d[i] * inv(sa))); break;
            case RGPU_BLEND_SOURCE_ATOP: o[i] = div255((uint16_t)(s[i] * d[3] + d[i] * inv(sa))); break;
            case RGPU_BLEND_XOR: o[i] = div255((uint16_t)(s[i] * inv(d[3]) + d[i] * inv(sa))); break;
            case RGPU_BLEND_PLUS: o[i] = std::min<uint16_t>((uint16_t)(s[i] + d[i]), 255); break;
            case RGPU_BLEND_MODULATE: o[i] = div255((uint16_t)(s[i] * d[i])); break;
            case RGPU_BLEND_SCREEN: o[i] = (uint16_t)(s[i] + d[i] - div255((uint16_t)(s[i] * d[i]))); break;
            default: o[i] = s[i]; break;  // Source: no blend stage
            }
        }
    }
    void pixel(int32_t x, int32_t y, uint8_t cov) {
        uint8_t *p = pm->px((uint32_t)x, (uint32_t)y);
        if (cov == 255 && memset_ok) { memcpy(p, memset_color, 4); return; }
        if (lowp) {
            uint16_t s[4] = {rgba16[0], rgba16[1], rgba16[2], rgba16[3]};
            if (shader->kind != SHADER_SOLID) gradient_eval_lowp(grad, shader->spread, x, y, s);
            uint16_t d[4] = {p[0], p[1], p[2], p[3]};
            uint16_t o[4];
            if (cov == 255) {
                if (blend == RGPU_BLEND_SOURCE) { for (int i = 0; i < 4; i++) o[i] = s[i]; }
                else lowp_blend(s, d, o);
            } else {
                uint16_t c = sat_u16(((float)cov * INV255) * 255.0f + 0.5f);
                if (pre_scale()) {
                    for (int i = 0; i < 4; i++) s[i] = div255((uint16_t)(s[i] * c));
                    lowp_blend(s, d, o);
                } else {
                    uint16_t b[4];
                    lowp_blend(s, d, b);
                    for (int i = 0; i < 4; i++) o[i] = lerp16(d[i], b[i], c);
                }
            }
            for (int i = 0; i < 4; i++) p[i] = (uint8_t)o[i];
            return;
        }
        // highp
        float s[4];
        if (shader->kind == SHADER_SOLID) {
            for (int i = 0; i < 4; i++) s[i] = colorf[i];
        } else if (shader->kind == SHADER_PATTERN) {
            pattern_eval(*shader, pinv, pquality, x, y, s);
        } else {
            ColorF c;
            if (!gradient_eval(grad, shader->spread, x, y, &c)) c = ColorF{0, 0, 0, 0};
            s[0] = c.r; s[1] = c.g; s[2] = c.b; s[3] = c.a;
        }
        float d[4] = {p[0] * INV255, p[1] * INV255, p[2] * INV255, p[3] * INV255};
        float o[4];
        if (cov == 255) {
            if (blend == RGPU_BLEND_SOURCE) { for (int i = 0; i < 4; i++) o[i] = s[i]; }
            else blend_sep(blend, s, d, o);
        } else {
            float c = (float)cov * INV255;
            if (pre_scale()) {
                for (int i = 0; i < 4; i++) s[i] = s[i] * c;
                blend_sep(blend, s, d, o);
            } else {
                float b[4];
                blend_sep(blend, s, d, b);
                for (int i = 0; i < 4; i++) o[i] = (b[i] - d[i]) * c + d[i];
            }
        }
        for (int i = 0; i < 4; i++) p[i] = unnorm(o[i]);
    }
};

static bool is_too_big_for_math(const Path &p) {
    const float limit = FLT_MAX * 0.25f;
    return !(p.bounds.l >= -limit && p.bounds.t >= -limit && p.bounds.r <= limit && p.bounds.b <= limit);
}

void fill_path(Pixmap &pm, const Path &path_in, const Paint &paint_in, uint32_t rule, const Transform &ts) {
    Path path = path_in;
    Paint paint = paint_in;
    if (!ts.is_identity()) {
        if (!path.transform(ts)) return;
        if (paint.shader.kind == SHADER_LINEAR || paint.shader.kind == SHADER_RADIAL ||
            paint.shader.kind == SHADER_PATTERN)
            paint.shader.transform = paint.shader.transform.post_concat(ts);
    } else {
        path.compute_bounds();
    }
    if (is_nearly_zero(path.bounds.w()) || is_nearly_zero(path.bounds.h())) return;
    if (is_too_big_for_math(path)) return;
    PipelineBlitter bl;
    if (!bl.setup(pm, paint)) return;
    IntRect clip{0, 0, (int32_t)pm.width, (int32_t)pm.height};
    scan_path(path, rule, paint.anti_alias, clip, [&](int32_t x, int32_t y, uint8_t c) { bl.pixel(x, y, c); });
}

// ---------------------------------------------------------------- anti-aliased hairlines
// scan/hairline_aa.rs: do_anti_hairline (Skia's SkScan_Antihair.cpp) with the
// HLine / Horish / VLine / Vertish anti-hair blitters, drawing through the
// pipeline blitter; a clip rect (the RectClipBlitter) drops pixels outside it.
namespace {
struct HairClip {
    bool on;
    int32_t l, t, r, b;
};
inline uint8_t hair_small_scale(uint32_t v, int32_t dot6) { return (uint8_t)((v * (uint32_t)dot6) >> 6); }
inline int32_t contribution_64(int32_t o) { return ((o - 1) & 63) + 1; }
inline int32_t fdot16_fast_div(int32_t a, int32_t b) {
    if (a >= -32768 && a <= 32767) return (int32_t)((uint32_t)a << 16) / b;
    int64_t v = ((int64_t)a << 16) / b;
    return (int32_t)std::min<int64_t>(std::max<int64_t>(v, INT32_MIN), INT32_MAX);
}
inline int32_t fdot16_ceil(int32_t x) { return (int32_t)(((int64_t)x + 0xFFFF) >> 16); }

struct HairBlit {
    PipelineBlitter &bl;
    HairClip clip;
    int32_t w, h;
    void px(int64_t x, int64_t y, uint8_t a) {
        if (a == 0) return;
        if (clip.on && (x < clip.l || x >= clip.r || y < clip.t || y >= clip.b)) return;
        if (x < 0 || y < 0 || x >= w || y >= h) return;
        bl.pixel((int32_t)x, (int32_t)y, a);
    }
};

enum HairKind { HK_HLINE, HK_HORISH, HK_VLINE, HK_VERTISH };

// draw_cap / draw_line of the four blitters for one step of the major axis
void hair_step(HairKind k, HairBlit &b, int32_t major, int32_t &f, int32_t slope, int32_t mod64) {
    const int32_t half = 1 << 15;
    int32_t fy = f + half;
    if (fy < 0) fy = 0;
    const int32_t hi = fy >> 16;
    const uint8_t a = (uint8_t)((fy >> 8) & 0xFF);
    switch (k) {
    case HK_HLINE: {
        uint8_t m = hair_small_scale(a, mod64);
        if (m) b.px(major, hi, m);
        m = hair_small_scale(255 - a, mod64);
        if (m && hi >= 1) b.px(major, hi - 1, m);
        f = fy - half;
        break;
    }
    case HK_HORISH: {
        const int32_t y0 = std::max(hi, 1) - 1;
        b.px(major, y0, hair_small_scale(255 - a, mod64));
        b.px(major, y0 + 1, hair_small_scale(a, mod64));
        f = fy + slope - half;
        break;
    }
    case HK_VLINE: {
        uint8_t m = hair_small_scale(a, mod64);
        if (m) b.px(hi, major, m);
        m = hair_small_scale(255 - a, mod64);
        if (m) b.px(std::max(hi, 1) - 1, major, m);
        f = fy - half;
        break;
    }
    case HK_VERTISH: {
        const int32_t x0 = std::max(hi, 1) - 1;
        b.px(x0, major, hair_small_scale(255 - a, mod64));
        b.px(x0 + 1, major, hair_small_scale(a, mod64));
        f = fy + slope - half;
        break;
    }
    }
}

void do_anti_hairline(int32_t x0, int32_t y0, int32_t x1, int32_t y1, HairClip clip, HairBlit &b) {
    auto bad = [](int32_t v) { return v == INT32_MIN; };
    if (bad(x0) || bad(y0) || bad(x1) || bad(y1)) return;
    if (std::abs(x1 - x0) > 511 * 64 || std::abs(y1 - y0) > 511 * 64) {
        const int32_t hx = (x0 >> 1) + (x1 >> 1), hy = (y0 >> 1) + (y1 >> 1);
        do_anti_hairline(x0, y0, hx, hy, clip, b);
        do_anti_hairline(hx, hy, x1, y1, clip, b);
        return;
    }
    int32_t scale_start, scale_stop, istart, istop, fstart, slope;
    HairKind kind;
    if (std::abs(x1 - x0) > std::abs(y1 - y0)) {
        if (x0 > x1) { std::swap(x0, x1); std::swap(y0, y1); }
        istart = x0 >> 6;
        istop = (x1 + 63) >> 6;
        fstart = (int32_t)((uint32_t)y0 << 10);
        if (y0 == y1) {
            slope = 0;
            kind = HK_HLINE;
        } else {
            slope = fdot16_fast_div(y1 - y0, x1 - x0);
            fstart += (slope * (32 - (x0 & 63)) + 32) >> 6;
            kind = HK_HORISH;
        }
        if (istop - istart == 1) { scale_start = x1 - x0; scale_stop = 0; }
        else { scale_start = 64 - (x0 & 63); scale_stop = x1 & 63; }
        if (clip.on) {
            if (istart >= clip.r || istop <= clip.l) return;
            if (istart < clip.l) {
                fstart += slope * (clip.l - istart);
                istart = clip.l;
                scale_start = 64;
                if (istop - istart == 1) { scale_start = contribution_64(x1); scale_stop = 0; }
            }
            if (istop > clip.r) { istop = clip.r; scale_stop = 0; }
            if (istart == istop) return;
            int32_t top, bottom;
            if (slope >= 0) {
                top = (fstart - (1 << 15)) >> 16;
                bottom = fdot16_ceil(fstart + (istop - istart - 1) * slope + (1 << 15));
            } else {
                bottom = fdot16_ceil(fstart + (1 << 15));
                top = (fstart + (istop - istart - 1) * slope - (1 << 15)) >> 16;
            }
            top -= 1;
            bottom += 1;
            if (top >= clip.b || bottom <= clip.t) return;
            if (clip.t <= top && clip.b >= bottom) clip.on = false;
        }
    } else {
        if (y0 > y1) { std::swap(x0, x1); std::swap(y0, y1); }
        istart = y0 >> 6;
        istop = (y1 + 63) >> 6;
        fstart = (int32_t)((uint32_t)x0 << 10);
        if (x0 == x1) {
            if (y0 == y1) return;
            slope = 0;
            kind = HK_VLINE;
        } else {
            slope = fdot16_fast_div(x1 - x0, y1 - y0);
            fstart += (slope * (32 - (y0 & 63)) + 32) >> 6;
            kind = HK_VERTISH;
        }
        if (istop - istart == 1) { scale_start = y1 - y0; scale_stop = 0; }
        else { scale_start = 64 - (y0 & 63); scale_stop = y1 & 63; }
        if (clip.on) {
            if (istart >= clip.b || istop <= clip.t) return;
            if (istart < clip.t) {
                fstart += slope * (clip.t - istart);
                istart = clip.t;
                scale_start = 64;
                if (istop - istart == 1) { scale_start = contribution_64(y1); scale_stop = 0; }
            }
            if (istop > clip.b) { istop = clip.b; scale_stop = 0; }
            if (istart == istop) return;
            int32_t left, right;
            if (slope >= 0) {
                left = (fstart - (1 << 15)) >> 16;
                right = fdot16_ceil(fstart + (istop - istart - 1) * slope + (1 << 15));
            } else {
                right = fdot16_ceil(fstart + (1 << 15));
                left = (fstart + (istop - istart - 1) * slope - (1 << 15)) >> 16;
            }
            left -= 1;
            right += 1;
            if (left >= clip.r || right <= clip.l) return;
            if (clip.l <= left && clip.r >= right) clip.on = false;
        }
    }
    HairBlit bb{b.bl, clip, b.w, b.h};
    int32_t f = fstart;
    hair_step(kind, bb, istart, f, slope, scale_start);
    istart += 1;
    const int32_t full = istop - istart - (scale_stop > 0 ? 1 : 0);
    for (int32_t i = 0; i < full; i++) hair_step(kind, bb, istart + i, f, slope, 64);
    if (scale_stop > 0) hair_step(kind, bb, istop - 1, f, slope, scale_stop);
}
}  // namespace

void anti_hairlines(Pixmap &pm, const Paint &paint, const int32_t *calls, size_t ncalls) {
    PipelineBlitter bl;
    if (!bl.setup(pm, paint)) return;
    HairBlit b{bl, HairClip{false, 0, 0, 0, 0}, (int32_t)pm.width, (int32_t)pm.height};
    for (size_t i = 0; i < ncalls; i++) {
        const int32_t *c = calls + 9 * i;
        HairClip clip{c[8] != 0, c[4], c[5], c[6], c[7]};
        do_anti_hairline(c[0], c[1], c[2], c[3], clip, b);
    }
}

void pixmap_fill(Pixmap &pm, ColorF c) {
    ColorF p = premultiply(c);
    uint8_t v[4] = {f32_to_u8_round(p.r), f32_to_u8_round(p.g), f32_to_u8_round(p.b), f32_to_u8_round(p.a)};
    for (size_t i = 0; i < (size_t)pm.width * pm.height; i++) memcpy(&pm.data[i * 4], v, 4);
}

// fill_rect with an integer-aligned rect (the only kind resvg's render passes):
// full coverage over rect ∩ pixmap.
void fill_rect(Pixmap &pm, const Rect &r, const Paint &paint) {
    int32_t l = sat_i32(std::nearbyint(r.l)), t = sat_i32(std::nearbyint(r.t));
    int32_t rr = sat_i32(std::nearbyint(r.r)), b = sat_i32(std::nearbyint(r.b));
    l = std::max(l, 0); t = std::max(t, 0);
    rr = std::min(rr, (int32_t)pm.width); b = std::min(b, (int32_t)pm.height);
    if (rr <= l || b <= t) return;
    PipelineBlitter bl;
    if (!bl.setup(pm, paint)) return;
    for (int32_t y = t; y < b; y++)
        for (int32_t x = l; x < rr; x++) bl.pixel(x, y, 255);
}

// draw_pixmap: Pattern(Pad, Nearest, opacity) + fill_rect, highp.
void draw_pixmap(Pixmap &dst, int32_t x, int32_t y, const Pixmap &src, float opacity, uint32_t blend) {
    int32_t l = std::max(x, 0), t = std::max(y, 0);
    int32_t r = std::min<int64_t>((int64_t)x + src.width, dst.width);
    int32_t b = std::min<int64_t>((int64_t)y + src.height, dst.height);
    if (r <= l || b <= t) return;
    if (blend == RGPU_BLEND_DESTINATION) return;
    for (int32_t py = t; py < b; py++) {
        for (int32_t px = l; px < r; px++) {
            // seed_shader + translate + gather (clamped)
            float fx = ((float)px + 0.5f) - (float)x, fy = ((float)py + 0.5f) - (float)y;
            fx = std::min(std::max(fx, 0.0f), (float)src.width - 1e-3f);
            fy = std::min(std::max(fy, 0.0f), (float)src.height - 1e-3f);
            const uint8_t *sp = src.px((uint32_t)fx, (uint32_t)fy);
            float s[4] = {sp[0] * INV255, sp[1] * INV255, sp[2] * INV255, sp[3] * INV255};
            if (opacity != 1.0f)
                for (int i = 0; i < 4; i++) s[i] = s[i] * opacity;
            uint8_t *dp = dst.px((uint32_t)px, (uint32_t)py);
            float d[4] = {dp[0] * INV255, dp[1] * INV255, dp[2] * INV255, dp[3] * INV255};
            float o[4];
            if (blend == RGPU_BLEND_SOURCE) { for (int i = 0; i < 4; i++) o[i] = s[i]; }
            else blend_sep(blend, s, d, o);
            for (int i = 0; i < 4; i++) dp[i] = unnorm(o[i]);
        }
    }
}

Mask mask_from_pixmap(const Pixmap &pm, bool luminance) {
    Mask m(pm.width, pm.height);
    size_t n = (size_t)pm.width * pm.height;
    for (size_t i = 0; i < n; i++) {
        const uint8_t *p = &pm.data[i * 4];
        if (!luminance) { m.data[i] = p[3]; continue; }
        float r = p[0] / 255.0f, g = p[1] / 255.0f, b = p[2] / 255.0f, a = p[3] / 255.0f;
        if (p[3] != 0) { r /= a; g /= a; b /= a; }
        // Rec. 709 luma coefficients (tiny-skia mask.rs from_pixmap)
        float luma = r * 0.2126f + g * 0.7152f + b * 0.0722f;
        float v = std::ceil(std::min(std::max((luma * a) * 255.0f, 0.0f), 255.0f));
        m.data[i] = sat_u8(v);
    }
    return m;
}
void mask_invert(Mask &m) { for (auto &a : m.data) a = (uint8_t)(255 - a); }
void apply_mask(Pixmap &pm, const Mask &m) {
    bool all_ff = true;
    for (auto a : m.data) if (a != 0xFF) { all_ff = false; break; }
    if (all_ff) return;
    size_t n = (size_t)pm.width * pm.height;
    for (size_t i = 0; i < n; i++) {
        uint16_t c = m.data[i];
        for (int k = 0; k < 4; k++) pm.data[i * 4 + k] = (uint8_t)div255((uint16_t)(pm.data[i * 4 + k] * c));
    }
}
void mask_fill_path(Mask &m, const Path &path_in, uint32_t rule, bool aa, const Transform &ts) {
    Path path = path_in;
    if (!ts.is_identity()) { if (!path.transform(ts)) return; }
    else path.compute_bounds();
    if (is_nearly_zero(path.bounds.w()) || is_nearly_zero(path.bounds.h())) return;
    if (is_too_big_for_math(path)) return;
    IntRect clip{0, 0, (int32_t)m.width, (int32_t)m.height};
    scan_path(path, rule, aa, clip, [&](int32_t x, int32_t y, uint8_t c) {
        uint8_t &d = m.data[(size_t)y * m.width + x];
        if (c == 255) { d = 255; return; }
        uint16_t cc = sat_u16(((float)c * INV255) * 255.0f + 0.5f);
        d = (uint8_t)lerp16(d, 255, cc);
    });
}

}  // namespace ora
