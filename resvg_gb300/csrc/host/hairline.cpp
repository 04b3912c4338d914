// Host-side geometry of anti-aliased hairline strokes (see hairline.h):
// tiny-skia 0.12 painter.rs (treat_as_hairline and the coverage-scaled
// paint), scan/hairline.rs (stroke_path_impl: cap extension, quad/cubic
// subdivision, inset/outset culling) and scan/hairline_aa.rs
// (anti_hair_line_rgn: fixed-range and clip clipping of each line), which
// port Skia's SkScan_Hairline.cpp / SkScan_Antihair.cpp.
#include "hairline.h"
#include <algorithm>
#include <climits>
#include <cmath>

namespace rgpu {
namespace {

struct P2 {
    float x = 0, y = 0;
};
inline P2 mk(float x, float y) { return P2{x, y}; }
inline bool is_zero(P2 p) { return p.x == 0.0f && p.y == 0.0f; }

enum : uint8_t { V_MOVE = 0, V_LINE = 1, V_QUAD = 2, V_CUBIC = 3, V_CLOSE = 4, V_NONE = 255 };

constexpr float kPi = 3.14159265f;
constexpr int kMaxQuadLevel = 5;
constexpr int kMaxCubicLevel = 9;

// Point::normalize (length computed in f64)
void normalize(P2 &p) {
    double xx = p.x, yy = p.y;
    double dmag = std::sqrt(xx * xx + yy * yy);
    double s = 1.0 / dmag;
    float x = p.x * (float)s, y = p.y * (float)s;
    if (!std::isfinite(x) || !std::isfinite(y) || (x == 0.0f && y == 0.0f)) { p = P2{}; return; }
    p = mk(x, y);
}

void map_points(const Xf &t, P2 *p, size_t n) {
    if (t.identity()) return;
    const bool translate_only = !t.skew() && t.sx == 1 && t.sy == 1;
    for (size_t i = 0; i < n; i++) {
        if (translate_only) { p[i].x += t.tx; p[i].y += t.ty; }
        else if (!t.skew()) { p[i].x = p[i].x * t.sx + t.tx; p[i].y = p[i].y * t.sy + t.ty; }
        else {
            float x = p[i].x * t.sx + p[i].y * t.kx + t.tx;
            float y = p[i].x * t.ky + p[i].y * t.sy + t.ty;
            p[i].x = x; p[i].y = y;
        }
    }
}

struct FRect {
    float l, t, r, b;
};
struct IRect {
    int32_t l, t, r, b;  // right/bottom exclusive
};

inline int32_t sat_i32(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}

// Rect::round_out: (floor x, floor y, max(1, ceil w), max(1, ceil h))
bool round_out(const FRect &r, IRect *o) {
    int64_t x = sat_i32(std::floor(r.l)), y = sat_i32(std::floor(r.t));
    int64_t w = std::max<int64_t>(1, (uint32_t)sat_i32(std::ceil(r.r - r.l)));
    int64_t h = std::max<int64_t>(1, (uint32_t)sat_i32(std::ceil(r.b - r.t)));
    if (x + w > INT32_MAX || y + h > INT32_MAX) return false;
    *o = IRect{(int32_t)x, (int32_t)y, (int32_t)(x + w), (int32_t)(y + h)};
    return true;
}
bool intersects(const IRect &a, const IRect &b) {
    return std::max(a.l, b.l) < std::min(a.r, b.r) && std::max(a.t, b.t) < std::min(a.b, b.b);
}
bool contains(const IRect &a, const IRect &b) { return a.l <= b.l && a.t <= b.t && a.r >= b.r && a.b >= b.b; }

// ---- line_clipper::intersect (used by anti_hair_line_rgn)
bool nested_lt(float a, float b, float dim) { return a <= b && (a < b || dim > 0.0f); }
double pin_unsorted(double v, double l0, double l1) {
    if (l1 < l0) std::swap(l0, l1);
    return v < l0 ? l0 : (v > l1 ? l1 : v);
}
float sect_with_horizontal(const P2 s[2], float y) {
    float dy = s[0].y - s[1].y;
    if (std::fabs(dy) <= 1.0f / 4096.0f) return (s[0].x + s[1].x) * 0.5f;
    double x0 = s[0].x, y0 = s[0].y, x1 = s[1].x, y1 = s[1].y;
    double r = x0 + ((double)y - y0) * (x1 - x0) / (y1 - y0);
    return (float)pin_unsorted(r, x0, x1);
}
float sect_with_vertical(const P2 s[2], float x) {
    float dx = s[0].x - s[1].x;
    if (std::fabs(dx) <= 1.0f / 4096.0f) return (s[0].y + s[1].y) * 0.5f;
    double x0 = s[0].x, y0 = s[0].y, x1 = s[1].x, y1 = s[1].y;
    double r = y0 + ((double)x - x0) * (y1 - y0) / (x1 - x0);
    return (float)pin_unsorted(r, y0, y1);
}
bool line_intersect(const P2 src[2], const FRect &clip, P2 dst[2]) {
    FRect bounds{std::min(src[0].x, src[1].x), std::min(src[0].y, src[1].y), std::max(src[0].x, src[1].x),
                 std::max(src[0].y, src[1].y)};
    if (std::isfinite(bounds.l) && std::isfinite(bounds.t) && std::isfinite(bounds.r) && std::isfinite(bounds.b)) {
        if (clip.l <= bounds.l && clip.t <= bounds.t && clip.r >= bounds.r && clip.b >= bounds.b) {
            dst[0] = src[0]; dst[1] = src[1];
            return true;
        }
        const float bw = bounds.r - bounds.l, bh = bounds.b - bounds.t;
        if (nested_lt(bounds.r, clip.l, bw) || nested_lt(clip.r, bounds.l, bw) || nested_lt(bounds.b, clip.t, bh) ||
            nested_lt(clip.b, bounds.t, bh))
            return false;
    }
    int i0 = src[0].y < src[1].y ? 0 : 1, i1 = 1 - i0;
    P2 tmp[2] = {src[0], src[1]};
    if (tmp[i0].y < clip.t) tmp[i0] = mk(sect_with_horizontal(src, clip.t), clip.t);
    if (tmp[i1].y > clip.b) tmp[i1] = mk(sect_with_horizontal(src, clip.b), clip.b);
    i0 = tmp[0].x < tmp[1].x ? 0 : 1;
    i1 = 1 - i0;
    if (tmp[i1].x <= clip.l || tmp[i0].x >= clip.r) {
        if (tmp[0].x != tmp[1].x || tmp[0].x < clip.l || tmp[0].x > clip.r) return false;
    }
    if (tmp[i0].x < clip.l) tmp[i0] = mk(clip.l, sect_with_vertical(src, clip.l));
    if (tmp[i1].x > clip.r) tmp[i1] = mk(clip.r, sect_with_vertical(src, clip.r));
    dst[0] = tmp[0]; dst[1] = tmp[1];
    return true;
}

inline int32_t fdot6_from(float v) {
    // (v * 64.0) as i32: truncation, saturating
    return sat_i32(v * 64.0f);
}
inline int32_t fdot6_floor(int32_t v) { return v >> 6; }
inline int32_t fdot6_ceil(int32_t v) { return (v + 63) >> 6; }

struct Emitter {
    std::vector<HairCall> &out;
    bool has_clip;
    IRect clip;
};

// anti_hair_line_rgn: every line of the polyline is clipped to fixed-point
// range and (outset by one pixel) to the target, converted to FDot6, and
// handed over with the sub-clip it needs.
void line_proc(const P2 *pts, size_t n, bool clipped, Emitter &em) {
    const float mx = 32767.0f;
    const FRect fixed{-mx, -mx, mx, mx};
    FRect clip_bounds{};
    if (clipped) {
        clip_bounds = FRect{(float)em.clip.l - 1.0f, (float)em.clip.t - 1.0f, (float)em.clip.r + 1.0f,
                            (float)em.clip.b + 1.0f};
    }
    for (size_t i = 0; i + 1 < n; i++) {
        P2 seg[2] = {pts[i], pts[i + 1]}, c[2];
        if (!line_intersect(seg, fixed, c)) continue;
        if (clipped) {
            P2 t2[2] = {c[0], c[1]};
            if (!line_intersect(t2, clip_bounds, c)) continue;
        }
        const int32_t x0 = fdot6_from(c[0].x), y0 = fdot6_from(c[0].y);
        const int32_t x1 = fdot6_from(c[1].x), y1 = fdot6_from(c[1].y);
        if (clipped) {
            IRect ir{fdot6_floor(std::min(x0, x1)) - 1, fdot6_floor(std::min(y0, y1)) - 1,
                     fdot6_ceil(std::max(x0, x1)) + 1, fdot6_ceil(std::max(y0, y1)) + 1};
            if (!intersects(em.clip, ir)) continue;
            if (!contains(em.clip, ir)) {
                IRect sub{std::max(ir.l, em.clip.l), std::max(ir.t, em.clip.t), std::min(ir.r, em.clip.r),
                          std::min(ir.b, em.clip.b)};
                if (sub.r > sub.l && sub.b > sub.t)
                    em.out.push_back(HairCall{x0, y0, x1, y1, sub.l, sub.t, sub.r, sub.b, 1u});
                continue;
            }
        }
        em.out.push_back(HairCall{x0, y0, x1, y1, 0, 0, 0, 0, 0u});
    }
}

// ---- scan/hairline.rs
uint32_t int_quad_dist(const P2 p[3]) {
    float dx = std::fabs((p[0].x + p[2].x) * 0.5f - p[1].x);
    float dy = std::fabs((p[0].y + p[2].y) * 0.5f - p[1].y);
    uint32_t idx = (uint32_t)sat_i32(std::ceil(dx)), idy = (uint32_t)sat_i32(std::ceil(dy));
    return idx > idy ? idx + (idy >> 1) : idy + (idx >> 1);
}
int quad_level(const P2 p[3]) {
    uint32_t d = int_quad_dist(p);
    int lz = d == 0 ? 32 : __builtin_clz(d);
    int level = (33 - lz) >> 1;
    return std::min(level, kMaxQuadLevel);
}

bool curve_bounds(const P2 *p, int n, FRect *r) {
    float l = p[0].x, t = p[0].y, rr = p[0].x, b = p[0].y;
    for (int i = 1; i < n; i++) {
        l = std::min(l, p[i].x); rr = std::max(rr, p[i].x);
        t = std::min(t, p[i].y); b = std::max(b, p[i].y);
    }
    if (!(std::isfinite(l) && std::isfinite(t) && std::isfinite(rr) && std::isfinite(b))) return false;
    *r = FRect{l, t, rr, b};
    return true;
}
bool geometric_overlap(const FRect &a, const FRect &b) { return a.l < b.r && b.l < a.r && a.t < b.b && b.t < a.b; }
bool geometric_contains(const FRect &outer, const FRect &inner) {
    return inner.r <= outer.r && inner.l >= outer.l && inner.b <= outer.b && inner.t >= outer.t;
}

void hair_quad(const P2 p[3], bool clipped, const FRect *inset, const FRect *outset, int level, Emitter &em) {
    if (inset) {
        FRect b;
        if (!curve_bounds(p, 3, &b)) return;
        if (!geometric_overlap(*outset, b)) return;
        if (geometric_contains(*inset, b)) clipped = false;
    }
    const int lines = 1 << level;
    P2 tmp[(1 << kMaxQuadLevel) + 1];
    // QuadCoeff: a = p2 - 2 p1 + p0, b = 2 (p1 - p0), c = p0; v = (a t + b) t + c
    const float ax = p[2].x - (p[1].x + p[1].x) + p[0].x, ay = p[2].y - (p[1].y + p[1].y) + p[0].y;
    const float bx = (p[1].x - p[0].x) * 2.0f, by = (p[1].y - p[0].y) * 2.0f;
    tmp[0] = p[0];
    const float dt = 1.0f / (float)lines;
    float t = 0.0f;
    for (int i = 1; i < lines; i++) {
        t = t + dt;
        tmp[i] = mk((ax * t + bx) * t + p[0].x, (ay * t + by) * t + p[0].y);
    }
    tmp[lines] = p[2];
    line_proc(tmp, (size_t)lines + 1, clipped, em);
}

int cubic_segments(const P2 p[4]) {
    const float one_third = 1.0f / 3.0f, two_third = 2.0f / 3.0f;
    const float p13x = one_third * p[3].x + two_third * p[0].x, p13y = one_third * p[3].y + two_third * p[0].y;
    const float p23x = one_third * p[0].x + two_third * p[3].x, p23y = one_third * p[0].y + two_third * p[3].y;
    const float dx = std::max(std::fabs(p[1].x - p13x), std::fabs(p[2].x - p23x));
    const float dy = std::max(std::fabs(p[1].y - p13y), std::fabs(p[2].y - p23y));
    const float diff = std::max(dx, dy);
    float tol = 1.0f / 8.0f;
    for (int i = 0; i < kMaxCubicLevel; i++) {
        if (diff < tol) return 1 << i;
        tol *= 4.0f;
    }
    return 1 << kMaxCubicLevel;
}

void hair_cubic2(const P2 p[4], bool clipped, Emitter &em) {
    const int lines = cubic_segments(p);
    if (lines == 1) {
        P2 two[2] = {p[0], p[3]};
        line_proc(two, 2, clipped, em);
        return;
    }
    // CubicCoeff: a = p3 + 3 (p1 - p2) - p0, b = 3 (p2 - 2 p1 + p0), c = 3 (p1 - p0), d = p0
    const float ax = p[3].x + 3.0f * (p[1].x - p[2].x) - p[0].x, ay = p[3].y + 3.0f * (p[1].y - p[2].y) - p[0].y;
    const float bx = 3.0f * (p[2].x - (p[1].x + p[1].x) + p[0].x), by = 3.0f * (p[2].y - (p[1].y + p[1].y) + p[0].y);
    const float cx = 3.0f * (p[1].x - p[0].x), cy = 3.0f * (p[1].y - p[0].y);
    std::vector<P2> tmp((size_t)lines + 1);
    tmp[0] = p[0];
    const float dt = 1.0f / (float)lines;
    float t = 0.0f;
    bool finite = true;
    for (int i = 1; i < lines; i++) {
        t = t + dt;
        tmp[i] = mk(((ax * t + bx) * t + cx) * t + p[0].x, ((ay * t + by) * t + cy) * t + p[0].y);
        finite = finite && std::isfinite(tmp[i].x) && std::isfinite(tmp[i].y);
    }
    if (!finite) return;
    tmp[lines] = p[3];
    line_proc(tmp.data(), tmp.size(), clipped, em);
}

bool lt_90(P2 a, P2 pivot, P2 b) { return (a.x - pivot.x) * (b.x - pivot.x) + (a.y - pivot.y) * (b.y - pivot.y) >= 0.0f; }

// find_cubic_max_curvature + chop_cubic_at (path_geometry.rs)
void formulate(const float s[4], float out[4]) {
    float a = s[1] - s[0], b = s[2] - 2.0f * s[1] + s[0], c = s[3] + 3.0f * (s[1] - s[2]) - s[0];
    out[0] = c * c; out[1] = 3.0f * b * c; out[2] = 2.0f * b * b + c * a; out[3] = a * b;
}
bool valid_unit_divide(float numer, float denom, float *r) {
    if (numer < 0.0f) { numer = -numer; denom = -denom; }
    if (denom == 0.0f || numer == 0.0f || numer >= denom) return false;
    float v = numer / denom;
    if (!(v > 0.0f && v < 1.0f)) return false;
    *r = v;
    return true;
}
int unit_quad_roots(float a, float b, float c, float r[3]) {
    if (a == 0.0f) return valid_unit_divide(-c, b, &r[0]) ? 1 : 0;
    double dr = (double)b * b - 4.0 * (double)a * c;
    if (dr < 0.0) return 0;
    float s = (float)std::sqrt(dr);
    if (!std::isfinite(s)) return 0;
    float q = b < 0.0f ? -(b - s) / 2.0f : -(b + s) / 2.0f;
    int n = 0;
    if (valid_unit_divide(q, a, &r[n])) n++;
    if (valid_unit_divide(c, q, &r[n])) n++;
    if (n == 2) {
        if (r[0] > r[1]) std::swap(r[0], r[1]);
        else if (r[0] == r[1]) n--;
    }
    return n;
}
inline float clamp01(float v) { return std::isfinite(v) ? std::min(std::max(v, 0.0f), 1.0f) : 0.0f; }
int max_curvature(const P2 p[4], float t[3]) {
    float xs[4] = {p[0].x, p[1].x, p[2].x, p[3].x}, ys[4] = {p[0].y, p[1].y, p[2].y, p[3].y}, cx[4], cy[4];
    formulate(xs, cx);
    formulate(ys, cy);
    for (int i = 0; i < 4; i++) cx[i] += cy[i];
    if (std::fabs(cx[0]) <= 1.0f / 4096.0f) return unit_quad_roots(cx[1], cx[2], cx[3], t);
    float inva = 1.0f / cx[0];
    float a = cx[1] * inva, b = cx[2] * inva, c = cx[3] * inva;
    float q = (a * a - b * 3.0f) / 9.0f;
    float r = (2.0f * a * a * a - 9.0f * a * b + 27.0f * c) / 54.0f;
    float q3 = q * q * q, r2mq3 = r * r - q3, adiv3 = a / 3.0f;
    if (r2mq3 < 0.0f) {
        float v = std::min(std::max(r / std::sqrt(q3), -1.0f), 1.0f);
        float theta = std::acos(v), n2 = -2.0f * std::sqrt(q);
        t[0] = clamp01(n2 * std::cos(theta / 3.0f) - adiv3);
        t[1] = clamp01(n2 * std::cos((theta + 2.0f * kPi) / 3.0f) - adiv3);
        t[2] = clamp01(n2 * std::cos((theta - 2.0f * kPi) / 3.0f) - adiv3);
        if (t[0] > t[1]) std::swap(t[0], t[1]);
        if (t[1] > t[2]) std::swap(t[1], t[2]);
        if (t[0] > t[1]) std::swap(t[0], t[1]);
        int len = 3;
        if (t[1] == t[2]) len = 2;
        if (t[0] == t[1]) { for (int i = 0; i < len - 1; i++) t[i] = t[i + 1]; len--; }
        return len;
    }
    float aa = std::pow(std::fabs(r) + std::sqrt(r2mq3), 0.3333333f);
    if (r > 0.0f) aa = -aa;
    if (aa != 0.0f) aa += q / aa;
    t[0] = clamp01(aa - adiv3);
    return 1;
}
void chop_cubic_at1(const P2 s[4], float t, P2 d[7]) {
    auto in = [t](P2 a, P2 b) { return mk(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t); };
    P2 ab = in(s[0], s[1]), bc = in(s[1], s[2]), cd = in(s[2], s[3]);
    P2 abc = in(ab, bc), bcd = in(bc, cd), abcd = in(abc, bcd);
    d[0] = s[0]; d[1] = ab; d[2] = abc; d[3] = abcd; d[4] = bcd; d[5] = cd; d[6] = s[3];
}
int chop_at_max_curvature(const P2 src[4], P2 dst[13]) {
    float roots[3];
    int nr = max_curvature(src, roots);
    float tv[3];
    int count = 0;
    for (int i = 0; i < nr; i++)
        if (0.0f < roots[i] && roots[i] < 1.0f) tv[count++] = roots[i];
    if (count == 0) {
        for (int i = 0; i < 4; i++) dst[i] = src[i];
        return 1;
    }
    // chop_cubic_at over several t
    P2 cur[4] = {src[0], src[1], src[2], src[3]};
    P2 *d = dst;
    float t = tv[0];
    for (int i = 0; i < count; i++) {
        chop_cubic_at1(cur, t, d);
        if (i == count - 1) break;
        d += 3;
        for (int k = 0; k < 4; k++) cur[k] = d[k];
        if (!valid_unit_divide(tv[i + 1] - tv[i], 1.0f - tv[i], &t)) {
            d[4] = d[5] = d[6] = cur[3];
            break;
        }
    }
    return count + 1;
}

void hair_cubic(const P2 p[4], bool clipped, const FRect *inset, const FRect *outset, Emitter &em) {
    if (inset) {
        FRect b;
        if (!curve_bounds(p, 4, &b)) return;
        if (!geometric_overlap(*outset, b)) return;
        if (geometric_contains(*inset, b)) clipped = false;
    }
    if (lt_90(p[1], p[0], p[3]) && lt_90(p[2], p[0], p[3]) && lt_90(p[1], p[3], p[0]) && lt_90(p[2], p[3], p[0])) {
        hair_cubic2(p, clipped, em);
    } else {
        P2 tmp[13];
        int n = chop_at_max_curvature(p, tmp);
        for (int i = 0; i < n; i++) hair_cubic2(&tmp[3 * i], clipped, em);
    }
}

// extend_pts: moves the open ends of a segment outwards by the cap's area
void extend_pts(uint32_t cap, uint8_t prev_verb, uint8_t next_verb, P2 *pts, int n) {
    const float outset = cap == 2 ? 0.5f : kPi / 8.0f;  // square : round
    if (prev_verb == V_MOVE) {
        P2 first = pts[0];
        int offset = 0, controls = n - 1;
        P2 tan;
        for (;;) {
            offset++;
            tan = mk(first.x - pts[offset].x, first.y - pts[offset].y);
            if (!is_zero(tan)) break;
            controls--;
            if (controls == 0) break;
        }
        if (is_zero(tan)) { tan = mk(1.0f, 0.0f); controls = n - 1; }
        else normalize(tan);
        offset = 0;
        for (;;) {
            pts[offset].x += tan.x * outset;
            pts[offset].y += tan.y * outset;
            offset++;
            controls++;
            if (controls >= n) break;
        }
    }
    if (next_verb == V_MOVE || next_verb == V_CLOSE || next_verb == V_NONE) {
        P2 last = pts[n - 1];
        int offset = n - 1, controls = n - 1;
        P2 tan;
        for (;;) {
            offset--;
            tan = mk(last.x - pts[offset].x, last.y - pts[offset].y);
            if (!is_zero(tan)) break;
            controls--;
            if (controls == 0) break;
        }
        if (is_zero(tan)) { tan = mk(-1.0f, 0.0f); controls = n - 1; }
        else normalize(tan);
        offset = n - 1;
        for (;;) {
            pts[offset].x += tan.x * outset;
            pts[offset].y += tan.y * outset;
            offset--;
            controls++;
            if (controls >= n) break;
        }
    }
}

}  // namespace

bool treat_as_hairline(bool anti_alias, float width, const Xf &ts, float *coverage) {
    if (width == 0.0f) { *coverage = 1.0f; return true; }
    if (!anti_alias) return false;
    // lengths of (width, 0) and (0, width) under the linear part of ts, by the
    // cheap estimate max + min/2
    auto fast_len = [](float x, float y) {
        x = std::fabs(x); y = std::fabs(y);
        if (x < y) std::swap(x, y);
        return x + y * 0.5f;
    };
    Xf t = ts;
    t.tx = 0.0f; t.ty = 0.0f;
    P2 pts[2] = {mk(width, 0.0f), mk(0.0f, width)};
    map_points(t, pts, 2);
    const float len0 = fast_len(pts[0].x, pts[0].y), len1 = fast_len(pts[1].x, pts[1].y);
    if (len0 <= 1.0f && len1 <= 1.0f) {
        *coverage = (len0 + len1) * 0.5f;
        return true;
    }
    return false;
}

float hairline_opacity(float coverage) {
    const int32_t scale = (int32_t)(coverage * 256.0f);
    const int32_t new_alpha = (255 * scale) >> 8;
    return (float)new_alpha / 255.0f;
}

void hairline_calls(const PathData &path, const Xf &ts, uint32_t cap, int32_t clip_w, int32_t clip_h,
                    std::vector<HairCall> &out) {
    const size_t npts = path.pts.size() / 2;
    if (path.verbs.empty() || npts == 0) return;
    std::vector<P2> P(npts);
    for (size_t i = 0; i < npts; i++) P[i] = mk(path.pts[2 * i], path.pts[2 * i + 1]);
    map_points(ts, P.data(), npts);  // Path::transform
    FRect bounds;
    if (!curve_bounds(P.data(), (int)npts, &bounds)) return;
    // stroke_path_impl
    const IRect clip{0, 0, clip_w, clip_h};
    const float cap_out = cap == 0 ? 1.0f : 2.0f;
    IRect ib;
    if (!round_out(FRect{bounds.l - cap_out, bounds.t - cap_out, bounds.r + cap_out, bounds.b + cap_out}, &ib)) return;
    if (!intersects(clip, ib)) return;
    FRect inset{}, outset{};
    bool have_inset = false;
    if (!contains(clip, ib)) {
        outset = FRect{-1.0f, -1.0f, (float)clip_w + 1.0f, (float)clip_h + 1.0f};
        if (clip_w > 2 && clip_h > 2) {
            inset = FRect{1.0f, 1.0f, (float)clip_w - 1.0f, (float)clip_h - 1.0f};
            have_inset = true;
        } else {
            return;  // ScreenIntRect::inset(1, 1) of a <= 2 px target fails: nothing is drawn
        }
    }
    Emitter em{out, true, clip};
    uint8_t prev_verb = V_MOVE;
    P2 first_pt, last_pt;
    size_t pi = 0;
    const size_t nv = path.verbs.size();
    for (size_t vi = 0; vi < nv; vi++) {
        const uint8_t verb = path.verbs[vi];
        const uint8_t next_verb = vi + 1 < nv ? path.verbs[vi + 1] : V_NONE;
        P2 moved_start = last_pt;
        switch (verb) {
        case V_MOVE:
            first_pt = last_pt = P[pi];
            moved_start = P[pi];
            pi += 1;
            break;
        case V_LINE: {
            P2 pts[2] = {last_pt, P[pi]};
            pi += 1;
            if (cap != 0) extend_pts(cap, prev_verb, next_verb, pts, 2);
            line_proc(pts, 2, true, em);
            last_pt = P[pi - 1];
            moved_start = pts[0];
            break;
        }
        case V_QUAD: {
            P2 pts[3] = {last_pt, P[pi], P[pi + 1]};
            pi += 2;
            if (cap != 0) extend_pts(cap, prev_verb, next_verb, pts, 3);
            hair_quad(pts, true, have_inset ? &inset : nullptr, have_inset ? &outset : nullptr, quad_level(pts), em);
            last_pt = P[pi - 1];
            moved_start = pts[0];
            break;
        }
        case V_CUBIC: {
            P2 pts[4] = {last_pt, P[pi], P[pi + 1], P[pi + 2]};
            pi += 3;
            if (cap != 0) extend_pts(cap, prev_verb, next_verb, pts, 4);
            hair_cubic(pts, true, have_inset ? &inset : nullptr, have_inset ? &outset : nullptr, em);
            last_pt = P[pi - 1];
            moved_start = pts[0];
            break;
        }
        case V_CLOSE: {
            P2 pts[2] = {last_pt, first_pt};
            if (cap != 0 && prev_verb == V_MOVE) extend_pts(cap, prev_verb, next_verb, pts, 2);
            line_proc(pts, 2, true, em);
            moved_start = pts[0];
            last_pt = first_pt;
            break;
        }
        default: break;
        }
        if (cap != 0) {
            if (prev_verb == V_MOVE && (verb == V_LINE || verb == V_QUAD || verb == V_CUBIC))
                first_pt = moved_start;  // the curve moved the initial point: close to it instead
            prev_verb = verb;
        }
    }
}

namespace {

inline int32_t contribution_64(int32_t o) { return ((o - 1) & 63) + 1; }
inline int32_t fast_div16(int32_t a, int32_t b) {
    if (a >= -32768 && a <= 32767) return (int32_t)((uint32_t)a << 16) / b;
    int64_t v = ((int64_t)a << 16) / b;
    return (int32_t)std::min<int64_t>(std::max<int64_t>(v, INT32_MIN), INT32_MAX);
}
inline int32_t ceil16(int32_t x) { return (int32_t)(((int64_t)x + 0xFFFF) >> 16); }

void setup_span(int32_t x0, int32_t y0, int32_t x1, int32_t y1, bool clip_on, int32_t cl, int32_t ct, int32_t cr,
                int32_t cb, std::vector<HairSpan> &out) {
    if (x0 == INT32_MIN || y0 == INT32_MIN || x1 == INT32_MIN || y1 == INT32_MIN) return;
    if (std::abs(x1 - x0) > 511 * 64 || std::abs(y1 - y0) > 511 * 64) {
        const int32_t hx = (x0 >> 1) + (x1 >> 1), hy = (y0 >> 1) + (y1 >> 1);
        setup_span(x0, y0, hx, hy, clip_on, cl, ct, cr, cb, out);
        setup_span(hx, hy, x1, y1, clip_on, cl, ct, cr, cb, out);
        return;
    }
    HairSpan sp{};
    int32_t kind, scale_start, scale_stop, istart, istop, fstart, slope;
    const bool horiz = std::abs(x1 - x0) > std::abs(y1 - y0);
    if (horiz) {
        if (x0 > x1) { std::swap(x0, x1); std::swap(y0, y1); }
        istart = x0 >> 6;
        istop = (x1 + 63) >> 6;
        fstart = (int32_t)((uint32_t)y0 << 10);
        if (y0 == y1) { slope = 0; kind = 0; }
        else {
            slope = fast_div16(y1 - y0, x1 - x0);
            fstart += (slope * (32 - (x0 & 63)) + 32) >> 6;
            kind = 1;
        }
        if (istop - istart == 1) { scale_start = x1 - x0; scale_stop = 0; }
        else { scale_start = 64 - (x0 & 63); scale_stop = x1 & 63; }
        if (clip_on) {
            if (istart >= cr || istop <= cl) return;
            if (istart < cl) {
                fstart += slope * (cl - istart);
                istart = cl;
                scale_start = 64;
                if (istop - istart == 1) { scale_start = contribution_64(x1); scale_stop = 0; }
            }
            if (istop > cr) { istop = cr; scale_stop = 0; }
            if (istart == istop) return;
            int32_t top, bottom;
            if (slope >= 0) {
                top = (fstart - (1 << 15)) >> 16;
                bottom = ceil16(fstart + (istop - istart - 1) * slope + (1 << 15));
            } else {
                bottom = ceil16(fstart + (1 << 15));
                top = (fstart + (istop - istart - 1) * slope - (1 << 15)) >> 16;
            }
            top -= 1;
            bottom += 1;
            if (top >= cb || bottom <= ct) return;
            if (ct <= top && cb >= bottom) clip_on = false;
        }
    } else {
        if (y0 > y1) { std::swap(x0, x1); std::swap(y0, y1); }
        istart = y0 >> 6;
        istop = (y1 + 63) >> 6;
        fstart = (int32_t)((uint32_t)x0 << 10);
        if (x0 == x1) {
            if (y0 == y1) return;
            slope = 0;
            kind = 2;
        } else {
            slope = fast_div16(x1 - x0, y1 - y0);
            fstart += (slope * (32 - (y0 & 63)) + 32) >> 6;
            kind = 3;
        }
        if (istop - istart == 1) { scale_start = y1 - y0; scale_stop = 0; }
        else { scale_start = 64 - (y0 & 63); scale_stop = y1 & 63; }
        if (clip_on) {
            if (istart >= cb || istop <= ct) return;
            if (istart < ct) {
                fstart += slope * (ct - istart);
                istart = ct;
                scale_start = 64;
                if (istop - istart == 1) { scale_start = contribution_64(y1); scale_stop = 0; }
            }
            if (istop > cb) { istop = cb; scale_stop = 0; }
            if (istart == istop) return;
            int32_t left, right;
            if (slope >= 0) {
                left = (fstart - (1 << 15)) >> 16;
                right = ceil16(fstart + (istop - istart - 1) * slope + (1 << 15));
            } else {
                right = ceil16(fstart + (1 << 15));
                left = (fstart + (istop - istart - 1) * slope - (1 << 15)) >> 16;
            }
            left -= 1;
            right += 1;
            if (left >= cr || right <= cl) return;
            if (cl <= left && cr >= right) clip_on = false;
        }
    }
    const int32_t n = istop - istart;
    sp.istart = istart;
    sp.f0 = fstart + (1 << 15);
    sp.slope = slope;
    sp.pack = (uint32_t)kind | (uint32_t)scale_start << 2 | (uint32_t)scale_stop << 9 | (uint32_t)n << 16;
    // bounds of the pixels touched: the minor coordinate runs monotonically
    auto clamped = [&](int32_t k) -> int64_t {
        return slope >= 0 ? (int64_t)std::max(sp.f0, 0) + (int64_t)k * slope
                          : std::max<int64_t>((int64_t)sp.f0 + (int64_t)k * slope, 0);
    };
    const int64_t h0 = clamped(0) >> 16, h1 = clamped(n - 1) >> 16;
    const int32_t lo = (int32_t)std::max<int64_t>(std::min(h0, h1) - 1, 0);
    const int32_t hi = (int32_t)std::min<int64_t>(std::max(h0, h1) + 2, INT32_MAX);
    if (kind < 2) { sp.x0 = istart; sp.x1 = istop; sp.y0 = lo; sp.y1 = hi; }
    else { sp.y0 = istart; sp.y1 = istop; sp.x0 = lo; sp.x1 = hi; }
    if (clip_on) {
        sp.x0 = std::max(sp.x0, cl); sp.y0 = std::max(sp.y0, ct);
        sp.x1 = std::min(sp.x1, cr); sp.y1 = std::min(sp.y1, cb);
    }
    if (sp.x0 >= sp.x1 || sp.y0 >= sp.y1) return;
    out.push_back(sp);
    // vline: column hi gets alpha, then column max(hi, 1) - 1 gets 255 - alpha;
    // the same column when hi = 0, which a second span draws
    if (kind == 2 && h0 == 0) {
        sp.pack |= HAIR_SECOND;
        out.push_back(sp);
    }
}

}  // namespace

void hairline_spans(const HairCall &c, std::vector<HairSpan> &out) {
    setup_span(c.x0, c.y0, c.x1, c.y1, c.has_clip != 0, c.clip_l, c.clip_t, c.clip_r, c.clip_b, out);
}

}  // namespace rgpu
