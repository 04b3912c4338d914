// Host-side path geometry: tight bounds, stroking and dashing (see geom.h).
//
// The stroker follows the structure of Skia's SkStroke as used by
// tiny-skia-path's PathStroker: per contour it builds an "outer" and an
// "inner" offset polyline, joins at vertices (miter with limit, round,
// bevel, miter-clip), caps on open contours (butt, round, square), and emits
// outer + reversed inner as closed outlines for a non-zero fill.  Curves are
// flattened first at a tolerance tied to the device resolution scale; the
// resulting outline therefore differs from tiny-skia's quad-offset curves by
// sub-pixel amounts (measured by the stroke golden tests).
#include "geom.h"
#include <algorithm>
#include <cmath>

namespace rgpu {

namespace {
struct V2 { double x, y; };
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator*(V2 a, double s) { return {a.x * s, a.y * s}; }
inline double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
inline double cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
inline double len(V2 a) { return std::sqrt(a.x * a.x + a.y * a.y); }
inline V2 norm(V2 a) { double l = len(a); return l > 0 ? a * (1.0 / l) : V2{0, 0}; }
inline V2 perp(V2 a) { return {-a.y, a.x}; }  // rotate +90

// A contour flattened into a polyline.  `smooth[i]` marks vertex i as interior
// to a curve (no user-visible join there).
struct Poly {
    std::vector<V2> p;
    std::vector<uint8_t> smooth;
    bool closed = false;
    bool has_seg = false;
};

void flatten_cubic(Poly &pl, V2 p0, V2 p1, V2 p2, V2 p3, double tol) {
    V2 dd1 = p0 - p1 * 2.0 + p2, dd2 = p1 - p2 * 2.0 + p3;
    double dd = std::max(len(dd1), len(dd2));
    int n = (int)std::ceil(std::sqrt(0.75 * dd / tol));
    n = std::max(1, std::min(n, 1024));
    for (int i = 1; i <= n; i++) {
        double t = (double)i / n, mt = 1.0 - t;
        V2 q = p0 * (mt * mt * mt) + p1 * (3 * mt * mt * t) + p2 * (3 * mt * t * t) + p3 * (t * t * t);
        pl.p.push_back(q);
        pl.smooth.push_back(i < n ? 1 : 0);
    }
}
void flatten_quad(Poly &pl, V2 p0, V2 p1, V2 p2, double tol) {
    V2 dd = p0 - p1 * 2.0 + p2;
    int n = (int)std::ceil(std::sqrt(0.25 * len(dd) / tol));
    n = std::max(1, std::min(n, 1024));
    for (int i = 1; i <= n; i++) {
        double t = (double)i / n, mt = 1.0 - t;
        V2 q = p0 * (mt * mt) + p1 * (2 * mt * t) + p2 * (t * t);
        pl.p.push_back(q);
        pl.smooth.push_back(i < n ? 1 : 0);
    }
}

std::vector<Poly> flatten(const uint8_t *verbs, size_t nv, const float *pts, double tol) {
    std::vector<Poly> out;
    Poly cur;
    size_t pi = 0;
    V2 last{0, 0}, start{0, 0};
    auto flush = [&]() {
        if (!cur.p.empty()) out.push_back(cur);
        cur = Poly();
    };
    for (size_t i = 0; i < nv; i++) {
        switch (verbs[i]) {
        case 0:
            flush();
            last = start = V2{pts[pi * 2], pts[pi * 2 + 1]}; pi++;
            cur.p.push_back(last); cur.smooth.push_back(0);
            break;
        case 1: {
            V2 q{pts[pi * 2], pts[pi * 2 + 1]}; pi++;
            if (cur.p.empty()) { cur.p.push_back(last); cur.smooth.push_back(0); }
            cur.p.push_back(q); cur.smooth.push_back(0); last = q; cur.has_seg = true;
            break;
        }
        case 2: {
            V2 a{pts[pi * 2], pts[pi * 2 + 1]}, b{pts[pi * 2 + 2], pts[pi * 2 + 3]}; pi += 2;
            if (cur.p.empty()) { cur.p.push_back(last); cur.smooth.push_back(0); }
            flatten_quad(cur, last, a, b, tol); last = b; cur.has_seg = true;
            break;
        }
        case 3: {
            V2 a{pts[pi * 2], pts[pi * 2 + 1]}, b{pts[pi * 2 + 2], pts[pi * 2 + 3]}, c{pts[pi * 2 + 4], pts[pi * 2 + 5]};
            pi += 3;
            if (cur.p.empty()) { cur.p.push_back(last); cur.smooth.push_back(0); }
            flatten_cubic(cur, last, a, b, c, tol); last = c; cur.has_seg = true;
            break;
        }
        case 4:
            if (cur.has_seg) cur.closed = true;
            flush();
            last = start;
            break;
        }
    }
    flush();
    return out;
}

// Remove zero-length segments; keep the smooth flag of the surviving vertex.
void dedupe(Poly &pl) {
    Poly o;
    o.closed = pl.closed;
    o.has_seg = pl.has_seg;
    for (size_t i = 0; i < pl.p.size(); i++) {
        if (!o.p.empty() && len(pl.p[i] - o.p.back()) <= 1e-9) { o.smooth.back() = pl.smooth[i] && o.smooth.back(); continue; }
        o.p.push_back(pl.p[i]);
        o.smooth.push_back(pl.smooth[i]);
    }
    if (o.closed && o.p.size() > 1 && len(o.p.back() - o.p.front()) <= 1e-9) {
        o.p.pop_back();
        o.smooth.pop_back();
    }
    pl = o;
}

struct Out {
    PathData &pd;
    void move(V2 p) { pd.move_to((float)p.x, (float)p.y); }
    void line(V2 p) { pd.line_to((float)p.x, (float)p.y); }
    void cubic(V2 a, V2 b, V2 c) { pd.cubic_to((float)a.x, (float)a.y, (float)b.x, (float)b.y, (float)c.x, (float)c.y); }
    void close() { pd.close(); }
};

// Circular arc around `c` from direction `a` to `b` (unit vectors), radius r,
// turning in the sign of `sweep` (+1 ccw in y-down = clockwise visually).
void arc(std::vector<V2> &poly, V2 c, V2 a, V2 b, double r, double sweep_sign, double tol) {
    double ang0 = std::atan2(a.y, a.x);
    double ang1 = std::atan2(b.y, b.x);
    double d = ang1 - ang0;
    if (sweep_sign > 0) { while (d <= 0) d += 2 * M_PI; }
    else { while (d >= 0) d -= 2 * M_PI; }
    double step = 2.0 * std::acos(std::max(-1.0, std::min(1.0, 1.0 - tol / std::max(r, 1e-9))));
    if (!(step > 1e-3)) step = 1e-3;
    int n = (int)std::ceil(std::fabs(d) / step);
    n = std::max(1, std::min(n, 1024));
    for (int i = 1; i <= n; i++) {
        double t = ang0 + d * i / n;
        poly.push_back(V2{c.x + r * std::cos(t), c.y + r * std::sin(t)});
    }
}

// Offsets one side of the polyline (sign +1: left normal, -1: right).  The
// side is built as a point list including joins.
void offset_side(const Poly &pl, double hw, const StrokeStyle &st, double tol, double sign, std::vector<V2> &side) {
    size_t n = pl.p.size();
    size_t segs = pl.closed ? n : n - 1;
    auto dir = [&](size_t s) { return norm(pl.p[(s + 1) % n] - pl.p[s]); };
    for (size_t s = 0; s < segs; s++) {
        V2 d = dir(s);
        V2 nrm = perp(d) * (hw * sign);
        V2 a = pl.p[s] + nrm, b = pl.p[(s + 1) % n] + nrm;
        if (s == 0 && !pl.closed) side.push_back(a);
        if (s == 0 && pl.closed) {
            // the join at vertex 0 is produced at the end
            side.push_back(a);
        }
        side.push_back(b);
        // join at vertex s+1
        bool last = (s + 1 == segs);
        if (last && !pl.closed) break;
        size_t v = (s + 1) % n;
        V2 d1 = dir((s + 1) % segs);
        V2 n1 = perp(d1) * (hw * sign);
        double turn = cross(d, d1) * sign;  // >0: this side is the inner side of the turn
        double dp = dot(d, d1);
        if (pl.smooth[v] || std::fabs(cross(d, d1)) < 1e-12) {
            // continuation of a flattened curve: intersection of the offset lines
            V2 m = norm(perp(d) + perp(d1));
            double c = dot(m, perp(d));
            if (c > 0.05) {
                side.back() = pl.p[v] + m * (hw * sign / c);
            } else {
                side.push_back(pl.p[v] + n1);
            }
            continue;
        }
        if (turn > 0) {
            // inner side: pivot connection (as Skia's inner joiner)
            side.push_back(pl.p[v]);
            side.push_back(pl.p[v] + n1);
            continue;
        }
        // outer side
        V2 p = pl.p[v];
        switch (st.join) {
        case 2: {  // round
            std::vector<V2> tmp;
            arc(tmp, p, norm(nrm), norm(n1), hw, cross(nrm, n1) >= 0 ? 1 : -1, tol);
            side.insert(side.end(), tmp.begin(), tmp.end());
            break;
        }
        case 3:  // bevel
            side.push_back(p + n1);
            break;
        default: {  // miter / miter-clip
            double cos_half = std::sqrt(std::max(0.0, (1.0 + dp) * 0.5));
            V2 mid = norm(norm(nrm) + norm(n1));
            if (cos_half > 1e-9 && 1.0 / cos_half <= st.miter_limit) {
                side.push_back(p + mid * (hw / cos_half));
                side.push_back(p + n1);
            } else if (st.join == 1 && cos_half > 1e-9) {
                // miter-clip: clip the miter at miter_limit * hw / 2 from the pivot
                double clipd = st.miter_limit * hw * 0.5;
                V2 tip = p + mid * (hw / cos_half);
                V2 e0 = p + nrm, e1 = p + n1;
                double dist_tip = hw / cos_half;
                double t = (clipd - dot(e0 - p, mid)) / std::max(1e-12, dist_tip - dot(e0 - p, mid));
                t = std::max(0.0, std::min(1.0, t));
                side.push_back(e0 + (tip - e0) * t);
                side.push_back(e1 + (tip - e1) * t);
                side.push_back(e1);
            } else {
                side.push_back(p + n1);
            }
        }
        }
    }
    if (pl.closed && !side.empty()) side.push_back(side.front());
}

void add_cap(std::vector<V2> &poly, V2 p, V2 d, double hw, uint32_t cap, double tol) {
    // cap at endpoint p, travelling in direction d (outward), from left side to right side
    V2 nl = perp(d) * hw;  // left of travel direction... (y-down: perp rotates +90)
    V2 from = p + nl, to = p - nl;
    if (cap == 1) {
        arc(poly, p, norm(nl), norm(nl * -1.0), hw, cross(nl, d) >= 0 ? -1 : 1, tol);
        (void)from;
        poly.back() = to;
    } else if (cap == 2) {
        poly.push_back(from + d * hw);
        poly.push_back(to + d * hw);
        poly.push_back(to);
    } else {
        poly.push_back(to);
    }
}
}  // namespace

float resolution_scale(float sx, float ky, float kx, float sy) {
    float a = std::sqrt(sx * sx + kx * kx), b = std::sqrt(ky * ky + sy * sy);
    if (std::isfinite(a) && std::isfinite(b)) {
        float s = std::max(a, b);
        if (s > 0) return s;
    }
    return 1.0f;
}

bool tight_bounds(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, float out[4]) {
    if (npts == 0) return false;
    double l = 1e300, t = 1e300, r = -1e300, b = -1e300;
    auto add = [&](double x, double y) { l = std::min(l, x); r = std::max(r, x); t = std::min(t, y); b = std::max(b, y); };
    size_t pi = 0;
    double lx = 0, ly = 0;
    for (size_t i = 0; i < nv; i++) {
        switch (verbs[i]) {
        case 0: lx = pts[pi * 2]; ly = pts[pi * 2 + 1]; pi++; add(lx, ly); break;
        case 1: lx = pts[pi * 2]; ly = pts[pi * 2 + 1]; pi++; add(lx, ly); break;
        case 2: {
            double x1 = pts[pi * 2], y1 = pts[pi * 2 + 1], x2 = pts[pi * 2 + 2], y2 = pts[pi * 2 + 3];
            pi += 2;
            add(x2, y2);
            for (int k = 0; k < 2; k++) {
                double a = k ? ly : lx, c1 = k ? y1 : x1, c2 = k ? y2 : x2;
                double den = a - 2 * c1 + c2;
                if (den != 0) {
                    double tt = (a - c1) / den;
                    if (tt > 0 && tt < 1) {
                        double mt = 1 - tt;
                        add(mt * mt * lx + 2 * mt * tt * x1 + tt * tt * x2, mt * mt * ly + 2 * mt * tt * y1 + tt * tt * y2);
                    }
                }
            }
            lx = x2; ly = y2;
            break;
        }
        case 3: {
            double x1 = pts[pi * 2], y1 = pts[pi * 2 + 1], x2 = pts[pi * 2 + 2], y2 = pts[pi * 2 + 3];
            double x3 = pts[pi * 2 + 4], y3 = pts[pi * 2 + 5];
            pi += 3;
            add(x3, y3);
            for (int k = 0; k < 2; k++) {
                double p0 = k ? ly : lx, p1 = k ? y1 : x1, p2 = k ? y2 : x2, p3 = k ? y3 : x3;
                double A = -p0 + 3 * p1 - 3 * p2 + p3, B = 2 * (p0 - 2 * p1 + p2), C = p1 - p0;
                double roots[2]; int nr = 0;
                if (std::fabs(A) < 1e-12) { if (B != 0) roots[nr++] = -C / B; }
                else {
                    double disc = B * B - 4 * A * C;
                    if (disc >= 0) { double s = std::sqrt(disc); roots[nr++] = (-B + s) / (2 * A); roots[nr++] = (-B - s) / (2 * A); }
                }
                for (int j = 0; j < nr; j++) {
                    double tt = roots[j];
                    if (tt > 0 && tt < 1) {
                        double mt = 1 - tt;
                        double x = mt * mt * mt * lx + 3 * mt * mt * tt * x1 + 3 * mt * tt * tt * x2 + tt * tt * tt * x3;
                        double y = mt * mt * mt * ly + 3 * mt * mt * tt * y1 + 3 * mt * tt * tt * y2 + tt * tt * tt * y3;
                        add(x, y);
                    }
                }
            }
            lx = x3; ly = y3;
            break;
        }
        default: break;
        }
    }
    if (!(l <= r && t <= b) || !std::isfinite(l) || !std::isfinite(r) || !std::isfinite(t) || !std::isfinite(b))
        return false;
    out[0] = (float)l; out[1] = (float)t; out[2] = (float)(r - l); out[3] = (float)(b - t);
    return true;
}

}  // namespace rgpu
