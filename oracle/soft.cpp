// FP64 reference of the differentiable soft-coverage renderer (TEST
// INFRASTRUCTURE ONLY: the checker of resvg_gb300/csrc/kernels/soft.cu, never
// linked into the product).
//
// It restates the same definitions in double precision: loops closed by
// construction (3n points for n cubics, the last cubic ending at the start),
// flattening of each cubic into 16 lines at uniform t, the winding-weighted pixel area of every
// clipped line (sdy * mean of clamp(1 - x, 0, 1) over the line's x range
// relative to the pixel), soft coverage min(|A|, 1), solid / 4-stop linear
// gradient paints whose alpha is multiplied by the path's opacity,
// premultiplied after interpolation, source-over in path
// order, a separable Gaussian blur of radius 12 with weights normalised over
// the kernel and zero outside the canvas, and the mean squared error.
//
// Gradients come from forward-mode dual numbers (value + one tangent) run
// through the same code: dloss/dv for a direction v over all parameters.
// This is independent of the device adjoint (reverse mode, hand-written).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "resvg_gpu.h"

namespace {

struct Dd {
    double v, d;
};
inline Dd D(double v, double d = 0.0) { return Dd{v, d}; }
inline Dd operator+(Dd a, Dd b) { return D(a.v + b.v, a.d + b.d); }
inline Dd operator-(Dd a, Dd b) { return D(a.v - b.v, a.d - b.d); }
inline Dd operator*(Dd a, Dd b) { return D(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dd operator/(Dd a, Dd b) { return D(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline Dd operator+(Dd a, double b) { return D(a.v + b, a.d); }
inline Dd operator-(Dd a, double b) { return D(a.v - b, a.d); }
inline Dd operator-(double a, Dd b) { return D(a - b.v, -b.d); }
inline Dd operator*(Dd a, double b) { return D(a.v * b, a.d * b); }
inline Dd operator*(double a, Dd b) { return D(a * b.v, a * b.d); }
inline Dd operator/(Dd a, double b) { return D(a.v / b, a.d / b); }
inline double val(double x) { return x; }
inline double val(Dd x) { return x.v; }
inline Dd dexp(Dd a) { double e = std::exp(a.v); return D(e, e * a.d); }
inline double dexp(double a) { return std::exp(a); }
template <class T> T cst(double v);
template <> double cst<double>(double v) { return v; }
template <> Dd cst<Dd>(double v) { return D(v); }
template <class T> T tmin(T a, T b) { return val(a) <= val(b) ? a : b; }
template <class T> T tmax(T a, T b) { return val(a) >= val(b) ? a : b; }
template <class T> T tabs(T a) { return val(a) < 0 ? cst<T>(0.0) - a : a; }

constexpr int kFlat = 16;
constexpr int kRadius = 12;

template <class T>
T mean_right(T a, T b) {
    if (val(a) > val(b)) std::swap(a, b);
    if (val(b) <= 0.0) return cst<T>(1.0);
    if (val(a) >= 1.0) return cst<T>(0.0);
    if (val(a) >= 0.0 && val(b) <= 1.0) return 1.0 - (a + b) * 0.5;
    if (val(a) < 0.0 && val(b) <= 1.0) return 1.0 - (b * b) / ((b - a) * 2.0);
    if (val(a) >= 0.0) return ((1.0 - a) * (1.0 - a)) / ((b - a) * 2.0);
    return (0.5 - a) / (b - a);
}

template <class T>
bool clip_row(T x0, T y0, T x1, T y1, double py, T *xl, T *xh, T *sdy) {
    if (val(y0) == val(y1)) return false;
    const double dir = val(y1) > val(y0) ? 1.0 : -1.0;
    T xa = x0, ya = y0, xb = x1, yb = y1;
    if (dir < 0) { xa = x1; ya = y1; xb = x0; yb = y0; }
    if (!(val(ya) < py + 1.0 && val(yb) > py)) return false;
    T ylo, yhi;
    if (val(ya) >= py) { ylo = ya; *xl = xa; }
    else { ylo = cst<T>(py); *xl = xa + (xb - xa) * ((py - ya) / (yb - ya)); }
    if (val(yb) <= py + 1.0) { yhi = yb; *xh = xb; }
    else { yhi = cst<T>(py + 1.0); *xh = xa + (xb - xa) * (((py + 1.0) - ya) / (yb - ya)); }
    if (!(val(yhi) > val(ylo))) return false;
    *sdy = (yhi - ylo) * dir;
    return true;
}

struct Host {
    const rgpu_soft_batch &b;
    uint32_t npaths() const { return b.scenes * b.paths_per_scene; }
};

template <class T>
struct Params {
    std::vector<T> pts, colors, offsets, stops, sigma, opacity;
};

template <class T>
void render(const rgpu_soft_batch &b, const Params<T> &pr, std::vector<T> &image, std::vector<T> &blurred) {
    const uint32_t S = b.scenes, W = b.width, H = b.height, P = b.paths_per_scene;
    image.assign((size_t)S * W * H * 4, cst<T>(0.0));
    blurred.assign(image.size(), cst<T>(0.0));
    for (uint32_t s = 0; s < S; s++) {
        // flatten
        std::vector<std::vector<T>> vx(P), vy(P);
        for (uint32_t p = 0; p < P; p++) {
            const uint32_t j = s * P + p;
            const uint32_t s0 = b.seg_offset[j], ns = b.seg_offset[j + 1] - s0;
            const size_t base = 3 * (size_t)s0;
            auto X = [&](size_t q) { return pr.pts[2 * (base + q)]; };
            auto Y = [&](size_t q) { return pr.pts[2 * (base + q) + 1]; };
            for (uint32_t c = 0; c < ns; c++) {
                const size_t e = c + 1 < ns ? 3 * c + 3 : 0;  // the last cubic ends at the start
                for (int i = 0; i < kFlat; i++) {
                    const double t = (double)i / kFlat, u = 1.0 - t;
                    const double b0 = u * u * u, b1 = 3 * u * u * t, b2 = 3 * u * t * t, b3 = t * t * t;
                    vx[p].push_back(b0 * X(3 * c) + b1 * X(3 * c + 1) + b2 * X(3 * c + 2) + b3 * X(e));
                    vy[p].push_back(b0 * Y(3 * c) + b1 * Y(3 * c + 1) + b2 * Y(3 * c + 2) + b3 * Y(e));
                }
            }
        }
        for (uint32_t py = 0; py < H; py++) {
            std::vector<T> C((size_t)W * 4, cst<T>(0.0));
            for (uint32_t p = 0; p < P; p++) {
                const uint32_t j = s * P + p;
                const size_t nv = vx[p].size();
                struct Cr { T xl, xh, sdy; };
                std::vector<Cr> cr;
                for (size_t l = 0; l < nv; l++) {
                    const size_t m = l + 1 < nv ? l + 1 : 0;
                    T xl, xh, sdy;
                    if (clip_row<T>(vx[p][l], vy[p][l], vx[p][m], vy[p][m], (double)py, &xl, &xh, &sdy))
                        cr.push_back(Cr{xl, xh, sdy});
                }
                if (cr.empty()) continue;
                for (uint32_t x = 0; x < W; x++) {
                    T A = cst<T>(0.0);
                    for (auto &c : cr) A = A + c.sdy * mean_right<T>(c.xl - (double)x, c.xh - (double)x);
                    T c = tmin<T>(tabs<T>(A), cst<T>(1.0));
                    if (val(c) == 0.0) continue;
                    // paint at the pixel centre
                    T r, g, bb, a;
                    const double cx = x + 0.5, cy = py + 0.5;
                    if (b.paint_kind[j] == 0) {
                        r = pr.colors[4 * j]; g = pr.colors[4 * j + 1]; bb = pr.colors[4 * j + 2]; a = pr.colors[4 * j + 3];
                    } else {
                        const float *ln = b.grad_line + 4 * (size_t)j;
                        const double dx = (double)ln[2] - ln[0], dy = (double)ln[3] - ln[1];
                        const double len2 = dx * dx + dy * dy;
                        double t = len2 > 0 ? ((cx - ln[0]) * dx + (cy - ln[1]) * dy) / len2 : 0.0;
                        t = std::fmin(std::fmax(t, 0.0), 1.0);
                        const T *off = &pr.offsets[4 * (size_t)j];
                        const T *sc = &pr.stops[16 * (size_t)j];
                        auto pick = [&](int i) { r = sc[4 * i]; g = sc[4 * i + 1]; bb = sc[4 * i + 2]; a = sc[4 * i + 3]; };
                        if (t < val(off[0])) pick(0);
                        else if (t >= val(off[3])) pick(3);
                        else {
                            int i = 0;
                            if (t >= val(off[1])) i = 1;
                            if (t >= val(off[2])) i = 2;
                            const T span = off[i + 1] - off[i];
                            const T w = val(span) > 0 ? (t - off[i]) / span : cst<T>(1.0);
                            r = sc[4 * i] + w * (sc[4 * i + 4] - sc[4 * i]);
                            g = sc[4 * i + 1] + w * (sc[4 * i + 5] - sc[4 * i + 1]);
                            bb = sc[4 * i + 2] + w * (sc[4 * i + 6] - sc[4 * i + 2]);
                            a = sc[4 * i + 3] + w * (sc[4 * i + 7] - sc[4 * i + 3]);
                        }
                    }
                    a = a * pr.opacity[j];
                    const T ca = c * a, keep = 1.0 - ca;
                    T *cp = &C[4 * (size_t)x];
                    cp[0] = c * (r * a) + keep * cp[0];
                    cp[1] = c * (g * a) + keep * cp[1];
                    cp[2] = c * (bb * a) + keep * cp[2];
                    cp[3] = ca + keep * cp[3];
                }
            }
            for (uint32_t x = 0; x < W; x++)
                for (int k = 0; k < 4; k++) image[(((size_t)s * H + py) * W + x) * 4 + k] = C[4 * (size_t)x + k];
        }
        // blur: horizontal then vertical
        T sig = pr.sigma[s];
        std::vector<T> w(2 * kRadius + 1);
        T z = cst<T>(0.0);
        for (int j = -kRadius; j <= kRadius; j++) {
            w[j + kRadius] = dexp(cst<T>(-(double)(j * j)) / (sig * sig * 2.0));
            z = z + w[j + kRadius];
        }
        for (auto &v : w) v = v / z;
        std::vector<T> tmp((size_t)W * H * 4, cst<T>(0.0));
        const T *img = &image[(size_t)s * W * H * 4];
        for (uint32_t y = 0; y < H; y++)
            for (uint32_t x = 0; x < W; x++)
                for (int k = 0; k < 4; k++) {
                    T acc = cst<T>(0.0);
                    for (int j = -kRadius; j <= kRadius; j++) {
                        const int xx = (int)x + j;
                        if (xx < 0 || xx >= (int)W) continue;
                        acc = acc + w[j + kRadius] * img[((size_t)y * W + xx) * 4 + k];
                    }
                    tmp[((size_t)y * W + x) * 4 + k] = acc;
                }
        T *out = &blurred[(size_t)s * W * H * 4];
        for (uint32_t y = 0; y < H; y++)
            for (uint32_t x = 0; x < W; x++)
                for (int k = 0; k < 4; k++) {
                    T acc = cst<T>(0.0);
                    for (int j = -kRadius; j <= kRadius; j++) {
                        const int yy = (int)y + j;
                        if (yy < 0 || yy >= (int)H) continue;
                        acc = acc + w[j + kRadius] * tmp[((size_t)yy * W + x) * 4 + k];
                    }
                    out[((size_t)y * W + x) * 4 + k] = acc;
                }
    }
}

size_t npoints(const rgpu_soft_batch &b) { return 3 * (size_t)b.total_segments; }

}  // namespace

extern "C" {

// Forward in FP64: image and blurred (scenes x H x W x 4 doubles each).
int oracle_soft_forward(const rgpu_soft_batch *b, double *image, double *blurred) {
    const size_t np = (size_t)b->scenes * b->paths_per_scene;
    Params<double> pr;
    pr.pts.assign(b->points, b->points + 2 * npoints(*b));
    pr.colors.assign(b->colors, b->colors + 4 * np);
    pr.offsets.assign(b->stop_offsets, b->stop_offsets + 4 * np);
    pr.stops.assign(b->stop_colors, b->stop_colors + 16 * np);
    pr.sigma.assign(b->sigma, b->sigma + b->scenes);
    pr.opacity.assign(np, 1.0);
    if (b->opacity) pr.opacity.assign(b->opacity, b->opacity + np);
    std::vector<double> im, bl;
    render<double>(*b, pr, im, bl);
    std::memcpy(image, im.data(), im.size() * 8);
    std::memcpy(blurred, bl.data(), bl.size() * 8);
    return 0;
}

// Loss = mean squared error of the blurred image against `target`, and its
// directional derivative along the parameter direction (same layouts as the
// parameters), by forward-mode dual numbers in FP64.
int oracle_soft_dloss(const rgpu_soft_batch *b, const float *target, const double *d_points, const double *d_colors,
                      const double *d_offsets, const double *d_stops, const double *d_sigma,
                      const double *d_opacity, double *loss, double *dloss) {
    const size_t np = (size_t)b->scenes * b->paths_per_scene;
    Params<Dd> pr;
    auto load = [](std::vector<Dd> &v, const float *x, const double *d, size_t n) {
        v.resize(n);
        for (size_t i = 0; i < n; i++) v[i] = D(x[i], d ? d[i] : 0.0);
    };
    load(pr.pts, b->points, d_points, 2 * npoints(*b));
    load(pr.colors, b->colors, d_colors, 4 * np);
    load(pr.offsets, b->stop_offsets, d_offsets, 4 * np);
    load(pr.stops, b->stop_colors, d_stops, 16 * np);
    load(pr.sigma, b->sigma, d_sigma, b->scenes);
    if (b->opacity) {
        load(pr.opacity, b->opacity, d_opacity, np);
    } else {
        pr.opacity.assign(np, D(1.0));
    }
    std::vector<Dd> im, bl;
    render<Dd>(*b, pr, im, bl);
    Dd L = D(0.0);
    for (size_t i = 0; i < bl.size(); i++) {
        const Dd d = bl[i] - (double)target[i];
        L = L + d * d;
    }
    L = L / (double)bl.size();
    *loss = L.v;
    *dloss = L.d;
    return 0;
}

}  // extern "C"
