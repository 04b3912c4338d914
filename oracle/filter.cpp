// CPU oracle — test infrastructure only.
//
// Restatement of resvg 0.48.1's filter module:
//   crates/resvg/src/filter/mod.rs:115-308   colour spaces, multiply/demultiply, LUTs, Image
//   crates/resvg/src/filter/mod.rs:335-564   apply / apply_inner / get_input, subregion crop
//   crates/resvg/src/filter/mod.rs:645-666   apply_blur, :1119-1147 resolve_std_dev
//   crates/resvg/src/filter/mod.rs:731-793   apply_composite, :795-818 apply_merge
//   crates/resvg/src/filter/mod.rs:905-956   colour matrix, convolve, morphology drivers
//   crates/resvg/src/filter/mod.rs:1100-1114 apply_to_canvas
//   crates/resvg/src/filter/box_blur.rs       box blur (5 box passes, V then H)
//   crates/resvg/src/filter/iir_blur.rs       IIR blur (f64)
//   crates/resvg/src/filter/color_matrix.rs, morphology.rs, composite.rs, convolve_matrix.rs
//   crates/resvg/src/filter/lighting.rs        diffuse / specular lighting, mod.rs:1020-1098 drivers
//   crates/resvg/src/filter/component_transfer.rs  transfer functions, mod.rs:891-903 driver
//   crates/resvg/src/filter/mod.rs:581-649   apply_drop_shadow
//   crates/resvg/src/filter/turbulence.rs, mod.rs:988-1018 apply_turbulence
//   crates/resvg/src/filter/mod.rs:835-859 apply_tile, displacement_map.rs + mod.rs:958-986
// The two sRGB <-> linearRGB tables are resvg's (mod.rs:161-238): both are
// the standard transfer functions evaluated and rounded to u8 (a data table
// has to be identical to give identical output).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include "raster.h"

namespace ora {
void render_group_children(const rgpu_tree_view &t, uint32_t gi, const Transform &ts, Pixmap &pm);

namespace {

const uint8_t SRGB_TO_LINEAR[256] = {
    0,   0,   0,   0,   0,   0,   0,   1,   1,   1,   1,   1,   1,   1,   1,   1,   1,   1,   2,   2,   2,   2,
    2,   2,   2,   2,   3,   3,   3,   3,   3,   3,   4,   4,   4,   4,   4,   5,   5,   5,   5,   6,   6,   6,
    6,   7,   7,   7,   8,   8,   8,   8,   9,   9,   9,   10,  10,  10,  11,  11,  12,  12,  12,  13,  13,  13,
    14,  14,  15,  15,  16,  16,  17,  17,  17,  18,  18,  19,  19,  20,  20,  21,  22,  22,  23,  23,  24,  24,
    25,  25,  26,  27,  27,  28,  29,  29,  30,  30,  31,  32,  32,  33,  34,  35,  35,  36,  37,  37,  38,  39,
    40,  41,  41,  42,  43,  44,  45,  45,  46,  47,  48,  49,  50,  51,  51,  52,  53,  54,  55,  56,  57,  58,
    59,  60,  61,  62,  63,  64,  65,  66,  67,  68,  69,  70,  71,  72,  73,  74,  76,  77,  78,  79,  80,  81,
    82,  84,  85,  86,  87,  88,  90,  91,  92,  93,  95,  96,  97,  99,  100, 101, 103, 104, 105, 107, 108, 109,
    111, 112, 114, 115, 116, 118, 119, 121, 122, 124, 125, 127, 128, 130, 131, 133, 134, 136, 138, 139, 141, 142,
    144, 146, 147, 149, 151, 152, 154, 156, 157, 159, 161, 163, 164, 166, 168, 170, 171, 173, 175, 177, 179, 181,
    183, 184, 186, 188, 190, 192, 194, 196, 198, 200, 202, 204, 206, 208, 210, 212, 214, 216, 218, 220, 222, 224,
    226, 229, 231, 233, 235, 237, 239, 242, 244, 246, 248, 250, 253, 255};
const uint8_t LINEAR_TO_SRGB[256] = {
    0,   13,  22,  28,  34,  38,  42,  46,  50,  53,  56,  59,  61,  64,  66,  69,  71,  73,  75,  77,  79,  81,
    83,  85,  86,  88,  90,  92,  93,  95,  96,  98,  99,  101, 102, 104, 105, 106, 108, 109, 110, 112, 113, 114,
    115, 117, 118, 119, 120, 121, 122, 124, 125, 126, 127, 128, 129, 130, 131, 132, 133, 134, 135, 136, 137, 138,
    139, 140, 141, 142, 143, 144, 145, 146, 147, 148, 148, 149, 150, 151, 152, 153, 154, 155, 155, 156, 157, 158,
    159, 159, 160, 161, 162, 163, 163, 164, 165, 166, 167, 167, 168, 169, 170, 170, 171, 172, 173, 173, 174, 175,
    175, 176, 177, 178, 178, 179, 180, 180, 181, 182, 182, 183, 184, 185, 185, 186, 187, 187, 188, 189, 189, 190,
    190, 191, 192, 192, 193, 194, 194, 195, 196, 196, 197, 197, 198, 199, 199, 200, 200, 201, 202, 202, 203, 203,
    204, 205, 205, 206, 206, 207, 208, 208, 209, 209, 210, 210, 211, 212, 212, 213, 213, 214, 214, 215, 215, 216,
    216, 217, 218, 218, 219, 219, 220, 220, 221, 221, 222, 222, 223, 223, 224, 224, 225, 226, 226, 227, 227, 228,
    228, 229, 229, 230, 230, 231, 231, 232, 232, 233, 233, 234, 234, 235, 235, 236, 236, 237, 237, 238, 238, 238,
    239, 239, 240, 240, 241, 241, 242, 242, 243, 243, 244, 244, 245, 245, 246, 246, 246, 247, 247, 248, 248, 249,
    249, 250, 250, 251, 251, 251, 252, 252, 253, 253, 254, 254, 255, 255};

inline uint8_t sat_u8f(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}
inline uint8_t sat_u8d(double v) {
    if (!(v > 0.0)) return 0;
    if (v >= 255.0) return 255;
    return (uint8_t)v;
}
// mod.rs:242-254
inline float f32_bound(float mn, float v, float mx) {
    if (v > mx) return mx;
    if (v >= mn) return v;
    return mn;
}
void multiply_alpha(std::vector<uint8_t> &d) {
    for (size_t i = 0; i < d.size(); i += 4) {
        float a = d[i + 3] / 255.0f;
        d[i + 2] = sat_u8f(d[i + 2] * a + 0.5f);
        d[i + 1] = sat_u8f(d[i + 1] * a + 0.5f);
        d[i + 0] = sat_u8f(d[i + 0] * a + 0.5f);
    }
}
void demultiply_alpha(std::vector<uint8_t> &d) {
    for (size_t i = 0; i < d.size(); i += 4) {
        float a = d[i + 3] / 255.0f;
        d[i + 2] = sat_u8f(d[i + 2] / a + 0.5f);
        d[i + 1] = sat_u8f(d[i + 1] / a + 0.5f);
        d[i + 0] = sat_u8f(d[i + 0] / a + 0.5f);
    }
}
void into_linear(Pixmap &p) {
    demultiply_alpha(p.data);
    for (size_t i = 0; i < p.data.size(); i += 4)
        for (int k = 0; k < 3; k++) p.data[i + k] = SRGB_TO_LINEAR[p.data[i + k]];
    multiply_alpha(p.data);
}
void into_srgb(Pixmap &p) {
    demultiply_alpha(p.data);
    for (size_t i = 0; i < p.data.size(); i += 4)
        for (int k = 0; k < 3; k++) p.data[i + k] = LINEAR_TO_SRGB[p.data[i + k]];
    multiply_alpha(p.data);
}

struct Image {
    std::shared_ptr<Pixmap> image;
    IntRect region;
    bool linear;
};

Image into_cs(const Image &im, bool linear) {
    if (im.linear == linear) return im;
    auto p = std::make_shared<Pixmap>(*im.image);
    if (linear) into_linear(*p); else into_srgb(*p);
    return Image{p, im.region, linear};
}

// ---- box blur (box_blur.rs)
inline float fround(float x) {
    volatile float y = x + 12582912.0f;
    return y - 12582912.0f;
}
void create_box_gauss(float sigma, int sizes[5]) {
    if (sigma > 0.0f) {
        float n = 5.0f;
        float w_ideal = std::sqrt(12.0f * sigma * sigma / n) + 1.0f;
        int wl = (int)std::floor(w_ideal);
        if (wl % 2 == 0) wl -= 1;
        int wu = wl + 2;
        float wlf = (float)wl;
        float m_ideal = (12.0f * sigma * sigma - n * wlf * wlf - 4.0f * n * wlf - 3.0f * n) / (-4.0f * wlf - 4.0f);
        float mr = std::round(m_ideal);  // Rust f32::round: half away from zero
        int m = mr <= 0.0f ? 0 : (int)mr;  // `as usize` saturates at 0
        for (int i = 0; i < 5; i++) sizes[i] = i < m ? wl : wu;
    } else {
        for (int i = 0; i < 5; i++) sizes[i] = 1;
    }
}
// One direction of the sliding-window box sum with zero padding; `stride`
// walks along the line, `lines`/`lstride` across lines.
void box_pass(const uint8_t *src, uint8_t *dst, int len, int lines, size_t stride, size_t lstride, int r) {
    if (r == 0) {
        for (int l = 0; l < lines; l++)
            for (int i = 0; i < len; i++) std::memcpy(dst + l * lstride + i * stride, src + l * lstride + i * stride, 4);
        return;
    }
    float iarr = 1.0f / (float)(r + r + 1);
    for (int l = 0; l < lines; l++) {
        const uint8_t *s = src + l * lstride;
        uint8_t *d = dst + l * lstride;
        long val[4] = {0, 0, 0, 0};
        for (int j = 0; j < std::min(r, len); j++)
            for (int k = 0; k < 4; k++) val[k] += s[j * stride + k];
        for (int i = 0; i < len; i++) {
            int add = i + r, sub = i - r - 1;
            if (add < len) for (int k = 0; k < 4; k++) val[k] += s[add * stride + k];
            if (sub >= 0) for (int k = 0; k < 4; k++) val[k] -= s[sub * stride + k];
            for (int k = 0; k < 4; k++) d[i * stride + k] = sat_u8f(fround((float)val[k] * iarr));
        }
    }
}
void box_blur(double sx, double sy, Pixmap &src) {
    int bh[5], bv[5];
    create_box_gauss((float)sx, bh);
    create_box_gauss((float)sy, bv);
    std::vector<uint8_t> back = src.data;
    int w = (int)src.width, h = (int)src.height;
    for (int i = 0; i < 5; i++) {
        int rh = (bh[i] - 1) / 2, rv = (bv[i] - 1) / 2;
        box_pass(src.data.data(), back.data(), h, w, (size_t)w * 4, 4, rv);   // vertical: src -> back
        box_pass(back.data(), src.data.data(), w, h, 4, (size_t)w * 4, rh);   // horizontal: back -> src
    }
}

// ---- IIR blur (iir_blur.rs)
void gen_coefficients(double sigma, int steps, double *lambda, double *dnu) {
    *lambda = (sigma * sigma) / (2.0 * steps);
    *dnu = (1.0 + 2.0 * *lambda - std::sqrt(1.0 + 4.0 * *lambda)) / (2.0 * *lambda);
}
void gaussianiir2d(int width, int height, double sx, double sy, std::vector<double> &buf) {
    const int steps = 4;
    double lx = 1.0, dx = 1.0, ly = 1.0, dy = 1.0;
    if (sx > 0.0) {
        gen_coefficients(sx, steps, &lx, &dx);
        for (int y = 0; y < height; y++)
            for (int s = 0; s < steps; s++) {
                size_t idx = (size_t)width * y;
                for (int x = 1; x < width; x++) buf[idx + x] += dx * buf[idx + x - 1];
                for (int x = width - 1; x > 0; x--) buf[idx + x - 1] += dx * buf[idx + x];
            }
    }
    if (sy > 0.0) {
        gen_coefficients(sy, steps, &ly, &dy);
        for (int x = 0; x < width; x++)
            for (int s = 0; s < steps; s++) {
                size_t idx = x;
                for (size_t y = width; y < buf.size(); y += width) buf[idx + y] += dy * buf[idx + y - width];
                for (size_t y = buf.size() - width; y > 0; y -= width) buf[idx + y - width] += dy * buf[idx + y];
            }
    }
    double post = std::pow(std::sqrt(dx * dy) / std::sqrt(lx * ly), 2 * steps);
    for (auto &v : buf) v *= post;
}
void iir_blur(double sx, double sy, Pixmap &src) {
    size_t n = (size_t)src.width * src.height;
    std::vector<double> buf(n);
    for (int ch = 0; ch < 4; ch++) {
        for (size_t i = 0; i < n; i++) buf[i] = src.data[i * 4 + ch] / 255.0;
        gaussianiir2d((int)src.width, (int)src.height, sx, sy, buf);
        for (size_t i = 0; i < n; i++) src.data[i * 4 + ch] = sat_u8d(buf[i] * 255.0);
    }
}

bool approx_zero_ulps(float v) {
    // ApproxEqUlps against 0.0 with 4 ulps
    int32_t a, b = 0;
    std::memcpy(&a, &v, 4);
    if ((a < 0) != (b < 0)) return v == 0.0f;
    return std::abs(a - b) <= 4;
}

bool resolve_std_dev(float sdx, float sdy, const Transform &ts, double *ox, double *oy, bool *box) {
    float sx, sy;
    ts.get_scale(&sx, &sy);
    float x = sdx * sx, y = sdy * sy;
    if (approx_zero_ulps(x) && approx_zero_ulps(y)) return false;
    if (x < 0.05f) x = 0.0f;
    if (y < 0.05f) y = 0.0f;
    *box = x >= 2.0f || y >= 2.0f;
    *ox = x; *oy = y;
    return true;
}

// ---- colour matrix (color_matrix.rs)
inline uint8_t from_normalized(float c) { return sat_u8f(f32_bound(0.0f, c, 1.0f) * 255.0f); }
void color_matrix(const rgpu_primitive &p, Pixmap &pm) {
    auto &d = pm.data;
    int kind = p.i[0];
    if (kind == RGPU_CM_MATRIX) {
        const float *m = p.f;
        for (size_t i = 0; i < d.size(); i += 4) {
            float r = d[i] / 255.0f, g = d[i + 1] / 255.0f, b = d[i + 2] / 255.0f, a = d[i + 3] / 255.0f;
            float nr = r * m[0] + g * m[1] + b * m[2] + a * m[3] + m[4];
            float ng = r * m[5] + g * m[6] + b * m[7] + a * m[8] + m[9];
            float nb = r * m[10] + g * m[11] + b * m[12] + a * m[13] + m[14];
            float na = r * m[15] + g * m[16] + b * m[17] + a * m[18] + m[19];
            d[i] = from_normalized(nr); d[i + 1] = from_normalized(ng);
            d[i + 2] = from_normalized(nb); d[i + 3] = from_normalized(na);
        }
    } else if (kind == RGPU_CM_SATURATE || kind == RGPU_CM_HUE_ROTATE) {
        float m[9];
        if (kind == RGPU_CM_SATURATE) {
            float v = std::max(p.f[0], 0.0f);
            float mm[9] = {0.213f + 0.787f * v, 0.715f - 0.715f * v, 0.072f - 0.072f * v,
                           0.213f - 0.213f * v, 0.715f + 0.285f * v, 0.072f - 0.072f * v,
                           0.213f - 0.213f * v, 0.715f - 0.715f * v, 0.072f + 0.928f * v};
            std::memcpy(m, mm, sizeof(m));
        } else {
            float angle = p.f[0] * (float)(M_PI / 180.0);
            float a1 = std::cos(angle), a2 = std::sin(angle);
            float mm[9] = {0.213f + 0.787f * a1 - 0.213f * a2, 0.715f - 0.715f * a1 - 0.715f * a2,
                           0.072f - 0.072f * a1 + 0.928f * a2, 0.213f - 0.213f * a1 + 0.143f * a2,
                           0.715f + 0.285f * a1 + 0.140f * a2, 0.072f - 0.072f * a1 - 0.283f * a2,
                           0.213f - 0.213f * a1 - 0.787f * a2, 0.715f - 0.715f * a1 + 0.715f * a2,
                           0.072f + 0.928f * a1 + 0.072f * a2};
            std::memcpy(m, mm, sizeof(m));
        }
        for (size_t i = 0; i < d.size(); i += 4) {
            float r = d[i] / 255.0f, g = d[i + 1] / 255.0f, b = d[i + 2] / 255.0f;
            d[i] = from_normalized(r * m[0] + g * m[1] + b * m[2]);
            d[i + 1] = from_normalized(r * m[3] + g * m[4] + b * m[5]);
            d[i + 2] = from_normalized(r * m[6] + g * m[7] + b * m[8]);
        }
    } else {
        for (size_t i = 0; i < d.size(); i += 4) {
            float r = d[i] / 255.0f, g = d[i + 1] / 255.0f, b = d[i + 2] / 255.0f;
            float na = r * 0.2125f + g * 0.7154f + b * 0.0721f;
            d[i] = d[i + 1] = d[i + 2] = 0;
            d[i + 3] = from_normalized(na);
        }
    }
}

// ---- morphology (morphology.rs)
void morphology(bool dilate, float rx, float ry, Pixmap &src) {
    uint32_t columns = std::min((uint32_t)std::ceil(rx) * 2, src.width);
    uint32_t rows = std::min((uint32_t)std::ceil(ry) * 2, src.height);
    uint32_t tx0 = (uint32_t)std::floor(columns / 2.0f), ty0 = (uint32_t)std::floor(rows / 2.0f);
    int32_t wmax = (int32_t)src.width - 1, hmax = (int32_t)src.height - 1;
    std::vector<uint8_t> buf(src.data.size(), 0);
    for (uint32_t y = 0; y < src.height; y++)
        for (uint32_t x = 0; x < src.width; x++) {
            uint8_t np[4];
            for (int k = 0; k < 4; k++) np[k] = dilate ? 0 : 255;
            for (uint32_t oy = 0; oy < rows; oy++)
                for (uint32_t ox = 0; ox < columns; ox++) {
                    int32_t tx = (int32_t)x - (int32_t)tx0 + (int32_t)ox, ty = (int32_t)y - (int32_t)ty0 + (int32_t)oy;
                    if (tx < 0 || tx > wmax || ty < 0 || ty > hmax) continue;
                    const uint8_t *p = src.px((uint32_t)tx, (uint32_t)ty);
                    for (int k = 0; k < 4; k++) np[k] = dilate ? std::max(np[k], p[k]) : std::min(np[k], p[k]);
                }
            std::memcpy(&buf[((size_t)y * src.width + x) * 4], np, 4);
        }
    src.data = buf;
}

// ---- arithmetic composite (composite.rs)
void arithmetic(float k1, float k2, float k3, float k4, const Pixmap &s1, const Pixmap &s2, Pixmap &dst) {
    auto calc = [&](uint8_t i1, uint8_t i2, float mx) {
        float a = i1 / 255.0f, b = i2 / 255.0f;
        float r = k1 * a * b + k2 * a + k3 * b + k4;
        return f32_bound(0.0f, r, mx);
    };
    size_t n = (size_t)dst.width * dst.height;
    for (size_t i = 0; i < n; i++) {
        const uint8_t *c1 = &s1.data[i * 4], *c2 = &s2.data[i * 4];
        float a = calc(c1[3], c2[3], 1.0f);
        if (approx_zero_ulps(a)) continue;
        uint8_t *d = &dst.data[i * 4];
        d[0] = sat_u8f(calc(c1[0], c2[0], a) * 255.0f);
        d[1] = sat_u8f(calc(c1[1], c2[1], a) * 255.0f);
        d[2] = sat_u8f(calc(c1[2], c2[2], a) * 255.0f);
        d[3] = sat_u8f(a * 255.0f);
    }
}

// ---- convolve matrix (convolve_matrix.rs)
void convolve(const rgpu_primitive &p, Pixmap &src) {
    int cols = p.i[0], rows = p.i[1], tx0 = p.i[2], ty0 = p.i[3], edge = p.i[4];
    bool preserve = p.i[5] != 0;
    float divisor = p.f[0], bias = p.f[1];
    const float *k = p.f + 2;
    int32_t wmax = (int32_t)src.width - 1, hmax = (int32_t)src.height - 1;
    std::vector<uint8_t> buf(src.data.size(), 0);
    for (uint32_t y = 0; y < src.height; y++)
        for (uint32_t x = 0; x < src.width; x++) {
            float nr = 0, ng = 0, nb = 0, na = 0;
            for (int oy = 0; oy < rows; oy++)
                for (int ox = 0; ox < cols; ox++) {
                    int32_t tx = (int32_t)x - tx0 + ox, ty = (int32_t)y - ty0 + oy;
                    if (edge == RGPU_EDGE_NONE) {
                        if (tx < 0 || tx > wmax || ty < 0 || ty > hmax) continue;
                    } else if (edge == RGPU_EDGE_DUPLICATE) {
                        tx = std::max(0, std::min(wmax, tx));
                        ty = std::max(0, std::min(hmax, ty));
                    } else {
                        while (tx < 0) tx += (int32_t)src.width;
                        tx %= (int32_t)src.width;
                        while (ty < 0) ty += (int32_t)src.height;
                        ty %= (int32_t)src.height;
                    }
                    float kv = k[(rows - oy - 1) * cols + (cols - ox - 1)];
                    const uint8_t *pp = src.px((uint32_t)tx, (uint32_t)ty);
                    nr += (float)pp[0] / 255.0f * kv;
                    ng += (float)pp[1] / 255.0f * kv;
                    nb += (float)pp[2] / 255.0f * kv;
                    if (!preserve) na += (float)pp[3] / 255.0f * kv;
                }
            const uint8_t *in_p = src.px(x, y);
            if (preserve) na = in_p[3] / 255.0f;
            else na = na / divisor + bias;
            float bna = f32_bound(0.0f, na, 1.0f);
            auto calc = [&](float v) {
                float q = v / divisor + bias * na;
                q = preserve ? f32_bound(0.0f, q, 1.0f) * bna : f32_bound(0.0f, q, bna);
                return sat_u8f(q * 255.0f + 0.5f);
            };
            uint8_t *o = &buf[((size_t)y * src.width + x) * 4];
            o[0] = calc(nr); o[1] = calc(ng); o[2] = calc(nb);
            o[3] = sat_u8f(bna * 255.0f + 0.5f);
        }
    src.data = buf;
}

// ---- diffuse / specular lighting (lighting.rs; light source mapping mod.rs:1062-1098)
struct V3 { float x, y, z; };
inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float len3(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 normalized_or_self(V3 v) {
    float l = len3(v);
    if (approx_zero_ulps(l)) return v;
    return V3{v.x / l, v.y / l, v.z / l};
}
bool approx_eq_ulps_f(float a, float b) {
    int32_t ia, ib;
    std::memcpy(&ia, &a, 4);
    std::memcpy(&ib, &b, 4);
    if ((ia < 0) != (ib < 0)) return a == b;
    return std::abs(ia - ib) <= 4;
}
inline float deg_to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

// Sobel-style surface normal of the alpha channel at (x, y) with the border
// variants of lighting.rs:296-476: (factor x, factor y, nx, ny).
void surface_normal(const Pixmap &img, uint32_t x, uint32_t y, float *fx, float *fy, int *nx, int *ny) {
    const uint32_t w = img.width, h = img.height;
    auto a = [&](uint32_t xx, uint32_t yy) -> int { return img.px(xx, yy)[3]; };
    const bool l = x == 0, r = x == w - 1, t = y == 0, b = y == h - 1;
    if (t && l) {
        int c = a(0, 0), rt = a(1, 0), bt = a(0, 1), br = a(1, 1);
        *fx = *fy = 2.0f / 3.0f;
        *nx = -2 * c + 2 * rt - bt + br; *ny = -2 * c - rt + 2 * bt + br;
    } else if (t && r) {
        int lf = a(w - 2, 0), c = a(w - 1, 0), bl = a(w - 2, 1), bt = a(w - 1, 1);
        *fx = *fy = 2.0f / 3.0f;
        *nx = -2 * lf + 2 * c - bl + bt; *ny = -lf - 2 * c + bl + 2 * bt;
    } else if (b && l) {
        int tp = a(0, h - 2), tr = a(1, h - 2), c = a(0, h - 1), rt = a(1, h - 1);
        *fx = *fy = 2.0f / 3.0f;
        *nx = -tp + tr - 2 * c + 2 * rt; *ny = -2 * tp - tr + 2 * c + rt;
    } else if (b && r) {
        int tl = a(w - 2, h - 2), tp = a(w - 1, h - 2), lf = a(w - 2, h - 1), c = a(w - 1, h - 1);
        *fx = *fy = 2.0f / 3.0f;
        *nx = -tl + tp - 2 * lf + 2 * c; *ny = -tl - 2 * tp + lf + 2 * c;
    } else if (t) {
        int lf = a(x - 1, 0), c = a(x, 0), rt = a(x + 1, 0), bl = a(x - 1, 1), bt = a(x, 1), br = a(x + 1, 1);
        *fx = 1.0f / 3.0f; *fy = 1.0f / 2.0f;
        *nx = -2 * lf + 2 * rt - bl + br; *ny = -lf - 2 * c - rt + bl + 2 * bt + br;
    } else if (b) {
        int tl = a(x - 1, h - 2), tp = a(x, h - 2), tr = a(x + 1, h - 2), lf = a(x - 1, h - 1), c = a(x, h - 1),
            rt = a(x + 1, h - 1);
        *fx = 1.0f / 3.0f; *fy = 1.0f / 2.0f;
        *nx = -tl + tr - 2 * lf + 2 * rt; *ny = -tl - 2 * tp - tr + lf + 2 * c + rt;
    } else if (l) {
        int tp = a(0, y - 1), tr = a(1, y - 1), c = a(0, y), rt = a(1, y), bt = a(0, y + 1), br = a(1, y + 1);
        *fx = 1.0f / 2.0f; *fy = 1.0f / 3.0f;
        *nx = -tp + tr - 2 * c + 2 * rt - bt + br; *ny = -2 * tp - tr + 2 * bt + br;
    } else if (r) {
        int tl = a(w - 2, y - 1), tp = a(w - 1, y - 1), lf = a(w - 2, y), c = a(w - 1, y), bl = a(w - 2, y + 1),
            bt = a(w - 1, y + 1);
        *fx = 1.0f / 2.0f; *fy = 1.0f / 3.0f;
        *nx = -tl + tp - 2 * lf + 2 * c - bl + bt; *ny = -tl - 2 * tp + bl + 2 * bt;
    } else {
        int tl = a(x - 1, y - 1), tp = a(x, y - 1), tr = a(x + 1, y - 1), lf = a(x - 1, y), rt = a(x + 1, y),
            bl = a(x - 1, y + 1), bt = a(x, y + 1), br = a(x + 1, y + 1);
        *fx = *fy = 1.0f / 4.0f;
        *nx = -tl + tr - 2 * lf + 2 * rt - bl + br; *ny = -tl - 2 * tp - tr + bl + 2 * bt + br;
    }
}

void lighting(bool specular, const rgpu_primitive &p, const Transform &ts, const IntRect &region, const Pixmap &src,
              Pixmap &dst) {
    const uint32_t w = src.width, h = src.height;
    if (w < 3 || h < 3) return;
    const float ss = p.f[0], kc = p.f[1], sexp = p.f[2];
    const int kind = p.i[0];
    const uint8_t lc[3] = {(uint8_t)p.i[1], (uint8_t)p.i[2], (uint8_t)p.i[3]};
    // the light source in the region's pixel space (transform_light_source)
    float lx = p.f[4], ly = p.f[5], lz = p.f[6], ax = p.f[7], ay = p.f[8], az = p.f[9];
    if (kind != RGPU_LIGHT_DISTANT) {
        const float sz = std::sqrt(ts.sx * ts.sx + ts.sy * ts.sy) / 1.41421356237309504880f;
        Point q{lx, ly};
        ts.map_points(&q, 1);
        lx = q.x - (float)region.x; ly = q.y - (float)region.y; lz = lz * sz;
        if (kind == RGPU_LIGHT_SPOT) {
            Point q2{ax, ay};
            ts.map_points(&q2, 1);
            ax = q2.x - (float)region.x; ay = q2.y - (float)region.y; az = az * sz;
        }
    }
    V3 lv{1.0f, 1.0f, 1.0f};
    if (kind == RGPU_LIGHT_DISTANT) {
        const float azi = deg_to_rad(p.f[4]), ele = deg_to_rad(p.f[5]);
        lv = V3{std::cos(azi) * std::cos(ele), std::sin(azi) * std::cos(ele), std::sin(ele)};
    }
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            if (kind != RGPU_LIGHT_DISTANT) {
                const float nz = (float)src.px(x, y)[3] / 255.0f * ss;
                lv = normalized_or_self(V3{lx - (float)x, ly - (float)y, lz - nz});
            }
            // light colour (light_color)
            uint8_t col[3] = {lc[0], lc[1], lc[2]};
            if (kind == RGPU_LIGHT_SPOT) {
                V3 d = normalized_or_self(V3{ax - lx, ay - ly, az - lz});
                const float mls = -dot3(lv, d);
                bool black = mls <= 0.0f;
                if (!black && !std::isnan(p.f[11]) && mls < std::cos(deg_to_rad(p.f[11]))) black = true;
                if (black) col[0] = col[1] = col[2] = 0;
                else {
                    const float fac = std::pow(mls, p.f[10]);
                    for (int k = 0; k < 3; k++) col[k] = (uint8_t)(f32_bound(0.0f, (float)lc[k] * fac, 255.0f) + 0.5f);
                }
            }
            float fx, fy;
            int inx, iny;
            surface_normal(src, x, y, &fx, &fy, &inx, &iny);
            const float nxv = (float)(int16_t)(-inx), nyv = (float)(int16_t)(-iny);
            const bool flat = approx_zero_ulps(nxv) && approx_zero_ulps(nyv);
            float factor;
            if (!specular) {
                float k;
                if (flat) k = lv.z;
                else {
                    const float sc = ss / 255.0f;
                    V3 n{nxv * sc * fx, nyv * sc * fy, 1.0f};
                    k = dot3(n, lv) / len3(n);
                }
                factor = kc * k;
            } else {
                V3 hv{lv.x + 0.0f, lv.y + 0.0f, lv.z + 1.0f};
                const float hl = len3(hv);
                if (approx_zero_ulps(hl)) factor = 0.0f;
                else {
                    float ndh;
                    if (flat) ndh = hv.z / hl;
                    else {
                        const float sc = ss / 255.0f;
                        V3 n{nxv * sc * fx, nyv * sc * fy, 1.0f};
                        ndh = dot3(n, hv) / len3(n) / hl;
                    }
                    const float k = approx_eq_ulps_f(sexp, 1.0f) ? ndh : std::pow(ndh, sexp);
                    factor = kc * k;
                }
            }
            uint8_t o[3];
            for (int k = 0; k < 3; k++) o[k] = (uint8_t)(f32_bound(0.0f, (float)col[k] * factor, 255.0f) + 0.5f);
            uint8_t *d = &dst.data[((size_t)y * w + x) * 4];
            d[0] = o[0]; d[1] = o[1]; d[2] = o[2];
            d[3] = specular ? std::max(std::max(o[0], o[1]), o[2]) : 255;
        }
}

bool int_rect_eq(const IntRect &a, const IntRect &b) { return a.x == b.x && a.y == b.y && a.w == b.w && a.h == b.h; }

struct Result { Image image; };

}  // namespace

// mod.rs:335-521 apply/apply_inner + mod.rs:1100-1114 apply_to_canvas
// ---- turbulence (turbulence.rs:33-304): the Perlin noise of the SVG 1.1
// specification, f64 throughout, lattice and gradients from a Park-Miller
// generator seeded by `seed`.
namespace turb {
const int32_t kRandM = 2147483647, kRandA = 16807, kRandQ = 127773, kRandR = 2836;
const int kB = 0x100, kBLen = 0x100 + 0x100 + 2, kBM = 0xff, kPerlinN = 0x1000;
struct Tables { int32_t sel[kBLen]; double grad[4][kBLen][2]; };
int32_t random(int32_t seed) {
    int32_t r = kRandA * (seed % kRandQ) - kRandR * (seed / kRandQ);
    if (r <= 0) r += kRandM;
    return r;
}
void init(int32_t seed, Tables &t) {
    if (seed <= 0) seed = (int32_t)(0u - (uint32_t)seed) % (kRandM - 1) + 1;  // -seed wraps, as in Rust
    if (seed > kRandM - 1) seed = kRandM - 1;
    for (int k = 0; k < 4; k++) {
        for (int i = 0; i < kB; i++) {
            t.sel[i] = i;
            for (int j = 0; j < 2; j++) {
                seed = random(seed);
                t.grad[k][i][j] = (double)((seed % (kB + kB)) - kB) / (double)kB;
            }
            const double s = std::sqrt(t.grad[k][i][0] * t.grad[k][i][0] + t.grad[k][i][1] * t.grad[k][i][1]);
            t.grad[k][i][0] /= s;
            t.grad[k][i][1] /= s;
        }
    }
    for (int i = kB - 1; i >= 1; i--) {
        const int32_t k = t.sel[i];
        seed = random(seed);
        const int32_t j = seed % kB;
        t.sel[i] = t.sel[j];
        t.sel[j] = k;
    }
    for (int i = 0; i < kB + 2; i++) {
        t.sel[kB + i] = t.sel[i];
        for (int g = 0; g < 4; g++)
            for (int j = 0; j < 2; j++) t.grad[g][kB + i][j] = t.grad[g][i][j];
    }
}
// Rust's saturating float -> integer casts
int32_t to_i32(double v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483647.0) return INT32_MAX;
    if (v <= -2147483648.0) return INT32_MIN;
    return (int32_t)v;
}
int64_t to_i64(double v) {
    if (std::isnan(v)) return 0;
    if (v >= 9223372036854775807.0) return INT64_MAX;
    if (v <= -9223372036854775808.0) return INT64_MIN;
    return (int64_t)v;
}
struct Stitch { int32_t width, height, wrap_x, wrap_y; };
inline double s_curve(double t) { return t * t * (3.0 - 2.0 * t); }
inline double lerp(double t, double a, double b) { return a + t * (b - a); }
double noise2(int ch, double x, double y, const Tables &t, const Stitch *st) {
    double tt = x + (double)kPerlinN;
    int32_t bx0 = to_i32(tt), bx1 = (int32_t)((uint32_t)bx0 + 1u);
    const double rx0 = tt - (double)to_i64(tt), rx1 = rx0 - 1.0;
    tt = y + (double)kPerlinN;
    int32_t by0 = to_i32(tt), by1 = (int32_t)((uint32_t)by0 + 1u);
    const double ry0 = tt - (double)to_i64(tt), ry1 = ry0 - 1.0;
    if (st) {
        if (bx0 >= st->wrap_x) bx0 = (int32_t)((uint32_t)bx0 - (uint32_t)st->width);
        if (bx1 >= st->wrap_x) bx1 = (int32_t)((uint32_t)bx1 - (uint32_t)st->width);
        if (by0 >= st->wrap_y) by0 = (int32_t)((uint32_t)by0 - (uint32_t)st->height);
        if (by1 >= st->wrap_y) by1 = (int32_t)((uint32_t)by1 - (uint32_t)st->height);
    }
    bx0 &= kBM; bx1 &= kBM; by0 &= kBM; by1 &= kBM;
    const int32_t i = t.sel[bx0], j = t.sel[bx1];
    const int32_t b00 = t.sel[i + by0], b10 = t.sel[j + by0], b01 = t.sel[i + by1], b11 = t.sel[j + by1];
    const double sx = s_curve(rx0), sy = s_curve(ry0);
    const double *q = t.grad[ch][b00];
    double u = rx0 * q[0] + ry0 * q[1];
    q = t.grad[ch][b10];
    double v = rx1 * q[0] + ry0 * q[1];
    const double a = lerp(sx, u, v);
    q = t.grad[ch][b01];
    u = rx0 * q[0] + ry1 * q[1];
    q = t.grad[ch][b11];
    v = rx1 * q[0] + ry1 * q[1];
    const double b = lerp(sx, u, v);
    return lerp(sy, a, b);
}
bool approx_zero_ulps_d(double v) {  // f64 approx_zero_ulps(4)
    int64_t a;
    std::memcpy(&a, &v, 8);
    if (a < 0) return v == 0.0;
    return a <= 4;
}
double turbulence(int ch, double x, double y, double tile_x, double tile_y, double tile_w, double tile_h,
                  double bfx, double bfy, uint32_t octaves, bool fractal, bool stitching, const Tables &t) {
    Stitch st{0, 0, 0, 0};
    if (stitching) {
        if (!approx_zero_ulps_d(bfx)) {
            const double lo = std::floor(tile_w * bfx) / tile_w, hi = std::ceil(tile_w * bfx) / tile_w;
            bfx = (bfx / lo < hi / bfx) ? lo : hi;
        }
        if (!approx_zero_ulps_d(bfy)) {
            const double lo = std::floor(tile_h * bfy) / tile_h, hi = std::ceil(tile_h * bfy) / tile_h;
            bfy = (bfy / lo < hi / bfy) ? lo : hi;
        }
        st.width = to_i32(tile_w * bfx + 0.5);
        st.height = to_i32(tile_h * bfy + 0.5);
        st.wrap_x = to_i32(tile_x * bfx + (double)kPerlinN + (double)st.width);
        st.wrap_y = to_i32(tile_y * bfy + (double)kPerlinN + (double)st.height);
    }
    double sum = 0.0, ratio = 1.0;
    x *= bfx;
    y *= bfy;
    for (uint32_t o = 0; o < octaves; o++) {
        const double n = noise2(ch, x, y, t, stitching ? &st : nullptr);
        sum += (fractal ? n : std::fabs(n)) / ratio;
        x *= 2.0;
        y *= 2.0;
        ratio *= 2.0;
        if (stitching) {  // wrapping i32 arithmetic, as Rust's release build
            st.width = (int32_t)((uint32_t)st.width * 2u);
            st.wrap_x = (int32_t)((uint32_t)st.wrap_x * 2u - (uint32_t)kPerlinN);
            st.height = (int32_t)((uint32_t)st.height * 2u);
            st.wrap_y = (int32_t)((uint32_t)st.wrap_y * 2u - (uint32_t)kPerlinN);
        }
    }
    return sum;
}
}  // namespace turb

// apply_turbulence (mod.rs:988-1018): a region-sized image, unpremultiplied
// noise then multiply_alpha.
void turbulence(const rgpu_primitive &p, const Transform &ts, const IntRect &region, Pixmap &pm) {
    float fsx, fsy;
    ts.get_scale(&fsx, &fsy);
    if (approx_zero_ulps(fsx) || approx_zero_ulps(fsy)) return;
    turb::Tables t;
    turb::init(p.i[1], t);
    const double ox = (double)region.x - (double)ts.tx, oy = (double)region.y - (double)ts.ty;
    const double sx = fsx, sy = fsy, bfx = p.f[0], bfy = p.f[1];
    const bool fractal = p.i[3] != 0, stitch = p.i[2] != 0;
    const uint32_t oct = (uint32_t)p.i[0];
    for (uint32_t y = 0; y < pm.height; y++)
        for (uint32_t x = 0; x < pm.width; x++)
            for (int ch = 0; ch < 4; ch++) {
                const double tx = ((double)x + ox) / sx, ty = ((double)y + oy) / sy;
                double n = turb::turbulence(ch, tx, ty, (double)x, (double)y, (double)pm.width, (double)pm.height,
                                            bfx, bfy, oct, fractal, stitch, t);
                n = fractal ? (n * 255.0 + 255.0) / 2.0 : n * 255.0;
                pm.data[((size_t)y * pm.width + x) * 4 + ch] = sat_u8f(f32_bound(0.0f, (float)n, 255.0f) + 0.5f);
            }
    multiply_alpha(pm.data);
}

// ---- tile (mod.rs:835-859): the input's region, cut from its image (the
// part inside the image), repeats from the region's origin over a
// region-sized image.  The pattern's transform is an integer translation, so
// its sampling is nearest and the repeat is an integer modulus.
bool tile(const Image &in, const IntRect &region, Pixmap &out) {
    const IntRect sub{in.region.x - region.x, in.region.y - region.y, in.region.w, in.region.h};
    const int32_t l = std::max(sub.x, 0), t = std::max(sub.y, 0);
    const int32_t r = std::min(sub.right(), (int32_t)in.image->width), b = std::min(sub.bottom(), (int32_t)in.image->height);
    if (r <= l || b <= t) return false;
    const int32_t tw = r - l, th = b - t;
    for (uint32_t y = 0; y < out.height; y++)
        for (uint32_t x = 0; x < out.width; x++) {
            int32_t u = ((int32_t)x - sub.x) % tw, v = ((int32_t)y - sub.y) % th;
            if (u < 0) u += tw;
            if (v < 0) v += th;
            std::memcpy(&out.data[((size_t)y * out.width + x) * 4],
                        &in.image->data[((size_t)(t + v) * in.image->width + (size_t)(l + u)) * 4], 4);
        }
    return true;
}

// ---- displacement map (displacement_map.rs:15-62, mod.rs:958-986); the map
// is read as stored (premultiplied), as the driver passes it.
void displacement_map(const rgpu_primitive &p, float sx, float sy, const Pixmap &src, const Pixmap &map,
                      Pixmap &dst) {
    const int32_t w = (int32_t)src.width, h = (int32_t)src.height;
    const float scale = p.f[0];
    for (uint32_t y = 0; y < map.height; y++)
        for (uint32_t x = 0; x < map.width; x++) {
            const uint8_t *m = &map.data[((size_t)y * map.width + x) * 4];
            const float dx = m[p.i[0] & 3] / 255.0f - 0.5f, dy = m[p.i[1] & 3] / 255.0f - 0.5f;
            const float fx = (float)x + dx * sx * scale, fy = (float)y + dy * sy * scale;
            const int32_t ox = sat_i32(std::round(fx)), oy = sat_i32(std::round(fy));
            if ((int32_t)x < w && (int32_t)y < h && ox >= 0 && ox < w && oy >= 0 && oy < h &&
                x < dst.width && y < dst.height)
                std::memcpy(&dst.data[((size_t)y * dst.width + x) * 4], &src.data[((size_t)oy * w + ox) * 4], 4);
        }
}

// ---- component transfer (component_transfer.rs:10-78), on demultiplied pixels
bool transfer_is_dummy(const rgpu_primitive &p, int ch) {
    switch (p.i[ch]) {
    case RGPU_TF_TABLE:
    case RGPU_TF_DISCRETE: return p.i[4 + ch] <= 0;
    case RGPU_TF_LINEAR:
    case RGPU_TF_GAMMA: return false;
    default: return true;
    }
}
uint8_t transfer(const rgpu_primitive &p, int ch, uint8_t c8) {
    const float *v = p.f + 16 * ch;
    float c = c8 / 255.0f;
    switch (p.i[ch]) {
    case RGPU_TF_TABLE: {
        const int n = p.i[4 + ch] - 1;
        float fk = std::floor(c * (float)n);
        int k = fk >= (float)n ? n : (int)fk;
        if (k == n) {
            c = v[k];
        } else {
            const float vk = v[k], vk1 = v[k + 1];
            const float kf = (float)k, nf = (float)n;
            c = vk + (c - kf / nf) * nf * (vk1 - vk);
        }
        break;
    }
    case RGPU_TF_DISCRETE: {
        const int n = p.i[4 + ch];
        float fk = std::floor(c * (float)n);
        int k = fk >= (float)(n - 1) ? n - 1 : (int)fk;
        c = v[k];
        break;
    }
    case RGPU_TF_LINEAR: c = v[0] * c + v[1]; break;
    case RGPU_TF_GAMMA: c = v[0] * std::pow(c, v[1]) + v[2]; break;
    default: break;
    }
    return sat_u8f(f32_bound(0.0f, c, 1.0f) * 255.0f);
}
// mod.rs:891-903: colour space, demultiply, transfer R, B, G, A, multiply
void component_transfer(const rgpu_primitive &p, Pixmap &pm) {
    demultiply_alpha(pm.data);
    static const int order[4] = {0, 2, 1, 3};
    for (int oi = 0; oi < 4; oi++) {
        const int ch = order[oi];
        if (transfer_is_dummy(p, ch)) continue;
        for (size_t i = 0; i < pm.data.size(); i += 4) pm.data[i + ch] = transfer(p, ch, pm.data[i + ch]);
    }
    multiply_alpha(pm.data);
}

// ---- drop shadow (mod.rs:581-649)
// The flood step: Color::from_rgba8(r, g, b, opacity.to_u8()), apply_opacity(alpha / 255),
// premultiply, to_color_u8.
void drop_shadow_flood(const rgpu_primitive &p, Pixmap &sh) {
    const ColorF col = color_from_rgba8((uint8_t)p.i[0], (uint8_t)p.i[1], (uint8_t)p.i[2], to_u8_norm(p.f[4]));
    auto clamp01 = [](float v) { return std::min(std::max(v, 0.0f), 1.0f); };
    for (size_t i = 0; i < sh.data.size(); i += 4) {
        ColorF c = col;
        c.a = clamp01(c.a * clamp01(sh.data[i + 3] / 255.0f));
        if (c.a != 1.0f) { c.r = clamp01(c.r * c.a); c.g = clamp01(c.g * c.a); c.b = clamp01(c.b * c.a); }
        sh.data[i + 0] = sat_u8f(c.r * 255.0f + 0.5f);
        sh.data[i + 1] = sat_u8f(c.g * 255.0f + 0.5f);
        sh.data[i + 2] = sat_u8f(c.b * 255.0f + 0.5f);
        sh.data[i + 3] = sat_u8f(c.a * 255.0f + 0.5f);
    }
}

bool filter_apply(const rgpu_tree_view &t, const rgpu_filter &f, const Transform &ts, Pixmap &source) {
    auto fail = [&]() { pixmap_fill(source, ColorF{0, 0, 0, 0}); return false; };
    bool ok;
    Rect fr = rect_transform(Rect{f.x, f.y, f.x + f.w, f.y + f.h}, ts, &ok);
    if (!ok) return fail();
    IntRect region;
    if (!rect_to_int_rect(fr, &region)) return fail();
    {
        IntRect src_rect{0, 0, (int32_t)source.width, (int32_t)source.height};
        int32_t l = std::max(region.x, 0), tt = std::max(region.y, 0);
        int32_t r = std::min(region.right(), src_rect.right()), b = std::min(region.bottom(), src_rect.bottom());
        if (r <= l || b <= tt) return fail();
        region = IntRect{l, tt, r - l, b - tt};
    }
    std::vector<Image> results;
    auto get_input = [&](int32_t in) -> Image {
        if (in >= 0 && (size_t)in < results.size()) return results[in];
        auto p = std::make_shared<Pixmap>(source);
        if (in == RGPU_IN_SOURCE_ALPHA)
            for (size_t i = 0; i < p->data.size(); i += 4) p->data[i] = p->data[i + 1] = p->data[i + 2] = 0;
        return Image{p, region, false};
    };
    for (uint32_t pi = 0; pi < f.prim_count; pi++) {
        const rgpu_primitive &p = t.prims[f.prim_offset + pi];
        Rect pr = rect_transform(Rect{p.x, p.y, p.x + p.w, p.y + p.h}, ts, &ok);
        if (!ok) return fail();
        IntRect subregion;
        if (!rect_to_int_rect(pr, &subregion)) return fail();
        // mod.rs:384-391: feOffset inherits its subregion from a referenced input
        if (p.kind == RGPU_FE_OFFSET && p.in1 >= 0 && (size_t)p.in1 < results.size()) subregion = results[p.in1].region;
        bool lin = p.linear_rgb != 0;
        Image res;
        switch (p.kind) {
        case RGPU_FE_BLUR: {
            Image in = get_input(p.in1);
            double sx, sy;
            bool box;
            if (!resolve_std_dev(p.f[0], p.f[1], ts, &sx, &sy, &box)) { res = in; break; }
            Image c = into_cs(in, lin);
            auto pm = std::make_shared<Pixmap>(*c.image);
            if (box) box_blur(sx, sy, *pm); else iir_blur(sx, sy, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_COLOR_MATRIX: {
            Image c = into_cs(get_input(p.in1), lin);
            auto pm = std::make_shared<Pixmap>(*c.image);
            demultiply_alpha(pm->data);
            color_matrix(p, *pm);
            multiply_alpha(pm->data);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_MORPHOLOGY: {
            Image c = into_cs(get_input(p.in1), lin);
            auto pm = std::make_shared<Pixmap>(*c.image);
            float sx, sy;
            ts.get_scale(&sx, &sy);
            float rx = p.f[0] * sx, ry = p.f[1] * sy;
            if (!(rx > 0.0f && ry > 0.0f)) pixmap_fill(*pm, ColorF{0, 0, 0, 0});
            else morphology(p.i[0] == 1, rx, ry, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_COMPOSITE: {
            Image i1 = into_cs(get_input(p.in1), lin), i2 = into_cs(get_input(p.in2), lin);
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            if (p.i[0] == RGPU_OP_ARITHMETIC) {
                arithmetic(p.f[0], p.f[1], p.f[2], p.f[3], *i1.image, *i2.image, *pm);
            } else {
                draw_pixmap(*pm, 0, 0, *i2.image, 1.0f, RGPU_BLEND_SOURCE_OVER);
                uint32_t bm = RGPU_BLEND_SOURCE_OVER;
                switch (p.i[0]) {
                case RGPU_OP_IN: bm = RGPU_BLEND_SOURCE_IN; break;
                case RGPU_OP_OUT: bm = RGPU_BLEND_SOURCE_OUT; break;
                case RGPU_OP_ATOP: bm = RGPU_BLEND_SOURCE_ATOP; break;
                case RGPU_OP_XOR: bm = RGPU_BLEND_XOR; break;
                default: break;
                }
                draw_pixmap(*pm, 0, 0, *i1.image, 1.0f, bm);
            }
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_CONVOLVE: {
            Image c = into_cs(get_input(p.in1), lin);
            auto pm = std::make_shared<Pixmap>(*c.image);
            if (p.i[5]) demultiply_alpha(pm->data);
            convolve(p, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_DIFFUSE:
        case RGPU_FE_SPECULAR: {
            Image in = get_input(p.in1);
            // lighting.rs indexes the region-sized result with the input's size
            // (debug-asserted equal): with a layer-sized input under a smaller
            // region the reference indexes out of range, so the filter fails
            if ((int32_t)in.image->width != region.w || (int32_t)in.image->height != region.h) return fail();
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            lighting(p.kind == RGPU_FE_SPECULAR, p, ts, region, *in.image, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_IMAGE: {
            // apply_image (mod.rs:861-889): the element at the layer's scale, moved
            // to the subregion, in a region-sized sRGB image
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            float sx, sy;
            ts.get_scale(&sx, &sy);
            if (p.i[0] >= 0 && (uint32_t)p.i[0] < t.group_count)
                render_group_children(t, (uint32_t)p.i[0],
                                      Transform::from_row(sx, 0, 0, sy, (float)subregion.x, (float)subregion.y), *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, false};
            break;
        }
        case RGPU_FE_TILE: {
            Image in = get_input(p.in1);
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            if (!tile(in, region, *pm)) return fail();
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, false};
            break;
        }
        case RGPU_FE_DISPLACEMENT_MAP: {
            Image i1 = into_cs(get_input(p.in1), lin), i2 = into_cs(get_input(p.in2), lin);
            // displacement_map.rs walks the map with the source's width and
            // writes the region-sized result at the same index (sizes
            // debug-asserted equal): any mismatch fails the filter
            if ((int32_t)i1.image->width != region.w || (int32_t)i1.image->height != region.h ||
                (int32_t)i2.image->width != region.w || (int32_t)i2.image->height != region.h)
                return fail();
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            float sx, sy;
            ts.get_scale(&sx, &sy);
            displacement_map(p, p.f[0] * sx, p.f[0] * sy, *i1.image, *i2.image, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_TURBULENCE: {
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            turbulence(p, ts, region, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_COMPONENT_TRANSFER: {
            Image c = into_cs(get_input(p.in1), lin);
            auto pm = std::make_shared<Pixmap>(*c.image);
            component_transfer(p, *pm);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_DROP_SHADOW: {
            Image c = into_cs(get_input(p.in1), lin);
            float sx, sy;
            ts.get_scale(&sx, &sy);
            const float dx = p.f[2] * sx, dy = p.f[3] * sy;
            Pixmap sh(*c.image);
            double bx, by;
            bool box;
            if (resolve_std_dev(p.f[0], p.f[1], ts, &bx, &by, &box)) {
                if (box) box_blur(bx, by, sh); else iir_blur(bx, by, sh);
            }
            drop_shadow_flood(p, sh);
            if (lin) into_linear(sh); else into_srgb(sh);
            auto pm = std::make_shared<Pixmap>(c.image->width, c.image->height);
            draw_pixmap(*pm, sat_i32(dx), sat_i32(dy), sh, 1.0f, RGPU_BLEND_SOURCE_OVER);
            draw_pixmap(*pm, 0, 0, *c.image, 1.0f, RGPU_BLEND_SOURCE_OVER);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_FLOOD: {
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            pixmap_fill(*pm, color_from_rgba8((uint8_t)p.i[0], (uint8_t)p.i[1], (uint8_t)p.i[2], to_u8_norm(p.f[0])));
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, false};
            break;
        }
        case RGPU_FE_OFFSET: {
            Image in = get_input(p.in1);
            float sx, sy;
            ts.get_scale(&sx, &sy);
            float dx = p.f[0] * sx, dy = p.f[1] * sy;
            if (approx_zero_ulps(dx) && approx_zero_ulps(dy)) { res = in; break; }
            auto pm = std::make_shared<Pixmap>(in.image->width, in.image->height);
            draw_pixmap(*pm, sat_i32(dx), sat_i32(dy), *in.image, 1.0f, RGPU_BLEND_SOURCE_OVER);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, in.linear};
            break;
        }
        case RGPU_FE_MERGE: {
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            for (int32_t k = 0; k < p.i[1]; k++) {
                Image c = into_cs(get_input(t.merge_inputs[p.i[0] + k]), lin);
                draw_pixmap(*pm, 0, 0, *c.image, 1.0f, RGPU_BLEND_SOURCE_OVER);
            }
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        case RGPU_FE_BLEND: {
            Image i1 = into_cs(get_input(p.in1), lin), i2 = into_cs(get_input(p.in2), lin);
            auto pm = std::make_shared<Pixmap>((uint32_t)region.w, (uint32_t)region.h);
            draw_pixmap(*pm, 0, 0, *i2.image, 1.0f, RGPU_BLEND_SOURCE_OVER);
            draw_pixmap(*pm, 0, 0, *i1.image, 1.0f, (uint32_t)p.i[0]);
            res = Image{pm, IntRect{0, 0, (int32_t)pm->width, (int32_t)pm->height}, lin};
            break;
        }
        default:
            return fail();
        }
        if (!int_rect_eq(region, subregion)) {
            IntRect sub2 = p.kind == RGPU_FE_OFFSET ? IntRect{0, 0, region.w, region.h}
                                                     : IntRect{subregion.x - region.x, subregion.y - region.y,
                                                               subregion.w, subregion.h};
            auto pm = std::make_shared<Pixmap>(*res.image);
            float w = (float)pm->width, h = (float)pm->height;
            Paint clear;
            clear.shader.color = ColorF{0, 0, 0, 1};
            clear.blend = RGPU_BLEND_CLEAR;
            if (sub2.y > 0) fill_rect(*pm, Rect{0, 0, w, (float)sub2.y}, clear);
            if (sub2.x > 0) fill_rect(*pm, Rect{0, 0, (float)sub2.x, h}, clear);
            fill_rect(*pm, Rect{(float)sub2.right(), 0, (float)sub2.right() + w, h}, clear);
            fill_rect(*pm, Rect{0, (float)sub2.bottom(), w, (float)sub2.bottom() + h}, clear);
            res = Image{pm, subregion, res.linear};
        }
        results.push_back(res);
    }
    if (results.empty()) return fail();
    Image last = into_cs(results.back(), false);
    pixmap_fill(source, ColorF{0, 0, 0, 0});
    draw_pixmap(source, 0, 0, *last.image, 1.0f, RGPU_BLEND_SOURCE_OVER);
    return true;
}

}  // namespace ora

extern "C" {
// filter::apply (mod.rs:335-354) on a premultiplied RGBA8 image, in place: one
// filter with its primitives, under the layer transform ts[6] (tests only).
void oracle_filter_apply(const rgpu_filter *f, const rgpu_primitive *prims, uint32_t n, const int32_t *merge,
                         uint32_t nm, const float *ts, uint8_t *img, uint32_t w, uint32_t h) {
    rgpu_filter ff = *f;
    ff.prim_offset = 0;
    ff.prim_count = n;
    const uint32_t ref = 0;
    rgpu_tree_view view;
    std::memset(&view, 0, sizeof(view));
    view.filters = &ff; view.filter_count = 1;
    view.filter_refs = &ref; view.filter_ref_count = 1;
    view.prims = prims; view.prim_count = n;
    view.merge_inputs = merge; view.merge_input_count = nm;
    ora::Pixmap p(w, h);
    std::memcpy(p.data.data(), img, (size_t)w * h * 4);
    ora::filter_apply(view, ff, ora::Transform::from_row(ts[0], ts[1], ts[2], ts[3], ts[4], ts[5]), p);
    std::memcpy(img, p.data.data(), (size_t)w * h * 4);
}
// Direct filter-kernel oracles (tests only): operate on a premultiplied RGBA8
// image in place.
void oracle_box_blur(uint8_t *img, uint32_t w, uint32_t h, double sx, double sy) {
    ora::Pixmap p(w, h);
    std::memcpy(p.data.data(), img, (size_t)w * h * 4);
    ora::box_blur(sx, sy, p);
    std::memcpy(img, p.data.data(), (size_t)w * h * 4);
}
void oracle_iir_blur(uint8_t *img, uint32_t w, uint32_t h, double sx, double sy) {
    ora::Pixmap p(w, h);
    std::memcpy(p.data.data(), img, (size_t)w * h * 4);
    ora::iir_blur(sx, sy, p);
    std::memcpy(img, p.data.data(), (size_t)w * h * 4);
}
void oracle_morphology(uint8_t *img, uint32_t w, uint32_t h, int dilate, float rx, float ry) {
    ora::Pixmap p(w, h);
    std::memcpy(p.data.data(), img, (size_t)w * h * 4);
    ora::morphology(dilate != 0, rx, ry, p);
    std::memcpy(img, p.data.data(), (size_t)w * h * 4);
}
void oracle_to_linear(uint8_t *img, uint32_t w, uint32_t h) {
    ora::Pixmap p(w, h);
    std::memcpy(p.data.data(), img, (size_t)w * h * 4);
    ora::into_linear(p);
    std::memcpy(img, p.data.data(), (size_t)w * h * 4);
}
void oracle_to_srgb(uint8_t *img, uint32_t w, uint32_t h) {
    ora::Pixmap p(w, h);
    std::memcpy(p.data.data(), img, (size_t)w * h * 4);
    ora::into_srgb(p);
    std::memcpy(img, p.data.data(), (size_t)w * h * 4);
}
}
