// Filter-primitive kernels on premultiplied RGBA8 images (row-major, 4 B/px).
//
// Each kernel restates the arithmetic of resvg's filter module so results are
// identical to the CPU implementation:
//   colour space   filter/mod.rs:115-146 (demultiply / LUT / multiply, f32)
//   box blur       filter/box_blur.rs (integer window sums, f32 scale, round-half-even)
//   IIR blur       filter/iir_blur.rs (f64 recursions in the same order)
//   colour matrix  filter/color_matrix.rs (+ demultiply/multiply around it)
//   morphology     filter/morphology.rs (min/max over the window; the window is a
//                  rectangle, so it is applied as a row pass then a column pass)
//   arithmetic     filter/composite.rs
//   convolve       filter/convolve_matrix.rs (f32 sums in kernel order)
//   lighting       filter/lighting.rs (Sobel normals with the border variants,
//                  N.L / (N.H)^e per pixel; powf is CUDA's, within 1/255)
// All memory-bound: each pass streams its input once and writes once; the
// sliding-window passes re-read a window edge from L1/L2.
#include <cuda_runtime.h>
#include <mutex>
#include <stdint.h>
#include <algorithm>
#include "kernels.h"

namespace rgpu {
namespace {

__constant__ __align__(16) uint8_t c_srgb_to_linear[256];
__constant__ __align__(16) uint8_t c_linear_to_srgb[256];

// The two resvg tables (filter/mod.rs:161-238): the sRGB transfer functions
// evaluated and rounded to u8.
const uint8_t kSrgbToLinear[256] = {
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
const uint8_t kLinearToSrgb[256] = {
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

__device__ __forceinline__ uint32_t sat_u8f(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint32_t)v;
}
__device__ __forceinline__ uint32_t sat_u8d(double v) {
    if (!(v > 0.0)) return 0;
    if (v >= 255.0) return 255;
    return (uint32_t)v;
}
__device__ __forceinline__ uint32_t chn(uint32_t p, int i) { return (p >> (8 * i)) & 0xff; }
__device__ __forceinline__ uint32_t pk(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return r | (g << 8) | (b << 16) | (a << 24);
}
__device__ __forceinline__ float f32_bound(float mn, float v, float mx) {
    if (v > mx) return mx;
    if (v >= mn) return v;
    return mn;
}

// demultiply: (c / (a/255) + 0.5) as u8; multiply: (c * (a/255) + 0.5) as u8
__device__ __forceinline__ uint32_t demul(uint32_t p) {
    float a = (float)chn(p, 3) / 255.0f;
    return pk(sat_u8f(__fdiv_rn((float)chn(p, 0), a) + 0.5f), sat_u8f(__fdiv_rn((float)chn(p, 1), a) + 0.5f),
              sat_u8f(__fdiv_rn((float)chn(p, 2), a) + 0.5f), chn(p, 3));
}
__device__ __forceinline__ uint32_t mul(uint32_t p) {
    float a = (float)chn(p, 3) / 255.0f;
    return pk(sat_u8f((float)chn(p, 0) * a + 0.5f), sat_u8f((float)chn(p, 1) * a + 0.5f),
              sat_u8f((float)chn(p, 2) * a + 0.5f), chn(p, 3));
}

// Exact per-(alpha, channel) tables, built once on the host with the same f32
// operations as demul / mul: demultiply, multiply, and the two colour-space
// conversions (demultiply -> transfer table -> multiply) in one lookup.
enum { TAB_DEMUL = 0, TAB_MUL = 1, TAB_TO_LINEAR = 2, TAB_TO_SRGB = 3 };
__device__ uint8_t g_tab[4][256 * 256];
__device__ __forceinline__ uint32_t tab(int t, uint32_t a, uint32_t c) { return __ldg(&g_tab[t][(a << 8) | c]); }
__device__ __forceinline__ uint32_t tab_px(int t, uint32_t p) {
    const uint32_t a = p >> 24;
    // demultiply and multiply by an alpha of 255 keep every channel (the
    // table rows for a = 255 are the identity): opaque pixels skip the lookups
    if ((t == TAB_DEMUL || t == TAB_MUL) && a == 255u) return p;
    return tab(t, a, p & 0xFFu) | (tab(t, a, (p >> 8) & 0xFFu) << 8) | (tab(t, a, (p >> 16) & 0xFFu) << 16) | (a << 24);
}

// Elementwise kernels take four pixels per thread: one 16-byte access when the
// group is whole and the image 16-byte aligned, else pixel by pixel.
__device__ __forceinline__ bool vec4(const void *p, size_t i, size_t n) {
    return i + 4 <= n && (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}
#define RGPU_MAP4(img, n, F)                                                         \
    do {                                                                             \
        const size_t i_ = 4 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x);      \
        if (i_ >= (n)) return;                                                       \
        if (vec4((img), i_, (n))) {                                                  \
            uint4 v_ = *reinterpret_cast<const uint4 *>((img) + i_);                 \
            v_.x = F(v_.x); v_.y = F(v_.y); v_.z = F(v_.z); v_.w = F(v_.w);          \
            *reinterpret_cast<uint4 *>((img) + i_) = v_;                             \
        } else {                                                                     \
            for (size_t k_ = i_; k_ < (n) && k_ < i_ + 4; k_++) (img)[k_] = F((img)[k_]); \
        }                                                                            \
    } while (0)

__global__ void k_color_space(uint32_t *img, size_t n, int to_linear) {
    const int t = to_linear ? TAB_TO_LINEAR : TAB_TO_SRGB;
    auto g = [t](uint32_t p) { return tab_px(t, p); };
    RGPU_MAP4(img, n, g);
}
// the same conversion from `src` into `dst` (a private copy in the other space, one pass)
__global__ void k_color_space_copy(const uint32_t *src, uint32_t *dst, size_t n, int to_linear) {
    const int t = to_linear ? TAB_TO_LINEAR : TAB_TO_SRGB;
    const size_t i = 4 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    if (vec4(src, i, n) && vec4(dst, i, n)) {
        uint4 v = *reinterpret_cast<const uint4 *>(src + i);
        v.x = tab_px(t, v.x); v.y = tab_px(t, v.y); v.z = tab_px(t, v.z); v.w = tab_px(t, v.w);
        *reinterpret_cast<uint4 *>(dst + i) = v;
    } else {
        for (size_t k = i; k < n && k < i + 4; k++) dst[k] = tab_px(t, src[k]);
    }
}

// One box pass along lines: line l, element k at base + l*lstride + k*stride.
// Each thread produces `seg` consecutive outputs with a zero-padded sliding
// window of radius r (box_blur.rs box_blur_vert / box_blur_horz).
__global__ void k_box_pass(const uint32_t *src, uint32_t *dst, int len, int lines, size_t stride, size_t lstride,
                           int r, int seg, float iarr) {
    int nseg = (len + seg - 1) / seg;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)lines * nseg) return;
    int l = (int)(t % lines), sgi = (int)(t / lines);  // consecutive threads: consecutive lines
    const uint32_t *s = src + (size_t)l * lstride;
    uint32_t *d = dst + (size_t)l * lstride;
    int i0 = sgi * seg, i1 = min(len, i0 + seg);
    int v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    // window sum for output i0: elements [i0 - r, i0 + r] within [0, len)
    int a = max(0, i0 - r), b = min(len - 1, i0 + r);
    for (int k = a; k <= b; k++) {
        uint32_t p = s[(size_t)k * stride];
        v0 += chn(p, 0); v1 += chn(p, 1); v2 += chn(p, 2); v3 += chn(p, 3);
    }
    for (int i = i0; i < i1; i++) {
        if (i > i0) {
            int add = i + r, sub = i - r - 1;
            if (add < len) { uint32_t p = s[(size_t)add * stride]; v0 += chn(p, 0); v1 += chn(p, 1); v2 += chn(p, 2); v3 += chn(p, 3); }
            if (sub >= 0) { uint32_t p = s[(size_t)sub * stride]; v0 -= chn(p, 0); v1 -= chn(p, 1); v2 -= chn(p, 2); v3 -= chn(p, 3); }
        }
        // round(x) = x + 1.5*2^23 - 1.5*2^23 in f32: round half to even
        d[(size_t)i * stride] = pk(sat_u8f(rintf(__fmul_rn((float)v0, iarr))), sat_u8f(rintf(__fmul_rn((float)v1, iarr))),
                                   sat_u8f(rintf(__fmul_rn((float)v2, iarr))), sat_u8f(rintf(__fmul_rn((float)v3, iarr))));
    }
}

// ---- IIR (iir_blur.rs): four f64 planes (one per channel), each row and each
// column a first-order recursion run forwards then backwards `steps` times in
// exactly the reference's operation order.  A thread owns one (line, channel)
// and moves the line through registers kIirChunk values at a time, so loads
// and stores stay off the dependency chain.
constexpr int kIirChunk = 16;
__global__ void k_iir_load4(const uint32_t *img, double *planes, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = img[i];
#pragma unroll
    for (int ch = 0; ch < 4; ch++) planes[(size_t)ch * n + i] = __ddiv_rn((double)chn(p, ch), 255.0);
}
// one line of `len` values at base[k * step]; the next chunk is loaded
// before the current one is computed, so memory latency overlaps the chain
__device__ __forceinline__ void iir_load_chunk(const double *base, size_t step, int k0, int dir, int m,
                                               double (&v)[kIirChunk]) {
#pragma unroll
    for (int j = 0; j < kIirChunk; j++)
        if (j < m) v[j] = base[(ptrdiff_t)(k0 + dir * j) * (ptrdiff_t)step];
}
__device__ __forceinline__ void iir_line(double *base, size_t step, int len, double dnu, int steps) {
    for (int s = 0; s < steps; s++) {
        // forwards over k = 1 .. len-1: v[k] += dnu * v[k - 1]; backwards over
        // k = len-2 .. 0: v[k] += dnu * v[k + 1]
        for (int dir = 1; dir >= -1; dir -= 2) {
            const int first = dir > 0 ? 1 : len - 2, count = len - 1;
            double carry = base[(ptrdiff_t)(first - dir) * (ptrdiff_t)step];
            double cur[kIirChunk], nxt[kIirChunk];
            int m = min(kIirChunk, count);
            if (m > 0) iir_load_chunk(base, step, first, dir, m, cur);
            for (int done = 0; done < count; done += kIirChunk) {
                const int mn = min(kIirChunk, count - done - kIirChunk);
                if (mn > 0) iir_load_chunk(base, step, first + dir * (done + kIirChunk), dir, mn, nxt);
#pragma unroll
                for (int j = 0; j < kIirChunk; j++)
                    if (j < m) { carry = __dadd_rn(cur[j], __dmul_rn(dnu, carry)); cur[j] = carry; }
#pragma unroll
                for (int j = 0; j < kIirChunk; j++)
                    if (j < m) base[(ptrdiff_t)(first + dir * (done + j)) * (ptrdiff_t)step] = cur[j];
#pragma unroll
                for (int j = 0; j < kIirChunk; j++) cur[j] = nxt[j];
                m = mn;
            }
        }
    }
}
__global__ void k_iir_rows4(double *planes, int w, int h, double dnu, int steps) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * h) return;
    const int ch = t / h, y = t - ch * h;
    iir_line(planes + (size_t)ch * w * h + (size_t)y * w, 1, w, dnu, steps);
}
__global__ void k_iir_cols4(double *planes, int w, int h, double dnu, int steps) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * w) return;
    const int ch = t / w, x = t - ch * w;  // consecutive threads: consecutive columns
    iir_line(planes + (size_t)ch * w * h + x, (size_t)w, h, dnu, steps);
}
__global__ void k_iir_store4(uint32_t *img, const double *planes, size_t n, double post) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t o = 0;
#pragma unroll
    for (int ch = 0; ch < 4; ch++) o |= sat_u8d(__dmul_rn(__dmul_rn(planes[(size_t)ch * n + i], post), 255.0)) << (8 * ch);
    img[i] = o;
}

// c / 255 in f32 for every u8 c, the IEEE quotient (host division is IEEE
// too): kernels read it from shared memory instead of dividing per channel.
__device__ float g_unit[256];
__device__ __forceinline__ void load_unit(float *u) {
    for (int k = threadIdx.x; k < 256; k += blockDim.x) u[k] = g_unit[k];
}
// ---- colour matrix (color_matrix.rs), demultiply and multiply fused
struct CmParams { int kind; float m[20]; };
__device__ __forceinline__ uint32_t from_normalized(float c) { return sat_u8f(f32_bound(0.0f, c, 1.0f) * 255.0f); }
// `unit[c]` = c / 255 (the IEEE quotient, from a table instead of a division per channel)
__device__ __forceinline__ uint32_t color_matrix_px(uint32_t px, const CmParams &cp, const float *unit) {
    uint32_t p = tab_px(TAB_DEMUL, px);
    float r = unit[chn(p, 0)], g = unit[chn(p, 1)], b = unit[chn(p, 2)], a = unit[chn(p, 3)];
    const float *m = cp.m;
    uint32_t o;
    if (cp.kind == 0) {
        float nr = r * m[0] + g * m[1] + b * m[2] + a * m[3] + m[4];
        float ng = r * m[5] + g * m[6] + b * m[7] + a * m[8] + m[9];
        float nb = r * m[10] + g * m[11] + b * m[12] + a * m[13] + m[14];
        float na = r * m[15] + g * m[16] + b * m[17] + a * m[18] + m[19];
        o = pk(from_normalized(nr), from_normalized(ng), from_normalized(nb), from_normalized(na));
    } else if (cp.kind == 1) {
        o = pk(from_normalized(r * m[0] + g * m[1] + b * m[2]), from_normalized(r * m[3] + g * m[4] + b * m[5]),
               from_normalized(r * m[6] + g * m[7] + b * m[8]), chn(p, 3));
    } else {
        float na = r * 0.2125f + g * 0.7154f + b * 0.0721f;
        o = pk(0, 0, 0, from_normalized(na));
    }
    return tab_px(TAB_MUL, o);
}
__global__ void k_color_matrix(const uint32_t *src, uint32_t *dst, size_t n, CmParams cp) {
    __shared__ float u[256];
    load_unit(u);
    __syncthreads();
    const size_t i = 4 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    if (vec4(src, i, n) && vec4(dst, i, n)) {
        uint4 v = *reinterpret_cast<const uint4 *>(src + i);
        v.x = color_matrix_px(v.x, cp, u); v.y = color_matrix_px(v.y, cp, u);
        v.z = color_matrix_px(v.z, cp, u); v.w = color_matrix_px(v.w, cp, u);
        *reinterpret_cast<uint4 *>(dst + i) = v;
    } else {
        for (size_t k = i; k < n && k < i + 4; k++) dst[k] = color_matrix_px(src[k], cp, u);
    }
}

// ---- morphology: window [x - tx, x - tx + cols) x [y - ty, y - ty + rows),
// out-of-range taps skipped; per channel min (erode) / max (dilate).
__global__ void k_morph_pass(const uint32_t *src, uint32_t *dst, int len, int lines, size_t stride, size_t lstride,
                             int taps, int target, int dilate) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)len * lines) return;
    // consecutive threads take consecutive pixels in memory: along the line
    // for a row pass (stride 1), across lines for a column pass
    int l, i;
    if (stride == 1) { l = (int)(t / len); i = (int)(t % len); }
    else { l = (int)(t % lines); i = (int)(t / lines); }
    const uint32_t *s = src + (size_t)l * lstride;
    uint32_t c0 = dilate ? 0 : 255, c1 = c0, c2 = c0, c3 = c0;
    for (int o = 0; o < taps; o++) {
        int k = i - target + o;
        if (k < 0 || k >= len) continue;
        uint32_t p = s[(size_t)k * stride];
        if (dilate) { c0 = max(c0, chn(p, 0)); c1 = max(c1, chn(p, 1)); c2 = max(c2, chn(p, 2)); c3 = max(c3, chn(p, 3)); }
        else { c0 = min(c0, chn(p, 0)); c1 = min(c1, chn(p, 1)); c2 = min(c2, chn(p, 2)); c3 = min(c3, chn(p, 3)); }
    }
    dst[(size_t)l * lstride + (size_t)i * stride] = pk(c0, c1, c2, c3);
}

// ---- arithmetic composite (composite.rs)
__device__ __forceinline__ bool approx_zero_ulps4(float v) {
    int32_t a = __float_as_int(v);
    if (a < 0) return v == 0.0f;
    return a <= 4;
}
__device__ __forceinline__ uint32_t arithmetic_px(uint32_t c1, uint32_t c2, float k1, float k2, float k3, float k4,
                                                  const float *u) {
    auto calc = [&](uint32_t i1, uint32_t i2, float mx) {
        float a = u[i1], b = u[i2];
        float r = k1 * a * b + k2 * a + k3 * b + k4;
        return f32_bound(0.0f, r, mx);
    };
    float a = calc(chn(c1, 3), chn(c2, 3), 1.0f);
    if (approx_zero_ulps4(a)) return 0u;  // pixel left as initialised (transparent)
    return pk(sat_u8f(calc(chn(c1, 0), chn(c2, 0), a) * 255.0f), sat_u8f(calc(chn(c1, 1), chn(c2, 1), a) * 255.0f),
              sat_u8f(calc(chn(c1, 2), chn(c2, 2), a) * 255.0f), sat_u8f(a * 255.0f));
}
__global__ void k_arithmetic(const uint32_t *s1, const uint32_t *s2, uint32_t *dst, size_t n, float k1, float k2,
                             float k3, float k4) {
    __shared__ float u[256];
    load_unit(u);
    __syncthreads();
    for (size_t i = 4 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (size_t)gridDim.x * blockDim.x) {
        if (vec4(s1, i, n) && vec4(s2, i, n) && vec4(dst, i, n)) {
            const uint4 a = *reinterpret_cast<const uint4 *>(s1 + i), b = *reinterpret_cast<const uint4 *>(s2 + i);
            *reinterpret_cast<uint4 *>(dst + i) =
                make_uint4(arithmetic_px(a.x, b.x, k1, k2, k3, k4, u), arithmetic_px(a.y, b.y, k1, k2, k3, k4, u),
                           arithmetic_px(a.z, b.z, k1, k2, k3, k4, u), arithmetic_px(a.w, b.w, k1, k2, k3, k4, u));
        } else {
            for (size_t k = i; k < n && k < i + 4; k++) dst[k] = arithmetic_px(s1[k], s2[k], k1, k2, k3, k4, u);
        }
    }
}

inline uint32_t nblk(size_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }
// at most 8 CTAs per SM, for grid-stride kernels that set up shared tables
uint32_t nblk_capped(size_t n, uint32_t t) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    }
    return std::max<uint32_t>(1u, std::min<uint32_t>(nblk(n, t), (uint32_t)sms * 8u));
}

uint32_t host_sat_u8(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint32_t)v;
}
bool g_luts_ready = false;
// host copy of g_tab, for tables derived from it on the host
uint8_t g_host_tab[4][256 * 256];
cudaError_t ensure_luts() {
    if (g_luts_ready) return cudaSuccess;
    cudaError_t e = cudaMemcpyToSymbol(c_srgb_to_linear, kSrgbToLinear, 256);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_linear_to_srgb, kLinearToSrgb, 256);
    float unit[256];
    for (int k = 0; k < 256; k++) unit[k] = (float)k / 255.0f;
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_unit, unit, sizeof(unit));
    // the same f32 operations as demul / mul (host and device division and
    // multiplication are both IEEE round-to-nearest, without contraction)
    uint8_t (*t)[256 * 256] = g_host_tab;
    for (uint32_t a = 0; a < 256 && e == cudaSuccess; a++) {
        const float af = (float)a / 255.0f;
        for (uint32_t c = 0; c < 256; c++) {
            const uint32_t d = host_sat_u8((float)c / af + 0.5f);
            t[TAB_DEMUL][(a << 8) | c] = (uint8_t)d;
            t[TAB_MUL][(a << 8) | c] = (uint8_t)host_sat_u8((float)c * af + 0.5f);
        }
    }
    for (uint32_t a = 0; a < 256 && e == cudaSuccess; a++) {
        for (uint32_t c = 0; c < 256; c++) {
            const uint32_t d = t[TAB_DEMUL][(a << 8) | c];
            t[TAB_TO_LINEAR][(a << 8) | c] = t[TAB_MUL][(a << 8) | kSrgbToLinear[d]];
            t[TAB_TO_SRGB][(a << 8) | c] = t[TAB_MUL][(a << 8) | kLinearToSrgb[d]];
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tab, g_host_tab, sizeof(g_host_tab));
    if (e == cudaSuccess) g_luts_ready = true;
    return e;
}

}  // namespace

// ---------------------------------------------------------------- launchers
cudaError_t filter_color_space(uint32_t *img, size_t n, bool to_linear, cudaStream_t s) {
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess || n == 0) return e;
    k_color_space<<<nblk((n + 3) / 4, 256), 256, 0, s>>>(img, n, to_linear ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t filter_color_space_copy(const uint32_t *src, uint32_t *dst, size_t n, bool to_linear, cudaStream_t s) {
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    k_color_space_copy<<<nblk((n + 3) / 4, 256), 256, 0, s>>>(src, dst, n, to_linear ? 1 : 0);
    return cudaGetLastError();
}

// box_blur.rs create_box_gauss
void box_sizes(float sigma, int sizes[5]) {
    if (sigma > 0.0f) {
        float nf = 5.0f;
        float w_ideal = sqrtf(12.0f * sigma * sigma / nf) + 1.0f;
        int wl = (int)floorf(w_ideal);
        if (wl % 2 == 0) wl -= 1;
        int wu = wl + 2;
        float wlf = (float)wl;
        float m_ideal = (12.0f * sigma * sigma - nf * wlf * wlf - 4.0f * nf * wlf - 3.0f * nf) / (-4.0f * wlf - 4.0f);
        float mr = roundf(m_ideal);
        int m = mr <= 0.0f ? 0 : (int)mr;
        for (int i = 0; i < 5; i++) sizes[i] = i < m ? wl : wu;
    } else {
        for (int i = 0; i < 5; i++) sizes[i] = 1;
    }
}

// Shared-memory tiled box passes (same sums and rounding as k_box_pass, which
// stays for radii beyond the tile halo).  Loads and stores are coalesced; each
// thread slides the zero-padded window over 32 outputs inside the tile.
constexpr int kBoxT = 128;     // outputs along the pass per tile
constexpr int kBoxMaxR = 96;   // largest radius the tiles take
// Window sums as two 16-bit lanes per register (r | b << 16, g | a << 16): a
// lane holds at most (2 * kBoxMaxR + 1) * 255 + kBoxMaxR < 65536 at any step,
// so lanes never carry or borrow into each other.  The reference rounds the
// f32 product sum * (1 / (2r + 1)) half to even; the quotient is never within
// 1 / (2 (2r + 1)) of a half while the f32 error stays below 2^-15, so that
// equals the integer (sum + r) / (2r + 1), here a multiply-high by
// m = ceil(2^32 / (2r + 1)) (exact for sums below 2^16; both identities are
// checked exhaustively in the tests).  No int <-> float conversions.
__device__ __forceinline__ uint32_t box_round2(uint32_t rb, uint32_t ga, uint32_t r, uint32_t m) {
    if (m == 0u) return rb | (ga << 8);  // r = 0: the window is the pixel itself
    rb += r * 0x10001u;
    ga += r * 0x10001u;
    const uint32_t cr = __umulhi(rb & 0xFFFFu, m), cb = __umulhi(rb >> 16, m);
    const uint32_t cg = __umulhi(ga & 0xFFFFu, m), ca = __umulhi(ga >> 16, m);
    return cr | (cg << 8) | (cb << 16) | (ca << 24);
}
inline uint32_t box_magic(int r) {
    return r == 0 ? 0u : (uint32_t)((0x100000000ull + (uint64_t)(2 * r)) / (uint64_t)(2 * r + 1));
}
#define BOX_ADD(p) do { rb += (p) & 0x00FF00FFu; ga += ((p) >> 8) & 0x00FF00FFu; } while (0)
#define BOX_SLIDE(pa, ps)                                                         \
    do {                                                                          \
        rb = rb + ((pa) & 0x00FF00FFu) - ((ps) & 0x00FF00FFu);                    \
        ga = ga + (((pa) >> 8) & 0x00FF00FFu) - (((ps) >> 8) & 0x00FF00FFu);      \
    } while (0)

// vertical: tile of 32 columns x kBoxT rows; thread (lane = column, warp = 32-row group)
__global__ void __launch_bounds__(256) k_box_v(const uint32_t *src, uint32_t *dst, int w, int h, int r, uint32_t m) {
    extern __shared__ uint32_t tile[];  // (kBoxT + 2r) rows x 32
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * kBoxT;
    const int rows = kBoxT + 2 * r;
    if ((w & 3) == 0 && x0 + 32 <= w) {
        // 16-byte loads: 8 threads per tile row, several rows in flight per thread
        const int q = threadIdx.x & 7;
#pragma unroll 4
        for (int ry = threadIdx.x >> 3; ry < rows; ry += 32) {
            const int y = y0 - r + ry;
            const uint4 v = (y >= 0 && y < h) ? __ldg(reinterpret_cast<const uint4 *>(src + (size_t)y * w + x0) + q)
                                              : make_uint4(0u, 0u, 0u, 0u);
            reinterpret_cast<uint4 *>(tile + ry * 32)[q] = v;
        }
    } else {
#pragma unroll 4
        for (int i = threadIdx.x; i < rows * 32; i += 256) {
            const int ry = i >> 5, x = x0 + (i & 31), y = y0 - r + ry;
            tile[i] = (x < w && y >= 0 && y < h) ? src[(size_t)y * w + x] : 0u;
        }
    }
    __syncthreads();
    const int c = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int x = x0 + c;
    constexpr int kPer = kBoxT / 8;  // outputs per thread
    const int oy0 = g * kPer;        // first output row of this thread, tile-relative
    uint32_t rb = 0, ga = 0;
    // window of output oy0: tile rows oy0 .. oy0 + 2r
    for (int k = oy0; k <= oy0 + 2 * r; k++) {
        const uint32_t p = tile[k * 32 + c];
        BOX_ADD(p);
    }
#pragma unroll 4
    for (int i = 0; i < kPer; i++) {
        const int oy = oy0 + i, y = y0 + oy;
        if (i > 0) {
            const uint32_t pa = tile[(oy + 2 * r) * 32 + c], ps = tile[(oy - 1) * 32 + c];
            BOX_SLIDE(pa, ps);
        }
        if (x < w && y < h) dst[(size_t)y * w + x] = box_round2(rb, ga, (uint32_t)r, m);
    }
}

// horizontal: tile of 32 rows x kBoxT columns; thread (lane = row, warp = 32-column
// group); the outputs go through shared memory so the stores are row-coalesced
__global__ void __launch_bounds__(256) k_box_h(const uint32_t *src, uint32_t *dst, int w, int h, int r, uint32_t m) {
    extern __shared__ uint32_t tile[];
    const int cols = kBoxT + 2 * r, stride = cols | 1;  // odd row stride: lanes hit distinct banks
    uint32_t *out = tile + 32 * stride;                  // 32 rows x (kBoxT + 1)
    const int ostride = kBoxT + 1;
    const int x0 = blockIdx.x * kBoxT, y0 = blockIdx.y * 32;
    // each warp copies rows: lane-consecutive columns, several loads in flight
    const int wp = threadIdx.x >> 5, ln = threadIdx.x & 31;
    for (int ry = wp; ry < 32; ry += 8) {
        const int y = y0 + ry;
        const uint32_t *srow = src + (size_t)y * w;
#pragma unroll 4
        for (int cx = ln; cx < cols; cx += 32) {
            const int x = x0 - r + cx;
            tile[ry * stride + cx] = (y < h && x >= 0 && x < w) ? __ldg(srow + x) : 0u;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    const uint32_t *row = tile + lane * stride;
    constexpr int kPer = kBoxT / 8;
    const int ox0 = g * kPer;
    uint32_t rb = 0, ga = 0;
    for (int k = ox0; k <= ox0 + 2 * r; k++) {
        const uint32_t p = row[k];
        BOX_ADD(p);
    }
#pragma unroll 4
    for (int i = 0; i < kPer; i++) {
        const int ox = ox0 + i;
        if (i > 0) {
            const uint32_t pa = row[ox + 2 * r], ps = row[ox - 1];
            BOX_SLIDE(pa, ps);
        }
        out[lane * ostride + ox] = box_round2(rb, ga, (uint32_t)r, m);
    }
    __syncthreads();
    for (int ry = wp; ry < 32; ry += 8) {
        const int y = y0 + ry;
        if (y >= h) break;
#pragma unroll 4
        for (int cx = ln; cx < kBoxT; cx += 32) {
            const int x = x0 + cx;
            if (x < w) dst[(size_t)y * w + x] = out[ry * ostride + cx];
        }
    }
}

// Tiles of the fused morphology kernel.
constexpr int kPairTX = 64, kPairTY = 32, kPairSeg = 16;
// (b0, b2) and (b1, b3) of a pixel as two 16-bit lanes
__device__ __forceinline__ uint32_t lanes02(uint32_t p) { return __byte_perm(p, 0u, 0x4240); }
__device__ __forceinline__ uint32_t lanes13(uint32_t p) { return __byte_perm(p, 0u, 0x4341); }

// Morphology passes on the same tiles: window [i - target, i - target + taps)
// along the pass, taps outside the image skipped (= the identity of min / max
// as padding), per-byte min or max of the premultiplied pixels.
__device__ __forceinline__ uint32_t morph_op(uint32_t a, uint32_t b, bool dilate) {
    return dilate ? __vmaxu4(a, b) : __vminu4(a, b);
}
__global__ void __launch_bounds__(256) k_morph_v(const uint32_t *src, uint32_t *dst, int w, int h, int taps,
                                                 int target, int dilate) {
    extern __shared__ uint32_t tile[];
    const uint32_t pad = dilate ? 0u : 0xFFFFFFFFu;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * kBoxT;
    const int rows = kBoxT + taps - 1;
    for (int i = threadIdx.x; i < rows * 32; i += 256) {
        const int ry = i >> 5, x = x0 + (i & 31), y = y0 - target + ry;
        tile[i] = (x < w && y >= 0 && y < h) ? __ldg(src + (size_t)y * w + x) : pad;
    }
    __syncthreads();
    const int c = threadIdx.x & 31, g = threadIdx.x >> 5, x = x0 + c;
    constexpr int kPer = kBoxT / 8;
    for (int i = 0; i < kPer; i++) {
        const int oy = g * kPer + i, y = y0 + oy;
        uint32_t v = pad;
        for (int k = 0; k < taps; k++) v = morph_op(v, tile[(oy + k) * 32 + c], dilate != 0);
        if (x < w && y < h) dst[(size_t)y * w + x] = v;
    }
}
__global__ void __launch_bounds__(256) k_morph_h(const uint32_t *src, uint32_t *dst, int w, int h, int taps,
                                                 int target, int dilate) {
    extern __shared__ uint32_t tile[];
    const uint32_t pad = dilate ? 0u : 0xFFFFFFFFu;
    const int cols = kBoxT + taps - 1, stride = cols | 1;
    uint32_t *out = tile + 32 * stride;
    const int ostride = kBoxT + 1;
    const int x0 = blockIdx.x * kBoxT, y0 = blockIdx.y * 32;
    const int wp = threadIdx.x >> 5, ln = threadIdx.x & 31;
    for (int ry = wp; ry < 32; ry += 8) {
        const int y = y0 + ry;
        const uint32_t *srow = src + (size_t)y * w;
        for (int cx = ln; cx < cols; cx += 32) {
            const int x = x0 - target + cx;
            tile[ry * stride + cx] = (y < h && x >= 0 && x < w) ? __ldg(srow + x) : pad;
        }
    }
    __syncthreads();
    const uint32_t *row = tile + ln * stride;
    constexpr int kPer = kBoxT / 8;
    for (int i = 0; i < kPer; i++) {
        const int ox = wp * kPer + i;
        uint32_t v = pad;
        for (int k = 0; k < taps; k++) v = morph_op(v, row[ox + k], dilate != 0);
        out[ln * ostride + ox] = v;
    }
    __syncthreads();
    for (int ry = wp; ry < 32; ry += 8) {
        const int y = y0 + ry;
        if (y >= h) break;
        for (int cx = ln; cx < kBoxT; cx += 32) {
            const int x = x0 + cx;
            if (x < w) dst[(size_t)y * w + x] = out[ry * ostride + cx];
        }
    }
}
// Both morphology passes fused on a TX x TY tile: the tile and its window
// halo are loaded once, columns then rows are reduced in shared memory (the
// rectangle's min / max is separable and exact, so this is the reference's
// 2-D window), and the tile leaves in coalesced rows.  Pixels are split into
// (r, b) and (g, a) 16-bit lanes so one 16x2 min / max handles two channels.
constexpr int kMorphPairMaxTaps = 64;
size_t morph_pair_smem(int tx, int ty) {
    const size_t st = (size_t)((kPairTX + tx - 1) | 1);
    return ((size_t)(kPairTY + ty - 1) * st + (size_t)kPairTY * st) * 4;
}
__device__ __forceinline__ uint32_t mm2(uint32_t a, uint32_t b, bool dilate) {
    return dilate ? __vmaxu2(a, b) : __vminu2(a, b);
}
__global__ void __launch_bounds__(256) k_morph_vh(const uint32_t *src, uint32_t *dst, int w, int h, int tx, int ty,
                                                  int ox, int oy, int dilate) {
    extern __shared__ uint32_t smem[];
    constexpr int TX = kPairTX, TY = kPairTY, SEG = kPairSeg;
    const bool dil = dilate != 0;
    const uint32_t pad = dil ? 0u : 0xFFFFFFFFu, pad2 = dil ? 0u : 0x00FF00FFu;
    const int cols = TX + tx - 1, rows = TY + ty - 1, st = cols | 1, cst = TX + 1;
    uint32_t *A = smem, *B = smem + rows * st, *C = smem;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int wp = threadIdx.x >> 5, ln = threadIdx.x & 31;
    for (int ry = wp; ry < rows; ry += 8) {
        const int y = y0 - oy + ry;
        const bool yin = y >= 0 && y < h;
        const uint32_t *srow = src + (size_t)(yin ? y : 0) * w;
#pragma unroll 4
        for (int cx = ln; cx < cols; cx += 32) {
            const int x = x0 - ox + cx;
            A[ry * st + cx] = (yin && x >= 0 && x < w) ? __ldg(srow + x) : pad;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < cols * (TY / SEG); t += 256) {
        const int c = t % cols, o0 = (t / cols) * SEG;
#pragma unroll 2
        for (int i = 0; i < SEG; i++) {
            const int o = o0 + i;
            uint32_t vr = pad2, vg = pad2;
            for (int k = 0; k < ty; k++) {
                const uint32_t p = A[(o + k) * st + c];
                vr = mm2(vr, lanes02(p), dil);
                vg = mm2(vg, lanes13(p), dil);
            }
            B[o * st + c] = vr | (vg << 8);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < TY * (TX / SEG); t += 256) {
        const int r = t % TY, o0 = (t / TY) * SEG;
        const uint32_t *row = B + r * st;
#pragma unroll 2
        for (int i = 0; i < SEG; i++) {
            const int o = o0 + i;
            uint32_t vr = pad2, vg = pad2;
            for (int k = 0; k < tx; k++) {
                const uint32_t p = row[o + k];
                vr = mm2(vr, lanes02(p), dil);
                vg = mm2(vg, lanes13(p), dil);
            }
            C[r * cst + o] = vr | (vg << 8);
        }
    }
    __syncthreads();
    for (int ry = wp; ry < TY; ry += 8) {
        const int y = y0 + ry;
        if (y >= h) break;
        uint32_t *drow = dst + (size_t)y * w;
#pragma unroll 4
        for (int cx = ln; cx < TX; cx += 32) {
            const int x = x0 + cx;
            if (x < w) drow[x] = C[ry * cst + cx];
        }
    }
}
size_t morph_v_smem(int taps) { return (size_t)(kBoxT + taps - 1) * 32 * 4; }
size_t morph_h_smem(int taps) { return ((size_t)32 * ((kBoxT + taps - 1) | 1) + (size_t)32 * (kBoxT + 1)) * 4; }
constexpr int kMorphMaxTaps = 192;

size_t box_v_smem(int r) { return (size_t)(kBoxT + 2 * r) * 32 * 4; }
size_t box_h_smem(int r) { return ((size_t)32 * ((kBoxT + 2 * r) | 1) + (size_t)32 * (kBoxT + 1)) * 4; }

// The shared-memory opt-ins are per device: a flag per device index, set
// under a lock once the attributes are in place on that device.
cudaError_t box_attrs() {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static bool done[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_box_v, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)box_v_smem(kBoxMaxR));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_box_h, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)box_h_smem(kBoxMaxR));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_morph_v, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)morph_v_smem(kMorphMaxTaps));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_morph_h, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)morph_h_smem(kMorphMaxTaps));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_morph_vh, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)morph_pair_smem(kMorphPairMaxTaps, kMorphPairMaxTaps));
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

// 5 x (vertical pass img -> tmp, horizontal pass tmp -> img)
cudaError_t filter_box_blur(uint32_t *img, uint32_t *tmp, int w, int h, double sx, double sy, cudaStream_t s) {
    // Beyond kBoxSigmaMax every box radius exceeds 256 x the longest line a
    // layer can have, so each pass already rounds every sum to zero; the clamp
    // keeps the box sizes inside int range without changing the result.
    // Non-finite or negative deviations mean no blur along that axis.
    sx = (sx >= 0.0 && sx <= kBoxSigmaMax) ? sx : (sx > kBoxSigmaMax ? kBoxSigmaMax : 0.0);
    sy = (sy >= 0.0 && sy <= kBoxSigmaMax) ? sy : (sy > kBoxSigmaMax ? kBoxSigmaMax : 0.0);
    int bh[5], bv[5];
    box_sizes((float)sx, bh);
    box_sizes((float)sy, bv);
    const int seg = 32;
    size_t n = (size_t)w * h;
    cudaError_t ae = box_attrs();
    if (ae != cudaSuccess) return ae;
    for (int i = 0; i < 5; i++) {
        int rh = (bh[i] - 1) / 2, rv = (bv[i] - 1) / 2;
        if (rv == 0) {
            cudaError_t ce = cudaMemcpyAsync(tmp, img, n * 4, cudaMemcpyDeviceToDevice, s);
            if (ce != cudaSuccess) return ce;
        }
        else if (rv <= kBoxMaxR) {
            dim3 g((unsigned)((w + 31) / 32), (unsigned)((h + kBoxT - 1) / kBoxT));
            k_box_v<<<g, 256, box_v_smem(rv), s>>>(img, tmp, w, h, rv, box_magic(rv));
        } else {
            size_t th = (size_t)w * ((h + seg - 1) / seg);
            k_box_pass<<<nblk(th, 256), 256, 0, s>>>(img, tmp, h, w, (size_t)w, 1, rv, seg, 1.0f / (float)(rv + rv + 1));
        }
        if (rh == 0) {
            cudaError_t ce = cudaMemcpyAsync(img, tmp, n * 4, cudaMemcpyDeviceToDevice, s);
            if (ce != cudaSuccess) return ce;
        }
        else if (rh <= kBoxMaxR) {
            dim3 g((unsigned)((w + kBoxT - 1) / kBoxT), (unsigned)((h + 31) / 32));
            k_box_h<<<g, 256, box_h_smem(rh), s>>>(tmp, img, w, h, rh, box_magic(rh));
        } else {
            size_t th = (size_t)h * ((w + seg - 1) / seg);
            k_box_pass<<<nblk(th, 256), 256, 0, s>>>(tmp, img, w, h, 1, (size_t)w, rh, seg, 1.0f / (float)(rh + rh + 1));
        }
    }
    return cudaGetLastError();
}

// ---- IIR blur, FP32 chunked-scan mode (opt-in; within 1/255 of the f64 path).
// Each line's first-order recursions (rightwards y[i] = x[i] + d y[i-1], then
// leftwards y[i] = y[i] + d y[i+1], `steps` times) run in parallel: a line is
// held by one 256-thread CTA, each thread owning E consecutive values in
// registers; a thread first runs the recursion over its chunk from zero, the
// chunk-end values are scanned across the CTA (the carry into chunk t is
// end(t-1) + d^E carry(t-1)), and value k of a chunk then gets d^(k+1) carry.
// Columns are rows of the transposed planes.
constexpr int kIirLine = 256;
constexpr int kIirFastMaxE = 16;  // lines of up to 4096 values
bool g_iir_fast = false;

// Exclusive scan of y_t = e_t + D y_(t-1) over the 256 threads of the CTA, in
// thread order (reverse = false) or from the last thread down (reverse = true):
// the carry a thread's chunk receives.
__device__ float iir_block_carry(float e, float D, bool reverse, float *tot) {
    const int t = reverse ? kIirLine - 1 - (int)threadIdx.x : (int)threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    // threads are renumbered by t; lanes of a hardware warp keep their order
    // or reverse it as a whole, so shuffles run on t's lane
    const unsigned full = 0xffffffffu;
    float v = e, Dk = D;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int src_hw = reverse ? (int)threadIdx.x + off : (int)threadIdx.x - off;
        const float u = __shfl_sync(full, v, src_hw & 31);
        if (lane >= off) v = v + Dk * u;
        Dk = Dk * Dk;  // D^(2 off)
    }
    // Dk = D^32 now; warp totals, then the carry into each warp
    if (lane == 31) tot[warp] = v;
    __syncthreads();
    float cw = 0.0f;
    for (int k = 0; k < warp; k++) cw = tot[k] + Dk * cw;
    // inclusive value of this thread, then the previous thread's (exclusive)
    float dl = D;  // D^(lane + 1)
    for (int k = 0; k < lane; k++) dl = dl * D;
    const float incl = v + dl * cw;
    const int src_hw = reverse ? (int)threadIdx.x + 1 : (int)threadIdx.x - 1;
    float prev = __shfl_sync(full, incl, src_hw & 31);
    __syncthreads();  // tot[] is reused by the next scan
    return lane == 0 ? cw : prev;
}

__global__ void __launch_bounds__(kIirLine) k_iir_fast_lines(float *planes, int len, float d, int steps) {
    __shared__ float tot[kIirLine / 32];
    float *line = planes + (size_t)blockIdx.x * len;
    const int E = (len + kIirLine - 1) / kIirLine;
    const int first = (int)threadIdx.x * E;
    float v[kIirFastMaxE];
#pragma unroll
    for (int k = 0; k < kIirFastMaxE; k++) v[k] = (k < E && first + k < len) ? line[first + k] : 0.0f;
    float dE = 1.0f;
    for (int k = 0; k < E; k++) dE = dE * d;
    for (int st = 0; st < steps; st++) {
        // rightwards
        float y = 0.0f;
#pragma unroll
        for (int k = 0; k < kIirFastMaxE; k++)
            if (k < E) { y = v[k] + d * y; v[k] = y; }
        float c = iir_block_carry(y, dE, false, tot);
        float p = d;
#pragma unroll
        for (int k = 0; k < kIirFastMaxE; k++)
            if (k < E) { v[k] = (first + k < len) ? v[k] + p * c : 0.0f; p = p * d; }
        // leftwards
        y = 0.0f;
#pragma unroll
        for (int k = kIirFastMaxE - 1; k >= 0; k--)
            if (k < E) { y = v[k] + d * y; v[k] = y; }
        c = iir_block_carry(y, dE, true, tot);
        p = d;
#pragma unroll
        for (int k = kIirFastMaxE - 1; k >= 0; k--)
            if (k < E) { v[k] = v[k] + p * c; p = p * d; }
    }
#pragma unroll
    for (int k = 0; k < kIirFastMaxE; k++)
        if (k < E && first + k < len) line[first + k] = v[k];
}

__global__ void k_iir_fast_load(const uint32_t *img, float *planes, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = img[i];
#pragma unroll
    for (int ch = 0; ch < 4; ch++) planes[(size_t)ch * n + i] = __ldg(&g_unit[chn(p, ch)]);
}

__global__ void k_iir_fast_store(uint32_t *img, const float *planes, size_t n, float post) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t o = 0;
#pragma unroll
    for (int ch = 0; ch < 4; ch++) o |= sat_u8f(planes[(size_t)ch * n + i] * post * 255.0f) << (8 * ch);
    img[i] = o;
}

// 4 planes of h rows x w columns -> 4 planes of w rows x h columns
__global__ void k_iir_transpose(const float *src, float *dst, int w, int h) {
    __shared__ float tile[32][33];
    const size_t n = (size_t)w * h;
    const float *sp = src + (size_t)blockIdx.z * n;
    float *dp = dst + (size_t)blockIdx.z * n;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = x0 + threadIdx.x, y = y0 + j;
        if (x < w && y < h) tile[j][threadIdx.x] = sp[(size_t)y * w + x];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = y0 + threadIdx.x, y = x0 + j;  // dst is h wide, w tall
        if (x < h && y < w) dp[(size_t)y * h + x] = tile[threadIdx.x][j];
    }
}

void filter_set_iir_fast(bool on) { g_iir_fast = on; }
bool filter_iir_fast() { return g_iir_fast; }

// buf: 32 bytes per pixel (the f64 mode's four planes), here 2 x 4 f32 planes
static cudaError_t iir_blur_fast(uint32_t *img, float *a, float *b, int w, int h, double dx, double dy, bool bx,
                                 bool by, double post, cudaStream_t s) {
    const int steps = 4;
    const size_t n = (size_t)w * h;
    cudaError_t te = ensure_luts();  // the c / 255 table the load reads
    if (te != cudaSuccess) return te;
    k_iir_fast_load<<<nblk(n, 256), 256, 0, s>>>(img, a, n);
    if (bx) k_iir_fast_lines<<<(unsigned)(4 * h), kIirLine, 0, s>>>(a, w, (float)dx, steps);
    if (by) {
        const dim3 blk(32, 8);
        k_iir_transpose<<<dim3((w + 31) / 32, (h + 31) / 32, 4), blk, 0, s>>>(a, b, w, h);
        k_iir_fast_lines<<<(unsigned)(4 * w), kIirLine, 0, s>>>(b, h, (float)dy, steps);
        k_iir_transpose<<<dim3((h + 31) / 32, (w + 31) / 32, 4), blk, 0, s>>>(b, a, h, w);
    }
    k_iir_fast_store<<<nblk(n, 256), 256, 0, s>>>(img, a, n, (float)post);
    return cudaGetLastError();
}

cudaError_t filter_iir_blur(uint32_t *img, double *buf, int w, int h, double sx, double sy, cudaStream_t s) {
    const int steps = 4;
    double lx = 1.0, dx = 1.0, ly = 1.0, dy = 1.0;
    if (sx > 0.0) { lx = (sx * sx) / (2.0 * steps); dx = (1.0 + 2.0 * lx - sqrt(1.0 + 4.0 * lx)) / (2.0 * lx); }
    if (sy > 0.0) { ly = (sy * sy) / (2.0 * steps); dy = (1.0 + 2.0 * ly - sqrt(1.0 + 4.0 * ly)) / (2.0 * ly); }
    double post = pow(sqrt(dx * dy) / sqrt(lx * ly), 2 * steps);
    size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    if (g_iir_fast && w <= kIirLine * kIirFastMaxE && h <= kIirLine * kIirFastMaxE)
        return iir_blur_fast(img, reinterpret_cast<float *>(buf), reinterpret_cast<float *>(buf) + 4 * n, w, h, dx,
                             dy, sx > 0.0, sy > 0.0, post, s);
    // buf holds four planes of n doubles
    k_iir_load4<<<nblk(n, 256), 256, 0, s>>>(img, buf, n);
    if (sx > 0.0) k_iir_rows4<<<nblk((size_t)4 * h, 64), 64, 0, s>>>(buf, w, h, dx, steps);
    if (sy > 0.0) k_iir_cols4<<<nblk((size_t)4 * w, 64), 64, 0, s>>>(buf, w, h, dy, steps);
    k_iir_store4<<<nblk(n, 256), 256, 0, s>>>(img, buf, n, post);
    return cudaGetLastError();
}

cudaError_t filter_color_matrix(uint32_t *img, size_t n, int kind, const float *values, cudaStream_t s) {
    return filter_color_matrix_to(img, img, n, kind, values, s);
}

cudaError_t filter_color_matrix_to(const uint32_t *src, uint32_t *dst, size_t n, int kind, const float *values,
                                   cudaStream_t s) {
    CmParams cp;
    cp.kind = 0;
    for (int i = 0; i < 20; i++) cp.m[i] = 0.0f;
    if (kind == RGPU_CM_MATRIX) {
        cp.kind = 0;
        for (int i = 0; i < 20; i++) cp.m[i] = values[i];
    } else if (kind == RGPU_CM_SATURATE || kind == RGPU_CM_HUE_ROTATE) {
        cp.kind = 1;
        if (kind == RGPU_CM_SATURATE) {
            float v = fmaxf(values[0], 0.0f);
            float m[9] = {0.213f + 0.787f * v, 0.715f - 0.715f * v, 0.072f - 0.072f * v,
                          0.213f - 0.213f * v, 0.715f + 0.285f * v, 0.072f - 0.072f * v,
                          0.213f - 0.213f * v, 0.715f - 0.715f * v, 0.072f + 0.928f * v};
            for (int i = 0; i < 9; i++) cp.m[i] = m[i];
        } else {
            float angle = values[0] * (float)(3.14159265358979323846 / 180.0);
            float a1 = cosf(angle), a2 = sinf(angle);
            float m[9] = {0.213f + 0.787f * a1 - 0.213f * a2, 0.715f - 0.715f * a1 - 0.715f * a2,
                          0.072f - 0.072f * a1 + 0.928f * a2, 0.213f - 0.213f * a1 + 0.143f * a2,
                          0.715f + 0.285f * a1 + 0.140f * a2, 0.072f - 0.072f * a1 - 0.283f * a2,
                          0.213f - 0.213f * a1 - 0.787f * a2, 0.715f - 0.715f * a1 + 0.715f * a2,
                          0.072f + 0.928f * a1 + 0.072f * a2};
            for (int i = 0; i < 9; i++) cp.m[i] = m[i];
        }
    } else {
        cp.kind = 2;
    }
    if (n == 0) return cudaSuccess;
    cudaError_t te = ensure_luts();
    if (te != cudaSuccess) return te;
    k_color_matrix<<<nblk((n + 3) / 4, 256), 256, 0, s>>>(src, dst, n, cp);
    return cudaGetLastError();
}

// morphology.rs: window columns = min(2*ceil(rx), w), rows likewise, target = floor(n/2)
cudaError_t filter_morphology_to(const uint32_t *src, uint32_t *dst, uint32_t *tmp, int w, int h, bool dilate,
                                 float rx, float ry, cudaStream_t s) {
    int cols = (int)fminf(ceilf(rx) * 2.0f, (float)w), rows = (int)fminf(ceilf(ry) * 2.0f, (float)h);
    int txc = (int)floorf((float)cols / 2.0f), tyr = (int)floorf((float)rows / 2.0f);
    size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    cudaError_t ae = box_attrs();
    if (ae != cudaSuccess) return ae;
    if (cols <= kMorphPairMaxTaps && rows <= kMorphPairMaxTaps) {
        dim3 g((unsigned)((w + kPairTX - 1) / kPairTX), (unsigned)((h + kPairTY - 1) / kPairTY));
        k_morph_vh<<<g, 256, morph_pair_smem(cols, rows), s>>>(src, dst, w, h, cols, rows, txc, tyr, dilate ? 1 : 0);
        return cudaGetLastError();
    }
    // separate passes: rows src -> tmp, columns tmp -> dst
    if (cols <= kMorphMaxTaps) {
        dim3 g((unsigned)((w + kBoxT - 1) / kBoxT), (unsigned)((h + 31) / 32));
        k_morph_h<<<g, 256, morph_h_smem(cols), s>>>(src, tmp, w, h, cols, txc, dilate ? 1 : 0);
    } else {
        k_morph_pass<<<nblk(n, 256), 256, 0, s>>>(src, tmp, w, h, 1, (size_t)w, cols, txc, dilate ? 1 : 0);
    }
    if (rows <= kMorphMaxTaps) {
        dim3 g((unsigned)((w + 31) / 32), (unsigned)((h + kBoxT - 1) / kBoxT));
        k_morph_v<<<g, 256, morph_v_smem(rows), s>>>(tmp, dst, w, h, rows, tyr, dilate ? 1 : 0);
    } else {
        k_morph_pass<<<nblk(n, 256), 256, 0, s>>>(tmp, dst, h, w, (size_t)w, 1, rows, tyr, dilate ? 1 : 0);
    }
    return cudaGetLastError();
}

cudaError_t filter_morphology(uint32_t *img, uint32_t *tmp, int w, int h, bool dilate, float rx, float ry,
                              cudaStream_t s) {
    int cols = (int)fminf(ceilf(rx) * 2.0f, (float)w), rows = (int)fminf(ceilf(ry) * 2.0f, (float)h);
    int txc = (int)floorf((float)cols / 2.0f), tyr = (int)floorf((float)rows / 2.0f);
    size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    cudaError_t ae = box_attrs();
    if (ae != cudaSuccess) return ae;
    if (cols <= kMorphPairMaxTaps && rows <= kMorphPairMaxTaps) {
        // one fused launch into tmp, then back
        dim3 g((unsigned)((w + kPairTX - 1) / kPairTX), (unsigned)((h + kPairTY - 1) / kPairTY));
        k_morph_vh<<<g, 256, morph_pair_smem(cols, rows), s>>>(img, tmp, w, h, cols, rows, txc, tyr, dilate ? 1 : 0);
        cudaError_t ce = cudaMemcpyAsync(img, tmp, n * 4, cudaMemcpyDeviceToDevice, s);
        if (ce != cudaSuccess) return ce;
        return cudaGetLastError();
    }
    if (cols <= kMorphMaxTaps) {
        dim3 g((unsigned)((w + kBoxT - 1) / kBoxT), (unsigned)((h + 31) / 32));
        k_morph_h<<<g, 256, morph_h_smem(cols), s>>>(img, tmp, w, h, cols, txc, dilate ? 1 : 0);
    } else {
        k_morph_pass<<<nblk(n, 256), 256, 0, s>>>(img, tmp, w, h, 1, (size_t)w, cols, txc, dilate ? 1 : 0);
    }
    if (rows <= kMorphMaxTaps) {
        dim3 g((unsigned)((w + 31) / 32), (unsigned)((h + kBoxT - 1) / kBoxT));
        k_morph_v<<<g, 256, morph_v_smem(rows), s>>>(tmp, img, w, h, rows, tyr, dilate ? 1 : 0);
    } else {
        k_morph_pass<<<nblk(n, 256), 256, 0, s>>>(tmp, img, h, w, (size_t)w, 1, rows, tyr, dilate ? 1 : 0);
    }
    return cudaGetLastError();
}

cudaError_t filter_arithmetic(const uint32_t *a, const uint32_t *b, uint32_t *dst, size_t n, const float k[4],
                              cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess) return e;
    k_arithmetic<<<nblk_capped((n + 3) / 4, 256), 256, 0, s>>>(a, b, dst, n, k[0], k[1], k[2], k[3]);
    return cudaGetLastError();
}

cudaError_t filter_copy(const uint32_t *src, uint32_t *dst, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToDevice, s);
}

}  // namespace rgpu

// ---- elementwise helpers for the remaining primitives
#include "pipeline.cuh"
namespace rgpu {
namespace {
__global__ void k_crop(uint32_t *img, int w, int h, int l, int t, int r, int b) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)w * h) return;
    int x = (int)(i % w), y = (int)(i / w);
    if (x < l || x >= r || y < t || y >= b) img[i] = 0;
}
// draw_pixmap(dx, dy, src) onto dst with a blend mode (highp, Nearest, opacity
// 1): src is sw x sh, dst dw x dh; only the overlap is drawn
__global__ void k_draw(const uint32_t *src, int sw, int sh, uint32_t *dst, int dw, int dh, int dx, int dy,
                       uint32_t blend) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)dw * dh) return;
    int x = (int)(i % dw), y = (int)(i / dw);
    int64_t sx = (int64_t)x - dx, sy = (int64_t)y - dy;
    if (sx < 0 || sy < 0 || sx >= sw || sy >= sh) return;
    dst[i] = dev::composite_pixel(src[(size_t)sy * sw + (size_t)sx], dst[i], 1.0f, blend);
}
__global__ void k_fill(uint32_t *img, size_t n, uint32_t v) {
    auto f = [v](uint32_t) { return v; };
    RGPU_MAP4(img, n, f);
}
}  // namespace

cudaError_t filter_crop(uint32_t *img, int w, int h, int l, int t, int r, int b, cudaStream_t s) {
    size_t n = (size_t)w * h;
    if (!n) return cudaSuccess;
    k_crop<<<nblk(n, 256), 256, 0, s>>>(img, w, h, l, t, r, b);
    return cudaGetLastError();
}
cudaError_t filter_draw(const uint32_t *src, int sw, int sh, uint32_t *dst, int dw, int dh, int dx, int dy,
                        uint32_t blend, cudaStream_t s) {
    size_t n = (size_t)dw * dh;
    if (!n || sw <= 0 || sh <= 0) return cudaSuccess;
    k_draw<<<nblk(n, 256), 256, 0, s>>>(src, sw, sh, dst, dw, dh, dx, dy, blend);
    return cudaGetLastError();
}
cudaError_t filter_fill(uint32_t *img, size_t n, uint32_t v, cudaStream_t s) {
    if (!n) return cudaSuccess;
    if ((v & 0xFFu) * 0x01010101u == v) return cudaMemsetAsync(img, (int)(v & 0xFFu), n * 4, s);
    k_fill<<<nblk((n + 3) / 4, 256), 256, 0, s>>>(img, n, v);
    return cudaGetLastError();
}
}  // namespace rgpu

namespace rgpu {
namespace {
__global__ void k_alpha_only(uint32_t *img, size_t n) {
    auto f = [](uint32_t p) { return p & 0xFF000000u; };
    RGPU_MAP4(img, n, f);
}
}  // namespace
cudaError_t filter_alpha_only(uint32_t *img, size_t n, cudaStream_t s) {
    if (!n) return cudaSuccess;
    k_alpha_only<<<nblk((n + 3) / 4, 256), 256, 0, s>>>(img, n);
    return cudaGetLastError();
}
namespace {

constexpr int kConvRows = 8;  // output rows per thread
__global__ void k_convolve(const uint32_t *src, uint32_t *dst, int w, int h, ConvolveParams cp) {
    __shared__ float u[256];
    __shared__ float kf[sizeof(cp.k) / sizeof(float)];  // the kernel, flipped: kf[oy * cols + ox]
    load_unit(u);
    for (int k = threadIdx.x; k < cp.rows * cp.cols; k += blockDim.x) kf[k] = cp.k[cp.rows * cp.cols - 1 - k];
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const bool pres = cp.preserve_alpha != 0;
    for (int y = blockIdx.y * kConvRows; y < min(h, (int)(blockIdx.y + 1) * kConvRows); y++) {
    float nr = 0.0f, ng = 0.0f, nb = 0.0f, na = 0.0f;
    for (int oy = 0; oy < cp.rows; oy++)
        for (int ox = 0; ox < cp.cols; ox++) {
            int tx = x - cp.tx + ox, ty = y - cp.ty + oy;
            if (cp.edge == RGPU_EDGE_NONE) {
                if (tx < 0 || tx >= w || ty < 0 || ty >= h) continue;
            } else if (cp.edge == RGPU_EDGE_DUPLICATE) {
                tx = min(max(tx, 0), w - 1);
                ty = min(max(ty, 0), h - 1);
            } else {
                tx = ((tx % w) + w) % w;
                ty = ((ty % h) + h) % h;
            }
            const float kv = kf[oy * cp.cols + ox];
            uint32_t p = src[(size_t)ty * w + tx];
            if (pres) p = demul(p);
            nr += u[chn(p, 0)] * kv;
            ng += u[chn(p, 1)] * kv;
            nb += u[chn(p, 2)] * kv;
            if (!pres) na += u[chn(p, 3)] * kv;
        }
    if (pres) na = u[chn(src[(size_t)y * w + x], 3)];
    else na = __fdiv_rn(na, cp.divisor) + cp.bias;
    const float bna = f32_bound(0.0f, na, 1.0f);
    auto calc = [&](float v) {
        float q = __fdiv_rn(v, cp.divisor) + cp.bias * na;
        q = pres ? f32_bound(0.0f, q, 1.0f) * bna : f32_bound(0.0f, q, bna);
        return sat_u8f(q * 255.0f + 0.5f);
    };
    dst[(size_t)y * w + x] = pk(calc(nr), calc(ng), calc(nb), sat_u8f(bna * 255.0f + 0.5f));
    }
}

// ApproxEqUlps(4) of two f32s, as in float-cmp
__device__ __forceinline__ bool ulps_eq4(float a, float b) {
    const int32_t ia = __float_as_int(a), ib = __float_as_int(b);
    if ((ia < 0) != (ib < 0)) return a == b;
    return abs(ia - ib) <= 4;
}

__global__ void k_lighting(const uint32_t *src, uint32_t *dst, int w, int h, LightingParams lp) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    auto A = [&](int xx, int yy) -> int { return (int)chn(src[(size_t)yy * w + xx], 3); };
    // surface normal: interior Sobel, or the edge / corner variant
    const bool l = x == 0, r = x == w - 1, t = y == 0, b = y == h - 1;
    float fx, fy;
    int nx, ny;
    if ((l || r) && (t || b)) {
        // corners: the 2x2 neighbourhood towards the inside
        const int xi = l ? 1 : w - 2, yi = t ? 1 : h - 2;
        const int sxn = l ? 1 : -1, syn = t ? 1 : -1;  // direction of the inner neighbour
        const int c = A(x, y), hx = A(xi, y), vy = A(x, yi), d = A(xi, yi);
        fx = fy = 2.0f / 3.0f;
        // d/dx ~ (2 (right - left) + (lower-right - lower-left)) in the 2x2 block
        nx = sxn * (2 * hx - 2 * c + d - vy);
        ny = syn * (2 * vy - 2 * c + d - hx);
    } else if (t || b) {
        const int yi = t ? 1 : h - 2, syn = t ? 1 : -1;
        const int lf = A(x - 1, y), c = A(x, y), rt = A(x + 1, y);
        const int il = A(x - 1, yi), ic = A(x, yi), ir = A(x + 1, yi);
        fx = 1.0f / 3.0f; fy = 1.0f / 2.0f;
        nx = -2 * lf + 2 * rt - il + ir;
        ny = syn * (-lf - 2 * c - rt + il + 2 * ic + ir);
    } else if (l || r) {
        const int xi = l ? 1 : w - 2, sxn = l ? 1 : -1;
        const int tp = A(x, y - 1), c = A(x, y), bt = A(x, y + 1);
        const int it = A(xi, y - 1), ic = A(xi, y), ib = A(xi, y + 1);
        fx = 1.0f / 2.0f; fy = 1.0f / 3.0f;
        nx = sxn * (-tp + it - 2 * c + 2 * ic - bt + ib);
        ny = -2 * tp - it + 2 * bt + ib;
    } else {
        const int tl = A(x - 1, y - 1), tp = A(x, y - 1), tr = A(x + 1, y - 1), lf = A(x - 1, y), rt = A(x + 1, y),
                  bl = A(x - 1, y + 1), bt = A(x, y + 1), br = A(x + 1, y + 1);
        fx = fy = 1.0f / 4.0f;
        nx = -tl + tr - 2 * lf + 2 * rt - bl + br;
        ny = -tl - 2 * tp - tr + bl + 2 * bt + br;
    }
    float lx = lp.lv[0], ly = lp.lv[1], lz = lp.lv[2];
    if (lp.kind != RGPU_LIGHT_DISTANT) {
        const float nz = __fdiv_rn((float)A(x, y), 255.0f) * lp.surface_scale;
        const float vx = lp.pos[0] - (float)x, vy = lp.pos[1] - (float)y, vz = lp.pos[2] - nz;
        const float len = __fsqrt_rn(vx * vx + vy * vy + vz * vz);
        if (ulps_eq4(len, 0.0f)) { lx = vx; ly = vy; lz = vz; }
        else { lx = __fdiv_rn(vx, len); ly = __fdiv_rn(vy, len); lz = __fdiv_rn(vz, len); }
    }
    uint32_t col[3] = {lp.color[0], lp.color[1], lp.color[2]};
    if (lp.kind == RGPU_LIGHT_SPOT) {
        const float mls = -(lx * lp.dir[0] + ly * lp.dir[1] + lz * lp.dir[2]);
        if (mls <= 0.0f || (lp.has_cone && mls < lp.cone_cos)) {
            col[0] = col[1] = col[2] = 0;
        } else {
            const float fac = powf(mls, lp.spot_exponent);
#pragma unroll
            for (int k = 0; k < 3; k++) col[k] = (uint32_t)(uint8_t)(f32_bound(0.0f, (float)lp.color[k] * fac, 255.0f) + 0.5f);
        }
    }
    const float nxv = (float)(int16_t)(-nx), nyv = (float)(int16_t)(-ny);
    const bool flat = ulps_eq4(nxv, 0.0f) && ulps_eq4(nyv, 0.0f);
    const float sc = __fdiv_rn(lp.surface_scale, 255.0f);
    float factor;
    if (!lp.specular) {
        float k;
        if (flat) k = lz;
        else {
            const float mx = nxv * sc * fx, my = nyv * sc * fy;
            k = __fdiv_rn(mx * lx + my * ly + 1.0f * lz, __fsqrt_rn(mx * mx + my * my + 1.0f * 1.0f));
        }
        factor = lp.constant * k;
    } else {
        const float hx = lx + 0.0f, hy = ly + 0.0f, hz = lz + 1.0f;
        const float hl = __fsqrt_rn(hx * hx + hy * hy + hz * hz);
        if (ulps_eq4(hl, 0.0f)) factor = 0.0f;
        else {
            float ndh;
            if (flat) ndh = __fdiv_rn(hz, hl);
            else {
                const float mx = nxv * sc * fx, my = nyv * sc * fy;
                ndh = __fdiv_rn(__fdiv_rn(mx * hx + my * hy + 1.0f * hz, __fsqrt_rn(mx * mx + my * my + 1.0f * 1.0f)), hl);
            }
            const float k = ulps_eq4(lp.exponent, 1.0f) ? ndh : powf(ndh, lp.exponent);
            factor = lp.constant * k;
        }
    }
    uint32_t o[3];
#pragma unroll
    for (int k = 0; k < 3; k++) o[k] = (uint32_t)(uint8_t)(f32_bound(0.0f, (float)col[k] * factor, 255.0f) + 0.5f);
    const uint32_t a = lp.specular ? max(max(o[0], o[1]), o[2]) : 255u;
    dst[(size_t)y * w + x] = pk(o[0], o[1], o[2], a);
}

}  // namespace

cudaError_t filter_convolve(const uint32_t *src, uint32_t *dst, int w, int h, const ConvolveParams &cp,
                            cudaStream_t s) {
    if (w <= 0 || h <= 0) return cudaSuccess;
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess) return e;
    k_convolve<<<dim3((unsigned)((w + 127) / 128), (unsigned)((h + kConvRows - 1) / kConvRows)), 128, 0, s>>>(
        src, dst, w, h, cp);
    return cudaGetLastError();
}

cudaError_t filter_lighting(const uint32_t *src, uint32_t *dst, int w, int h, const LightingParams &lp,
                            cudaStream_t s) {
    if (w < 3 || h < 3) return cudaMemsetAsync(dst, 0, (size_t)(w > 0 ? w : 0) * (h > 0 ? h : 0) * 4, s);
    k_lighting<<<dim3((unsigned)((w + 127) / 128), (unsigned)h), 128, 0, s>>>(src, dst, w, h, lp);
    return cudaGetLastError();
}

}  // namespace rgpu

namespace rgpu {
namespace {

// ---- component transfer (component_transfer.rs): demultiply, the four
// channel functions as one 256-entry table of packed (r, g, b, a) results,
// multiply.  The table sits in shared memory; each thread maps four pixels.
struct Lut256 { uint32_t v[256]; };
__global__ void k_component_transfer(uint32_t *img, size_t n, Lut256 lut) {
    __shared__ uint32_t s_lut[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) s_lut[k] = lut.v[k];
    __syncthreads();
    auto f = [](uint32_t px) {
        const uint32_t p = tab_px(TAB_DEMUL, px);
        const uint32_t o = (s_lut[chn(p, 0)] & 0xFFu) | (s_lut[chn(p, 1)] & 0xFF00u) |
                           (s_lut[chn(p, 2)] & 0xFF0000u) | (s_lut[chn(p, 3)] & 0xFF000000u);
        return tab_px(TAB_MUL, o);
    };
    RGPU_MAP4(img, n, f);
}

// ---- drop shadow (mod.rs:581-649), after the shadow copy is blurred: the
// flooded, colour-space converted shadow is a function of the blurred alpha
// alone (a 256-entry table); it is drawn at (dx, dy) onto a transparent
// image, then the input is drawn over it, both source-over.
__global__ void k_drop_shadow(const uint32_t *in, const uint32_t *shadow, uint32_t *out, int w, int h, int dx,
                              int dy, Lut256 lut) {
    __shared__ uint32_t s_lut[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) s_lut[k] = lut.v[k];
    __syncthreads();
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)w * h) return;
    const int x = (int)(i % w), y = (int)(i / w);
    const int64_t sx = (int64_t)x - dx, sy = (int64_t)y - dy;
    uint32_t d = 0;
    if (sx >= 0 && sy >= 0 && sx < w && sy < h)
        d = dev::composite_pixel(s_lut[shadow[(size_t)sy * w + (size_t)sx] >> 24], 0u, 1.0f, RGPU_BLEND_SOURCE_OVER);
    out[i] = dev::composite_pixel(in[i], d, 1.0f, RGPU_BLEND_SOURCE_OVER);
}

}  // namespace

cudaError_t filter_component_transfer(uint32_t *img, size_t n, const uint32_t lut[256], cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess) return e;
    Lut256 l;
    for (int k = 0; k < 256; k++) l.v[k] = lut[k];
    k_component_transfer<<<nblk((n + 3) / 4, 256), 256, 0, s>>>(img, n, l);
    return cudaGetLastError();
}

cudaError_t filter_drop_shadow(const uint32_t *in, const uint32_t *shadow, uint32_t *out, int w, int h, int dx,
                               int dy, uint32_t flood, bool linear, cudaStream_t s) {
    const size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess) return e;
    // Color::from_rgba8(r, g, b, opacity.to_u8()); apply_opacity(alpha / 255) clamps
    // the product; premultiply (skipped when opaque) clamps each channel;
    // to_color_u8 rounds v * 255 + 0.5 down.  Then into_srgb / into_linear_rgb.
    auto clamp01 = [](float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); };
    const float cr = (float)(flood & 0xFFu) / 255.0f, cg = (float)((flood >> 8) & 0xFFu) / 255.0f,
                cb = (float)((flood >> 16) & 0xFFu) / 255.0f, ca = (float)(flood >> 24) / 255.0f;
    const int t = linear ? TAB_TO_LINEAR : TAB_TO_SRGB;
    Lut256 l;
    for (uint32_t sa = 0; sa < 256; sa++) {
        const float a = clamp01(ca * clamp01((float)sa / 255.0f));
        float r = cr, g = cg, b = cb;
        if (a != 1.0f) { r = clamp01(r * a); g = clamp01(g * a); b = clamp01(b * a); }
        const uint32_t pa = host_sat_u8(a * 255.0f + 0.5f);
        const uint32_t pr = host_sat_u8(r * 255.0f + 0.5f), pg = host_sat_u8(g * 255.0f + 0.5f),
                       pb = host_sat_u8(b * 255.0f + 0.5f);
        l.v[sa] = (uint32_t)g_host_tab[t][(pa << 8) | pr] | ((uint32_t)g_host_tab[t][(pa << 8) | pg] << 8) |
                  ((uint32_t)g_host_tab[t][(pa << 8) | pb] << 16) | (pa << 24);
    }
    k_drop_shadow<<<nblk(n, 256), 256, 0, s>>>(in, shadow, out, w, h, dx, dy, l);
    return cudaGetLastError();
}
}  // namespace rgpu

namespace rgpu {
namespace {

// ---- turbulence (turbulence.rs): the SVG 1.1 Perlin noise in f64.  Each CTA
// rebuilds the lattice and gradient tables in shared memory: the generator is
// Park-Miller, seed_n = 16807^n * seed_0 mod (2^31 - 1), so every draw is
// computed independently; only the 255 swaps of the lattice shuffle are
// sequential (one thread, shared memory).
constexpr uint32_t kTurbM = 2147483647u, kTurbA = 16807u;
constexpr int kTurbB = 256, kTurbBLen = 514, kTurbPerlinN = 4096;

__device__ __forceinline__ uint32_t mulmod_m(uint32_t a, uint32_t b) {
    const uint64_t p = (uint64_t)a * b;
    uint64_t r = (p & kTurbM) + (p >> 31);
    if (r >= kTurbM) r -= kTurbM;
    return (uint32_t)r;
}
__device__ uint32_t powmod_a(uint32_t e) {
    uint32_t r = 1u, b = kTurbA;
    while (e) {
        if (e & 1u) r = mulmod_m(r, b);
        b = mulmod_m(b, b);
        e >>= 1;
    }
    return r;
}
__device__ __forceinline__ int32_t sat_i32_d(double v) { return __double2int_rz(v); }
__device__ __forceinline__ int64_t sat_i64_d(double v) { return __double2ll_rz(v); }

struct TurbStitch { int32_t width, height, wrap_x, wrap_y; };

__device__ __forceinline__ double turb_noise2(int ch, double x, double y, const int32_t *sel, const double2 *grad,
                                              bool stitch, const TurbStitch &st) {
    double t = __dadd_rn(x, (double)kTurbPerlinN);
    int32_t bx0 = sat_i32_d(t), bx1 = (int32_t)((uint32_t)bx0 + 1u);
    const double rx0 = __dsub_rn(t, (double)sat_i64_d(t)), rx1 = __dsub_rn(rx0, 1.0);
    t = __dadd_rn(y, (double)kTurbPerlinN);
    int32_t by0 = sat_i32_d(t), by1 = (int32_t)((uint32_t)by0 + 1u);
    const double ry0 = __dsub_rn(t, (double)sat_i64_d(t)), ry1 = __dsub_rn(ry0, 1.0);
    if (stitch) {
        if (bx0 >= st.wrap_x) bx0 = (int32_t)((uint32_t)bx0 - (uint32_t)st.width);
        if (bx1 >= st.wrap_x) bx1 = (int32_t)((uint32_t)bx1 - (uint32_t)st.width);
        if (by0 >= st.wrap_y) by0 = (int32_t)((uint32_t)by0 - (uint32_t)st.height);
        if (by1 >= st.wrap_y) by1 = (int32_t)((uint32_t)by1 - (uint32_t)st.height);
    }
    bx0 &= 0xff; bx1 &= 0xff; by0 &= 0xff; by1 &= 0xff;
    const int32_t i = sel[bx0], j = sel[bx1];
    const double2 *g = grad + ch * kTurbBLen;
    const double sx = __dmul_rn(__dmul_rn(rx0, rx0), __dsub_rn(3.0, __dmul_rn(2.0, rx0)));
    const double sy = __dmul_rn(__dmul_rn(ry0, ry0), __dsub_rn(3.0, __dmul_rn(2.0, ry0)));
    double2 q = g[sel[i + by0]];
    double u = __dadd_rn(__dmul_rn(rx0, q.x), __dmul_rn(ry0, q.y));
    q = g[sel[j + by0]];
    double v = __dadd_rn(__dmul_rn(rx1, q.x), __dmul_rn(ry0, q.y));
    const double a = __dadd_rn(u, __dmul_rn(sx, __dsub_rn(v, u)));
    q = g[sel[i + by1]];
    u = __dadd_rn(__dmul_rn(rx0, q.x), __dmul_rn(ry1, q.y));
    q = g[sel[j + by1]];
    v = __dadd_rn(__dmul_rn(rx1, q.x), __dmul_rn(ry1, q.y));
    const double b = __dadd_rn(u, __dmul_rn(sx, __dsub_rn(v, u)));
    return __dadd_rn(a, __dmul_rn(sy, __dsub_rn(b, a)));
}

__device__ __forceinline__ bool approx_zero_ulps_d(double v) {
    const long long a = __double_as_longlong(v);
    if (a < 0) return v == 0.0;
    return a <= 4;
}

__global__ void __launch_bounds__(256) k_turbulence(uint32_t *out, int w, int h, TurbParams tp) {
    __shared__ int32_t sel[kTurbBLen];
    __shared__ double2 grad[4 * kTurbBLen];
    __shared__ int32_t swap_j[kTurbB];
    const int t = threadIdx.x;
    // tables (turbulence.rs init): draw n (1-based) is seed_0 * A^n mod M
    {
        const uint32_t base = mulmod_m(tp.seed0, powmod_a(2u * (uint32_t)t + 1u));
        for (int k = 0; k < 4; k++) {
            const uint32_t s0 = k == 0 ? base : mulmod_m(base, powmod_a(512u * (uint32_t)k));
            const uint32_t s1 = mulmod_m(s0, kTurbA);
            double g0 = (double)((int32_t)(s0 % 512u) - kTurbB) / (double)kTurbB;
            double g1 = (double)((int32_t)(s1 % 512u) - kTurbB) / (double)kTurbB;
            const double s = __dsqrt_rn(__dadd_rn(__dmul_rn(g0, g0), __dmul_rn(g1, g1)));
            grad[k * kTurbBLen + t] = make_double2(__ddiv_rn(g0, s), __ddiv_rn(g1, s));
        }
        sel[t] = t;
        // the shuffle step for lattice index i = 255 .. 1 uses draw 2048 + (256 - i)
        if (t >= 1) swap_j[t] = (int32_t)(mulmod_m(tp.seed0, powmod_a(2048u + 256u - (uint32_t)t)) % 256u);
    }
    __syncthreads();
    if (t == 0) {
        for (int i = kTurbB - 1; i >= 1; i--) {
            const int32_t k = sel[i], j = swap_j[i];
            sel[i] = sel[j];
            sel[j] = k;
        }
    }
    __syncthreads();
    for (int i = t; i < kTurbB + 2; i += blockDim.x) {
        sel[kTurbB + i] = sel[i % kTurbB];
        for (int k = 0; k < 4; k++) grad[k * kTurbBLen + kTurbB + i] = grad[k * kTurbBLen + (i % kTurbB)];
    }
    __syncthreads();

    const size_t n = (size_t)w * h;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + t; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(idx % w), y = (int)(idx / w);
        uint32_t px = 0;
        for (int ch = 0; ch < 4; ch++) {
            double bfx = tp.bfx, bfy = tp.bfy;
            TurbStitch st{0, 0, 0, 0};
            const double tile_w = (double)w, tile_h = (double)h;
            if (tp.stitch) {
                if (!approx_zero_ulps_d(bfx)) {
                    const double lo = __ddiv_rn(floor(__dmul_rn(tile_w, bfx)), tile_w);
                    const double hi = __ddiv_rn(ceil(__dmul_rn(tile_w, bfx)), tile_w);
                    bfx = __ddiv_rn(bfx, lo) < __ddiv_rn(hi, bfx) ? lo : hi;
                }
                if (!approx_zero_ulps_d(bfy)) {
                    const double lo = __ddiv_rn(floor(__dmul_rn(tile_h, bfy)), tile_h);
                    const double hi = __ddiv_rn(ceil(__dmul_rn(tile_h, bfy)), tile_h);
                    bfy = __ddiv_rn(bfy, lo) < __ddiv_rn(hi, bfy) ? lo : hi;
                }
                st.width = sat_i32_d(__dadd_rn(__dmul_rn(tile_w, bfx), 0.5));
                st.height = sat_i32_d(__dadd_rn(__dmul_rn(tile_h, bfy), 0.5));
                st.wrap_x = sat_i32_d(__dadd_rn(__dadd_rn(__dmul_rn((double)x, bfx), (double)kTurbPerlinN),
                                                (double)st.width));
                st.wrap_y = sat_i32_d(__dadd_rn(__dadd_rn(__dmul_rn((double)y, bfy), (double)kTurbPerlinN),
                                                (double)st.height));
            }
            double vx = __dmul_rn(__ddiv_rn(__dadd_rn((double)x, tp.ox), tp.sx), bfx);
            double vy = __dmul_rn(__ddiv_rn(__dadd_rn((double)y, tp.oy), tp.sy), bfy);
            double sum = 0.0, ratio = 1.0;
            for (int o = 0; o < tp.octaves; o++) {
                const double nz = turb_noise2(ch, vx, vy, sel, grad, tp.stitch != 0, st);
                sum = __dadd_rn(sum, __ddiv_rn(tp.fractal ? nz : fabs(nz), ratio));
                vx = __dmul_rn(vx, 2.0);
                vy = __dmul_rn(vy, 2.0);
                ratio = __dmul_rn(ratio, 2.0);
                if (tp.stitch) {
                    st.width = (int32_t)((uint32_t)st.width * 2u);
                    st.wrap_x = (int32_t)((uint32_t)st.wrap_x * 2u - (uint32_t)kTurbPerlinN);
                    st.height = (int32_t)((uint32_t)st.height * 2u);
                    st.wrap_y = (int32_t)((uint32_t)st.wrap_y * 2u - (uint32_t)kTurbPerlinN);
                }
            }
            const double v = tp.fractal ? __ddiv_rn(__dadd_rn(__dmul_rn(sum, 255.0), 255.0), 2.0) : __dmul_rn(sum, 255.0);
            px |= sat_u8f(f32_bound(0.0f, __double2float_rn(v), 255.0f) + 0.5f) << (8 * ch);
        }
        out[idx] = tab_px(TAB_MUL, px);
    }
}

}  // namespace

cudaError_t filter_turbulence(uint32_t *out, int w, int h, const TurbParams &tp, cudaStream_t s) {
    const size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    cudaError_t e = ensure_luts();
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t want = (n + 255) / 256;
    const uint32_t grid = (uint32_t)std::min<size_t>(want, (size_t)std::max(sms, 1) * 4);
    k_turbulence<<<grid, 256, 0, s>>>(out, w, h, tp);
    return cudaGetLastError();
}
}  // namespace rgpu

namespace rgpu {
namespace {
// feTile: out(x, y) = src(l + (x - ox) mod tw, t + (y - oy) mod th), the tile
// being the input's region cut at (l, t, tw, th) of the sw-wide source and
// repeated from (ox, oy) over the w x h output.
__global__ void k_tile(const uint32_t *src, int sw, uint32_t *dst, int w, int h, int ox, int oy, int l, int t, int tw,
                       int th) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)w * h) return;
    const int x = (int)(i % w), y = (int)(i / w);
    int u = (int)(((int64_t)x - ox) % tw), v = (int)(((int64_t)y - oy) % th);
    if (u < 0) u += tw;
    if (v < 0) v += th;
    dst[i] = src[(size_t)(t + v) * sw + (size_t)(l + u)];
}
// feDisplacementMap (displacement_map.rs): each pixel takes the source pixel
// at its position moved by (map channel / 255 - 0.5) * scale * s, rounded half
// away from zero; 0 outside.
__global__ void k_displace(const uint32_t *src, const uint32_t *map, uint32_t *dst, int w, int h, float sx, float sy,
                           float scale, int xch, int ych) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)w * h) return;
    const int x = (int)(i % w), y = (int)(i / w);
    const uint32_t m = map[i];
    const float dx = __fsub_rn(__fdiv_rn((float)chn(m, xch), 255.0f), 0.5f);
    const float dy = __fsub_rn(__fdiv_rn((float)chn(m, ych), 255.0f), 0.5f);
    const float fx = __fadd_rn((float)x, __fmul_rn(__fmul_rn(dx, sx), scale));
    const float fy = __fadd_rn((float)y, __fmul_rn(__fmul_rn(dy, sy), scale));
    const int ox = __float2int_rz(roundf(fx)), oy = __float2int_rz(roundf(fy));
    dst[i] = (ox >= 0 && ox < w && oy >= 0 && oy < h) ? src[(size_t)oy * w + ox] : 0u;
}
}  // namespace

cudaError_t filter_tile(const uint32_t *src, int sw, int sh, uint32_t *dst, int w, int h, int ox, int oy, int l,
                        int t, int tw, int th, cudaStream_t s) {
    const size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    if (tw <= 0 || th <= 0 || l < 0 || t < 0 || l + tw > sw || t + th > sh) return cudaErrorInvalidValue;
    k_tile<<<nblk(n, 256), 256, 0, s>>>(src, sw, dst, w, h, ox, oy, l, t, tw, th);
    return cudaGetLastError();
}
cudaError_t filter_displacement_map(const uint32_t *src, const uint32_t *map, uint32_t *dst, int w, int h, float sx,
                                    float sy, float scale, int xch, int ych, cudaStream_t s) {
    const size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    k_displace<<<nblk(n, 256), 256, 0, s>>>(src, map, dst, w, h, sx, sy, scale, xch & 3, ych & 3);
    return cudaGetLastError();
}
}  // namespace rgpu

namespace rgpu {
namespace {
// ---- the Pattern shader (tiny-skia shaders/pattern.rs, highp stages; raster
// images use it padded, image.rs:167-201): the
// same f32 operations in the same order as the CPU restatement, no contraction.
struct PatternParams {
    float sx, ky, kx, sy, tx, ty;
    int tw, th, bx, by, bw, bh, quality, repeat;
    float opacity;
};
__device__ __forceinline__ float ulp_below_f(float v) { return __int_as_float(__float_as_int(v) - 1); }
__device__ __forceinline__ float4 pattern_gather(const uint32_t *tile, const PatternParams &pp, float x, float y) {
    const float w = (float)pp.tw, h = (float)pp.th;
    if (pp.repeat) {
        x = __fsub_rn(x, __fmul_rn(floorf(__fmul_rn(x, __fdiv_rn(1.0f, w))), w));
        y = __fsub_rn(y, __fmul_rn(floorf(__fmul_rn(y, __fdiv_rn(1.0f, h))), h));
    }
    x = fminf(fmaxf(x, 0.0f), ulp_below_f(w));
    y = fminf(fmaxf(y, 0.0f), ulp_below_f(h));
    const uint32_t p = __ldg(tile + (size_t)(uint32_t)y * (uint32_t)pp.tw + (uint32_t)x);
    const float k = __fdiv_rn(1.0f, 255.0f);
    return make_float4(__fmul_rn((float)(p & 0xFFu), k), __fmul_rn((float)((p >> 8) & 0xFFu), k),
                       __fmul_rn((float)((p >> 16) & 0xFFu), k), __fmul_rn((float)(p >> 24), k));
}
__device__ __forceinline__ float bicubic_near_f(float t) {
    return __fadd_rn(__fmul_rn(t, __fadd_rn(__fmul_rn(t, __fadd_rn(__fmul_rn(-21.0f / 18.0f, t), 27.0f / 18.0f)),
                                            9.0f / 18.0f)),
                     1.0f / 18.0f);
}
__device__ __forceinline__ float bicubic_far_f(float t) {
    return __fmul_rn(__fmul_rn(t, t), __fadd_rn(__fmul_rn(7.0f / 18.0f, t), -6.0f / 18.0f));
}
__global__ void k_pattern_shade(const uint32_t *tile, float4 *out, PatternParams pp) {
    const size_t n = (size_t)pp.bw * pp.bh;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int x = pp.bx + (int)(i % pp.bw), y = pp.by + (int)(i / pp.bw);
        const float px = __fadd_rn((float)x, 0.5f), py = __fadd_rn((float)y, 0.5f);
        const float u = __fadd_rn(__fmul_rn(px, pp.sx), __fadd_rn(__fmul_rn(py, pp.kx), pp.tx));
        const float v = __fadd_rn(__fmul_rn(px, pp.ky), __fadd_rn(__fmul_rn(py, pp.sy), pp.ty));
        float4 o;
        if (pp.quality == 0) {
            o = pattern_gather(tile, pp, u, v);
        } else if (pp.quality == 1) {
            const float fx = __fsub_rn(__fadd_rn(u, 0.5f), floorf(__fadd_rn(u, 0.5f)));
            const float fy = __fsub_rn(__fadd_rn(v, 0.5f), floorf(__fadd_rn(v, 0.5f)));
            const float wx[2] = {__fsub_rn(1.0f, fx), fx}, wy[2] = {__fsub_rn(1.0f, fy), fy};
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            float sy = __fsub_rn(v, 0.5f);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                float sx = __fsub_rn(u, 0.5f);
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    const float4 c = pattern_gather(tile, pp, sx, sy);
                    const float wgt = __fmul_rn(wx[k], wy[j]);
                    acc.x = __fadd_rn(__fmul_rn(wgt, c.x), acc.x);
                    acc.y = __fadd_rn(__fmul_rn(wgt, c.y), acc.y);
                    acc.z = __fadd_rn(__fmul_rn(wgt, c.z), acc.z);
                    acc.w = __fadd_rn(__fmul_rn(wgt, c.w), acc.w);
                    sx = __fadd_rn(sx, 1.0f);
                }
                sy = __fadd_rn(sy, 1.0f);
            }
            o = acc;
        } else {
            const float fx = __fsub_rn(__fadd_rn(u, 0.5f), floorf(__fadd_rn(u, 0.5f)));
            const float fy = __fsub_rn(__fadd_rn(v, 0.5f), floorf(__fadd_rn(v, 0.5f)));
            const float wx[4] = {bicubic_far_f(__fsub_rn(1.0f, fx)), bicubic_near_f(__fsub_rn(1.0f, fx)),
                                 bicubic_near_f(fx), bicubic_far_f(fx)};
            const float wy[4] = {bicubic_far_f(__fsub_rn(1.0f, fy)), bicubic_near_f(__fsub_rn(1.0f, fy)),
                                 bicubic_near_f(fy), bicubic_far_f(fy)};
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            float sy = __fsub_rn(v, 1.5f);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                float sx = __fsub_rn(u, 1.5f);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float4 c = pattern_gather(tile, pp, sx, sy);
                    const float wgt = __fmul_rn(wx[k], wy[j]);
                    acc.x = __fadd_rn(__fmul_rn(wgt, c.x), acc.x);
                    acc.y = __fadd_rn(__fmul_rn(wgt, c.y), acc.y);
                    acc.z = __fadd_rn(__fmul_rn(wgt, c.z), acc.z);
                    acc.w = __fadd_rn(__fmul_rn(wgt, c.w), acc.w);
                    sx = __fadd_rn(sx, 1.0f);
                }
                sy = __fadd_rn(sy, 1.0f);
            }
            acc.x = fmaxf(acc.x, 0.0f); acc.y = fmaxf(acc.y, 0.0f); acc.z = fmaxf(acc.z, 0.0f); acc.w = fmaxf(acc.w, 0.0f);
            acc.x = fminf(acc.x, acc.w); acc.y = fminf(acc.y, acc.w); acc.z = fminf(acc.z, acc.w);
            o = acc;
        }
        if (pp.opacity != 1.0f)
            o = make_float4(__fmul_rn(o.x, pp.opacity), __fmul_rn(o.y, pp.opacity), __fmul_rn(o.z, pp.opacity),
                            __fmul_rn(o.w, pp.opacity));
        out[i] = o;
    }
}
}  // namespace

cudaError_t filter_pattern_shade(const uint32_t *tile, int tw, int th, float *out, int bx, int by, int bw, int bh,
                                 const float inv[6], int quality, bool repeat, float opacity, cudaStream_t s) {
    const size_t n = (size_t)bw * bh;
    if (n == 0 || tw <= 0 || th <= 0) return cudaSuccess;
    PatternParams pp{inv[0], inv[1], inv[2], inv[3], inv[4], inv[5], tw, th, bx, by, bw, bh, quality,
                     repeat ? 1 : 0, opacity};
    k_pattern_shade<<<nblk_capped(n, 256), 256, 0, s>>>(tile, reinterpret_cast<float4 *>(out), pp);
    return cudaGetLastError();
}
}  // namespace rgpu
