// Differentiable soft-coverage renderer: a forward pass and a hand-written
// adjoint for batches of scenes of closed cubic paths (no counterpart in the
// reference; resvg renders hard-edged, non-differentiable coverage).
//
// Forward, per scene (premultiplied RGBA in FP32):
//   * a path of n cubics is closed by construction: its 3n points are the
//     start S, then (control 1, control 2, end) per cubic, where the last
//     cubic ends at S; every cubic is flattened into kFlat lines at uniform t
//     (vertex list: P_c(i/kFlat), i = 0..kFlat-1, for each cubic c; the line
//     from the last vertex back to the first closes the loop);
//   * soft coverage of pixel (px, py) by a path is c = min(|A|, 1), where A is
//     the winding-weighted area of the pixel: for every line, the integral over
//     y in [py, py+1] of the part of the pixel row right of the line, signed by
//     the line's y direction; for a line clipped to the row, from (xl, yl) to
//     (xh, yh) with sdy = +-(yh - yl), the pixel gets sdy * G(xl - px, xh - px)
//     with G(a, b) the mean of clamp(1 - x, 0, 1) over x from a to b, written
//     in closed, well-conditioned form per case;
//   * paints (at pixel centres): a straight RGBA colour or a linear gradient of
//     4 stops (pad spread, offsets ascending), its alpha multiplied by the
//     path's opacity, premultiplied after interpolation; paths composite
//     source-over in order from transparent;
//   * a Gaussian blur of the composite, separable, radius kRadius, weights
//     exp(-j^2 / 2 sigma^2) normalised over [-kRadius, kRadius], zero outside
//     the canvas.
// Adjoint: given dL/d(blurred), the blur is transposed (the same symmetric
// filter) and d sigma is accumulated from the derivative weights; then every
// row is re-rendered (coverage recomputed, never stored across rows: the only
// per-row state is a bounded per-CTA scratch of areas and pre-composite
// colours), the composite is reversed path by path, paint-parameter
// gradients are reduced per warp, and the area derivatives of each crossing
// line come from forward-mode dual numbers over the same area function the
// forward pass uses; vertex gradients are chained to control points with the
// Bernstein weights of the flattening.
#include <cuda_runtime.h>
#include <stdint.h>
#include <cmath>
#include <mutex>
#include "kernels.h"
#include "resvg_gpu.h"

namespace rgpu {
void set_last_error_message(const char *msg);  // render.cpp

namespace soft {
namespace {

constexpr int kFlat = 16;      // lines per cubic
constexpr int kThreads = 256;  // threads per row CTA
constexpr int kMaxPx = 4;      // pixels per thread: canvases up to 1024 wide
constexpr int kRadius = 12;    // blur radius (3 x the largest sigma of the workload)
constexpr int kMaxCross = 512; // crossing lines per (path, row) kept in shared memory

// ---- forward-mode dual numbers over the 4 endpoint coordinates of a line
struct D4 {
    float v, d[4];
};
__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float val(const D4 &x) { return x.v; }
__device__ __forceinline__ D4 mk(float v) { D4 r; r.v = v; r.d[0] = r.d[1] = r.d[2] = r.d[3] = 0.f; return r; }
__device__ __forceinline__ D4 operator+(const D4 &a, const D4 &b) {
    D4 r; r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < 4; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ D4 operator-(const D4 &a, const D4 &b) {
    D4 r; r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < 4; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
__device__ __forceinline__ D4 operator*(const D4 &a, const D4 &b) {
    D4 r; r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < 4; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ D4 operator/(const D4 &a, const D4 &b) {
    D4 r; r.v = a.v / b.v;
    const float ib2 = 1.0f / (b.v * b.v);
#pragma unroll
    for (int i = 0; i < 4; i++) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) * ib2;
    return r;
}
__device__ __forceinline__ D4 operator+(const D4 &a, float b) { D4 r = a; r.v += b; return r; }
__device__ __forceinline__ D4 operator-(const D4 &a, float b) { D4 r = a; r.v -= b; return r; }
__device__ __forceinline__ D4 operator-(float a, const D4 &b) {
    D4 r; r.v = a - b.v;
#pragma unroll
    for (int i = 0; i < 4; i++) r.d[i] = -b.d[i];
    return r;
}
__device__ __forceinline__ D4 operator*(const D4 &a, float b) {
    D4 r; r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < 4; i++) r.d[i] = a.d[i] * b;
    return r;
}
__device__ __forceinline__ D4 operator*(float a, const D4 &b) { return b * a; }

template <class T> __device__ __forceinline__ T cst(float v);
template <> __device__ __forceinline__ float cst<float>(float v) { return v; }
template <> __device__ __forceinline__ D4 cst<D4>(float v) { return mk(v); }

// Mean of clamp(1 - x, 0, 1) over x running linearly from a to b.
template <class T>
__device__ __forceinline__ T mean_right(T a, T b) {
    if (val(a) > val(b)) { T t = a; a = b; b = t; }
    if (val(b) <= 0.0f) return cst<T>(1.0f);
    if (val(a) >= 1.0f) return cst<T>(0.0f);
    if (val(a) >= 0.0f && val(b) <= 1.0f) return 1.0f - (a + b) * 0.5f;
    if (val(a) < 0.0f && val(b) <= 1.0f) return 1.0f - (b * b) / ((b - a) * 2.0f);
    if (val(a) >= 0.0f) return ((1.0f - a) * (1.0f - a)) / ((b - a) * 2.0f);
    return (0.5f - a) / (b - a);
}

// A line from (x0, y0) to (x1, y1) clipped to the row [py, py + 1]:
// (xl, xh) the x at the clipped ends and sdy the signed clipped height.
// Returns false when nothing of the line lies in the row.
template <class T>
__device__ __forceinline__ bool clip_row(T x0, T y0, T x1, T y1, float py, T *xl, T *xh, T *sdy) {
    if (val(y0) == val(y1)) return false;
    const float dir = val(y1) > val(y0) ? 1.0f : -1.0f;
    T xa = x0, ya = y0, xb = x1, yb = y1;
    if (dir < 0.0f) { xa = x1; ya = y1; xb = x0; yb = y0; }
    if (!(val(ya) < py + 1.0f && val(yb) > py)) return false;
    T ylo, yhi;
    if (val(ya) >= py) { ylo = ya; *xl = xa; }
    else { ylo = cst<T>(py); *xl = xa + (xb - xa) * ((py - ya) / (yb - ya)); }
    if (val(yb) <= py + 1.0f) { yhi = yb; *xh = xb; }
    else { yhi = cst<T>(py + 1.0f); *xh = xa + (xb - xa) * (((py + 1.0f) - ya) / (yb - ya)); }
    if (!(val(yhi) > val(ylo))) return false;
    *sdy = (yhi - ylo) * dir;
    return true;
}

// ---- paints
struct PaintOut {
    float r, g, b, a;  // straight colour at the pixel, alpha times the path's opacity
    float raw_a;       // the paint's alpha before the opacity
    float op;          // the path's opacity
    int seg;           // gradient: stop interval (-1: below first, 3: at/above last), solid: -2
    float w, t;        // interpolation weight and gradient parameter
};

__device__ __forceinline__ PaintOut eval_paint_raw(const rgpu_soft_batch &B, uint32_t j, float x, float y);

__device__ __forceinline__ PaintOut eval_paint(const rgpu_soft_batch &B, uint32_t j, float x, float y) {
    PaintOut o = eval_paint_raw(B, j, x, y);
    o.op = B.opacity ? B.opacity[j] : 1.0f;
    o.raw_a = o.a;
    o.a = o.a * o.op;
    return o;
}

__device__ __forceinline__ PaintOut eval_paint_raw(const rgpu_soft_batch &B, uint32_t j, float x, float y) {
    PaintOut o;
    o.w = 0.0f; o.t = 0.0f;
    if (B.paint_kind[j] == 0) {
        const float4 c = reinterpret_cast<const float4 *>(B.colors)[j];
        o.r = c.x; o.g = c.y; o.b = c.z; o.a = c.w; o.seg = -2;
        return o;
    }
    const float4 ln = reinterpret_cast<const float4 *>(B.grad_line)[j];
    const float dx = ln.z - ln.x, dy = ln.w - ln.y;
    const float len2 = dx * dx + dy * dy;
    float t = len2 > 0.0f ? ((x - ln.x) * dx + (y - ln.y) * dy) / len2 : 0.0f;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    o.t = t;
    const float *off = B.stop_offsets + 4 * (size_t)j;
    const float4 *sc = reinterpret_cast<const float4 *>(B.stop_colors) + 4 * (size_t)j;
    if (t < off[0]) { const float4 c = sc[0]; o.r = c.x; o.g = c.y; o.b = c.z; o.a = c.w; o.seg = -1; return o; }
    if (t >= off[3]) { const float4 c = sc[3]; o.r = c.x; o.g = c.y; o.b = c.z; o.a = c.w; o.seg = 3; return o; }
    int i = 0;
    if (t >= off[1]) i = 1;
    if (t >= off[2]) i = 2;
    const float span = off[i + 1] - off[i];
    const float w = span > 0.0f ? (t - off[i]) / span : 1.0f;
    const float4 c0 = sc[i], c1 = sc[i + 1];
    o.r = c0.x + w * (c1.x - c0.x);
    o.g = c0.y + w * (c1.y - c0.y);
    o.b = c0.z + w * (c1.z - c0.z);
    o.a = c0.w + w * (c1.w - c0.w);
    o.seg = i; o.w = w;
    return o;
}

struct RowShared {
    float4 cross[kMaxCross];   // (xl, xh, sdy, line index as float bits) per crossing line
    int ncross;
    int warp_count[kThreads / 32];
    float sbuf[kThreads * kMaxPx];  // adjoint: suffix sums of dL/dA over the row, by pixel x
    float dbuf[kThreads * kMaxPx];  // adjoint: dL/dA by pixel x
    // row areas in 2^-40 fixed point, so the sums are exact whatever the order:
    // lines wholly left of a pixel (a difference array, then a prefix sum), and
    // the partial contributions of the lines crossing the pixel's column span
    long long full[kThreads * kMaxPx];
    long long part[kThreads * kMaxPx];
    long long wtot[kThreads / 32];
    float wtotf[kThreads / 32];
};

__device__ __forceinline__ uint32_t path_vbase(const rgpu_soft_batch &B, uint32_t j) { return kFlat * B.seg_offset[j]; }
__device__ __forceinline__ uint32_t path_nverts(const rgpu_soft_batch &B, uint32_t j) {
    return kFlat * (B.seg_offset[j + 1] - B.seg_offset[j]);
}

// Gathers the lines of path j that cross row py into sh.cross, in line order
// (deterministic), with their clipped ends.  All threads call it.
__device__ void gather_crossings(RowShared &sh, const float2 *verts, uint32_t vb, uint32_t nv, float py) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) sh.ncross = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nv; base += kThreads) {
        const uint32_t s = base + (uint32_t)tid;
        float xl = 0.f, xh = 0.f, sdy = 0.f;
        bool hit = false;
        if (s < nv) {
            const float2 a = verts[vb + s];
            const float2 b = verts[vb + (s + 1 < nv ? s + 1 : 0)];
            hit = clip_row<float>(a.x, a.y, b.x, b.y, py, &xl, &xh, &sdy);
        }
        const uint32_t m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) sh.warp_count[warp] = __popc(m);
        __syncthreads();
        int before = 0;
        for (int w = 0; w < warp; w++) before += sh.warp_count[w];
        int total = 0;
        for (int w = 0; w < kThreads / 32; w++) total += sh.warp_count[w];
        const int idx = sh.ncross + before + __popc(m & ((1u << lane) - 1u));
        if (hit && idx < kMaxCross) sh.cross[idx] = make_float4(xl, xh, sdy, __uint_as_float(s));
        __syncthreads();
        if (tid == 0) sh.ncross = min(sh.ncross + total, kMaxCross);
        __syncthreads();
    }
}

constexpr float kFix = 1099511627776.0f;  // 2^40

// The area A(x) = sum over the crossing lines of sdy * mean_right(xl - x, xh - x)
// for every pixel x of the row, by line instead of by pixel: a line adds sdy
// in full to every pixel from ceil(max(xl, xh)) on (there mean_right is 1),
// and evaluates mean_right only over the pixels its x range touches (from
// floor(min(xl, xh)); 0 left of them).  The per-pixel loop over all lines
// costs W x lines; this costs W + the lines' pixel spans.  Sums are taken in
// 2^-40 fixed point with 64-bit shared atomics, so they do not depend on the
// order lines are added in.  All threads call it; A[k] is pixel tid + k x kThreads.
__device__ void row_areas(RowShared &sh, int W, float A[kMaxPx]) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int x = tid; x < W; x += kThreads) {
        sh.full[x] = 0;
        sh.part[x] = 0;
    }
    __syncthreads();
    for (int ci = warp; ci < sh.ncross; ci += kThreads / 32) {
        const float4 c = sh.cross[ci];
        const float xmin = fminf(c.x, c.y), xmax = fmaxf(c.x, c.y);
        const int xr = (int)ceilf(fminf(fmaxf(xmax, -1.0f), (float)W));  // first pixel with mean_right = 1
        if (lane == 0 && xr < W)
            atomicAdd((unsigned long long *)&sh.full[max(xr, 0)], (unsigned long long)__float2ll_rn(c.z * kFix));
        const int x_lo = max((int)floorf(fminf(fmaxf(xmin, -1.0f), (float)W)), 0);
        const int x_hi = min(xr, W) - 1;
        for (int x = x_lo + lane; x <= x_hi; x += 32) {
            const float v = c.z * mean_right<float>(c.x - (float)x, c.y - (float)x);
            if (v != 0.0f) atomicAdd((unsigned long long *)&sh.part[x], (unsigned long long)__float2ll_rn(v * kFix));
        }
    }
    __syncthreads();
    // inclusive prefix sum of `full`: each thread a run of kMaxPx pixels
    long long v[kMaxPx];
    long long run = 0;
    const int base = tid * kMaxPx;
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) {
        run += base + k < W ? sh.full[base + k] : 0;
        v[k] = run;
    }
    long long sc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, sc, o);
        if (lane >= o) sc += t;
    }
    if (lane == 31) sh.wtot[warp] = sc;
    __syncthreads();
    long long off = sc - run;
    for (int w = 0; w < warp; w++) off += sh.wtot[w];
#pragma unroll
    for (int k = 0; k < kMaxPx; k++)
        if (base + k < W) sh.full[base + k] = v[k] + off;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) {
        const int x = tid + k * kThreads;
        A[k] = x < W ? __ll2float_rn(sh.full[x] + sh.part[x]) * (1.0f / kFix) : 0.0f;
    }
    __syncthreads();  // the accumulators are read before the next path clears them
}

// sbuf[x] = sum of dbuf[q] for q >= x, x < W: a block-wide scan over the
// reversed row (each thread a run of kMaxPx pixels from the right), ending
// with a barrier.
__device__ void suffix_sums(RowShared &sh, int W) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float v[kMaxPx];
    float run = 0.0f;
    const int base = tid * kMaxPx;  // reversed position y = W - 1 - x
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) {
        const int y = base + k;
        run += y < W ? sh.dbuf[W - 1 - y] : 0.0f;
        v[k] = run;
    }
    float sc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, sc, o);
        if (lane >= o) sc += t;
    }
    if (lane == 31) sh.wtotf[warp] = sc;
    __syncthreads();
    float off = 0.0f;
    for (int w = 0; w < warp; w++) off += sh.wtotf[w];
    off += sc - run;
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) {
        const int y = base + k;
        if (y < W) sh.sbuf[W - 1 - y] = v[k] + off;
    }
    __syncthreads();
}

// A(x) for this thread's pixels: summed per pixel over the row's lines when
// they are few (lines x pixels per thread <= kLineLoopMax: cheaper than
// row_areas' four barriers), else by row_areas.  The choice depends only on
// shared values, so every thread takes the same branch.
constexpr int kLineLoopMax = 24;
__device__ void areas(RowShared &sh, int W, float A[kMaxPx]) {
    const int ppt = (W + kThreads - 1) / kThreads;
    if (sh.ncross * ppt > kLineLoopMax) {
        row_areas(sh, W, A);
        return;
    }
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) {
        const int x = (int)threadIdx.x + k * kThreads;
        float a = 0.0f;
        if (x < W)
            for (int i = 0; i < sh.ncross; i++) {
                const float4 c = sh.cross[i];
                a += c.z * mean_right<float>(c.x - (float)x, c.y - (float)x);
            }
        A[k] = a;
    }
}

// ---- forward: one CTA per (scene, row)
__global__ void __launch_bounds__(kThreads) k_forward(rgpu_soft_batch B, const float2 *verts, float4 *image,
                                                      uint32_t *overflow) {
    __shared__ RowShared sh;
    const uint32_t s = blockIdx.x / B.height, py = blockIdx.x % B.height;
    const int W = (int)B.width;
    float4 C[kMaxPx];
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) C[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t P = B.paths_per_scene;
    for (uint32_t p = 0; p < P; p++) {
        const uint32_t j = s * P + p;
        gather_crossings(sh, verts, path_vbase(B, j), path_nverts(B, j), (float)py);
        if (threadIdx.x == 0 && sh.ncross >= kMaxCross) atomicOr(overflow, 1u);
        if (sh.ncross > 0) {
            float Ar[kMaxPx];
            areas(sh, W, Ar);
#pragma unroll
            for (int k = 0; k < kMaxPx; k++) {
                const int x = (int)threadIdx.x + k * kThreads;
                if (x >= W) continue;
                const float A = Ar[k];
                const float c = fminf(fabsf(A), 1.0f);
                if (c == 0.0f) continue;
                const PaintOut po = eval_paint(B, j, (float)x + 0.5f, (float)py + 0.5f);
                const float ca = c * po.a;
                const float keep = 1.0f - ca;
                C[k].x = c * (po.r * po.a) + keep * C[k].x;
                C[k].y = c * (po.g * po.a) + keep * C[k].y;
                C[k].z = c * (po.b * po.a) + keep * C[k].z;
                C[k].w = ca + keep * C[k].w;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < kMaxPx; k++) {
        const int x = (int)threadIdx.x + k * kThreads;
        if (x < W) image[((size_t)s * B.height + py) * W + x] = C[k];
    }
}

// ---- flattening: one thread per (path, vertex)
// Control points of cubic c of an n-cubic path (points base 3 * seg_offset):
// start pts[3c] (the previous cubic's end; pts[0] for c = 0), controls
// pts[3c+1], pts[3c+2], end pts[3c+3], or pts[0] for the last cubic.
__device__ __forceinline__ float bern(int role, float t) {
    const float u = 1.0f - t;
    return role == 0 ? u * u * u : role == 1 ? 3.0f * u * u * t : role == 2 ? 3.0f * u * t * t : t * t * t;
}

__global__ void k_flatten(rgpu_soft_batch B, uint32_t npaths, float2 *verts) {
    const uint32_t j = blockIdx.y;
    if (j >= npaths) return;
    const uint32_t s0 = B.seg_offset[j], ns = B.seg_offset[j + 1] - s0;
    const float2 *pts = reinterpret_cast<const float2 *>(B.points) + 3 * s0;
    float2 *v = verts + kFlat * s0;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < kFlat * ns; q += gridDim.x * blockDim.x) {
        const uint32_t c = q / kFlat, i = q % kFlat;
        const float t = (float)i / (float)kFlat;
        const float b0 = bern(0, t), b1 = bern(1, t), b2 = bern(2, t), b3 = bern(3, t);
        const float2 P0 = pts[3 * c], P1 = pts[3 * c + 1], P2 = pts[3 * c + 2];
        const float2 P3 = c + 1 < ns ? pts[3 * c + 3] : pts[0];
        v[q] = make_float2(b0 * P0.x + b1 * P1.x + b2 * P2.x + b3 * P3.x, b0 * P0.y + b1 * P1.y + b2 * P2.y + b3 * P3.y);
    }
}

// vertex gradients -> control-point gradients (the transpose of k_flatten)
__global__ void k_unflatten(rgpu_soft_batch B, uint32_t npaths, const float2 *vgrad, float *pgrad) {
    const uint32_t j = blockIdx.y;
    if (j >= npaths) return;
    const uint32_t s0 = B.seg_offset[j], ns = B.seg_offset[j + 1] - s0;
    const float2 *vg = vgrad + kFlat * s0;
    float2 *pg = reinterpret_cast<float2 *>(pgrad) + 3 * s0;
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < 3 * ns; m += gridDim.x * blockDim.x) {
        float gx = 0.f, gy = 0.f;
        auto add = [&](uint32_t c, int role) {
            for (int i = 0; i < kFlat; i++) {
                const float b = bern(role, (float)i / (float)kFlat);
                const float2 g = vg[kFlat * c + i];
                gx += b * g.x;
                gy += b * g.y;
            }
        };
        const uint32_t c = m / 3, r = m % 3;
        if (r == 0) {
            add(c, 0);                          // start of cubic c
            add(c == 0 ? ns - 1 : c - 1, 3);    // end of the previous cubic (of the last one for c = 0)
        } else {
            add(c, (int)r);
        }
        pg[m] = make_float2(gx, gy);
    }
}

// ---- blur
__device__ __forceinline__ void blur_weights(float sigma, float *w, float *dw) {
    // w_j = exp(-j^2 / 2s^2) / Z; dw_j = d w_j / d sigma
    float z = 0.0f, m = 0.0f;
    float e[2 * kRadius + 1];
    for (int j = -kRadius; j <= kRadius; j++) {
        const float v = expf(-(float)(j * j) / (2.0f * sigma * sigma));
        e[j + kRadius] = v;
        z += v;
        m += v * (float)(j * j);
    }
    const float s3 = sigma * sigma * sigma;
    for (int j = -kRadius; j <= kRadius; j++) {
        const float wj = e[j + kRadius] / z;
        w[j + kRadius] = wj;
        if (dw) dw[j + kRadius] = wj * ((float)(j * j) - m / z) / s3;
    }
}

// out = K (derivative kernel when `deriv`) applied along x (horiz) or y
__global__ void k_blur(const float4 *in, float4 *out, const float *sigma, uint32_t W, uint32_t H, int horiz,
                       int deriv) {
    __shared__ float w[2 * kRadius + 1], dw[2 * kRadius + 1];
    const uint32_t s = blockIdx.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) blur_weights(sigma[s], w, dw);
    __syncthreads();
    const float *k = deriv ? dw : w;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float4 *img = in + (size_t)s * W * H;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int j = -kRadius; j <= kRadius; j++) {
        const int xx = horiz ? (int)x + j : (int)x, yy = horiz ? (int)y : (int)y + j;
        if (xx < 0 || yy < 0 || xx >= (int)W || yy >= (int)H) continue;
        const float4 v = img[(size_t)yy * W + xx];
        const float kj = k[j + kRadius];
        acc.x += kj * v.x; acc.y += kj * v.y; acc.z += kj * v.z; acc.w += kj * v.w;
    }
    out[(size_t)s * W * H + (size_t)y * W + x] = acc;
}

// dsigma[s] += sum over pixels of a . (dK applied to b) along x or y
__global__ void k_dsigma(const float4 *a, const float4 *b, const float *sigma, uint32_t W, uint32_t H, int horiz,
                         float *dsigma) {
    __shared__ float w[2 * kRadius + 1], dw[2 * kRadius + 1];
    __shared__ float red[32];
    const uint32_t s = blockIdx.z;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid == 0) blur_weights(sigma[s], w, dw);
    __syncthreads();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    float sum = 0.0f;
    if (x < W && y < H) {
        const float4 *img = b + (size_t)s * W * H;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int j = -kRadius; j <= kRadius; j++) {
            const int xx = horiz ? (int)x + j : (int)x, yy = horiz ? (int)y : (int)y + j;
            if (xx < 0 || yy < 0 || xx >= (int)W || yy >= (int)H) continue;
            const float4 v = img[(size_t)yy * W + xx];
            const float kj = dw[j + kRadius];
            acc.x += kj * v.x; acc.y += kj * v.y; acc.z += kj * v.z; acc.w += kj * v.w;
        }
        const float4 g = a[(size_t)s * W * H + (size_t)y * W + x];
        sum = g.x * acc.x + g.y * acc.y + g.z * acc.z + g.w * acc.w;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const int nthreads = blockDim.x * blockDim.y;
    if ((tid & 31) == 0) red[tid >> 5] = sum;
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int i = 0; i < nthreads / 32; i++) t += red[i];
        atomicAdd(&dsigma[s], t);
    }
}

// ---- adjoint of the rows: persistent CTAs with bounded scratch
// per path: 16 stop colours + 4 stop offsets (gradient) or 4 colour
// channels (solid), then the opacity at index 20
constexpr int kAcc = 21;

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kThreads, 3) k_backward(rgpu_soft_batch B, rgpu_soft_grads G, const float2 *verts,
                                                       const float4 *grad_image, float *scratch_area,
                                                       float4 *scratch_color, float2 *vgrad, uint32_t *row_counter,
                                                       uint32_t *overflow) {
    __shared__ RowShared sh;
    __shared__ float pacc[kAcc];
    __shared__ int row_sh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = (int)B.width;
    const uint32_t P = B.paths_per_scene;
    const uint32_t nrows = B.scenes * B.height;
    float *areaS = scratch_area + (size_t)blockIdx.x * P * kThreads * kMaxPx;
    float4 *colS = scratch_color + (size_t)blockIdx.x * P * kThreads * kMaxPx;
    for (;;) {
        if (tid == 0) row_sh = (int)atomicAdd(row_counter, 1u);
        __syncthreads();
        const int row = row_sh;
        __syncthreads();
        if (row >= (int)nrows) break;
        const uint32_t s = (uint32_t)row / B.height, py = (uint32_t)row % B.height;
        // forward recompute: areas and pre-composite colours per path
        float4 C[kMaxPx];
#pragma unroll
        for (int k = 0; k < kMaxPx; k++) C[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (uint32_t p = 0; p < P; p++) {
            const uint32_t j = s * P + p;
            gather_crossings(sh, verts, path_vbase(B, j), path_nverts(B, j), (float)py);
            if (tid == 0 && sh.ncross >= kMaxCross) atomicOr(overflow, 1u);
            float Ar[kMaxPx] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (sh.ncross > 0) areas(sh, W, Ar);
#pragma unroll
            for (int k = 0; k < kMaxPx; k++) {
                const int x = tid + k * kThreads;
                const size_t si = ((size_t)p * kMaxPx + k) * kThreads + tid;
                const float A = x < W ? Ar[k] : 0.0f;
                if (x < W) {  // scratch only for the row's pixels
                    areaS[si] = A;
                    colS[si] = C[k];
                }
                const float c = fminf(fabsf(A), 1.0f);
                if (x < W && c != 0.0f) {
                    const PaintOut po = eval_paint(B, j, (float)x + 0.5f, (float)py + 0.5f);
                    const float ca = c * po.a, keep = 1.0f - ca;
                    C[k].x = c * (po.r * po.a) + keep * C[k].x;
                    C[k].y = c * (po.g * po.a) + keep * C[k].y;
                    C[k].z = c * (po.b * po.a) + keep * C[k].z;
                    C[k].w = ca + keep * C[k].w;
                }
            }
            __syncthreads();
        }
        // reverse composite: paint gradients and dL/dA per pixel
        float4 gC[kMaxPx];
#pragma unroll
        for (int k = 0; k < kMaxPx; k++) {
            const int x = tid + k * kThreads;
            gC[k] = x < W ? grad_image[((size_t)s * B.height + py) * W + x] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int p = (int)P - 1; p >= 0; p--) {
            const uint32_t j = s * P + (uint32_t)p;
            float acc[kAcc];
#pragma unroll
            for (int q = 0; q < kAcc; q++) acc[q] = 0.0f;
            const bool is_grad = B.paint_kind[j] != 0;
#pragma unroll
            for (int k = 0; k < kMaxPx; k++) {
                const int x = tid + k * kThreads;
                const size_t si = ((size_t)p * kMaxPx + k) * kThreads + tid;
                const float A = x < W ? areaS[si] : 0.0f;
                const float c = fminf(fabsf(A), 1.0f);
                float dA = 0.0f;
                if (x < W && c != 0.0f) {
                    const float4 Cp = colS[si];
                    const PaintOut po = eval_paint(B, j, (float)x + 0.5f, (float)py + 0.5f);
                    const float4 g = gC[k];
                    const float Pr = po.r * po.a, Pg = po.g * po.a, Pb = po.b * po.a, Pa = po.a;
                    // C = c P + (1 - c a) Cp
                    const float dc = g.x * (Pr - po.a * Cp.x) + g.y * (Pg - po.a * Cp.y) + g.z * (Pb - po.a * Cp.z) +
                                     g.w * (Pa - po.a * Cp.w);
                    const float da_keep = -c * (g.x * Cp.x + g.y * Cp.y + g.z * Cp.z + g.w * Cp.w);
                    const float dPr = c * g.x, dPg = c * g.y, dPb = c * g.z, dPa = c * g.w;
                    // straight colour; `da` is d/d(alpha times opacity): the
                    // paint's own alpha gets da * opacity, the opacity da * alpha
                    const float dr = dPr * po.a, dg = dPg * po.a, db = dPb * po.a;
                    const float da_eff = dPr * po.r + dPg * po.g + dPb * po.b + dPa + da_keep;
                    const float da = da_eff * po.op;
                    acc[20] += da_eff * po.raw_a;
                    if (!is_grad) {
                        acc[0] += dr; acc[1] += dg; acc[2] += db; acc[3] += da;
                    } else if (po.seg < 0 || po.seg == 3) {
                        // flat below the first / above the last stop: that stop's colour
                        const int i = po.seg < 0 ? 0 : 3;
                        acc[4 * i] += dr; acc[4 * i + 1] += dg; acc[4 * i + 2] += db; acc[4 * i + 3] += da;
                    } else {
                        // acc[0..15]: stop colours (4 x RGBA), acc[16..19]: stop offsets
                        const int i = po.seg;
                        const float w = po.w, u = 1.0f - w;
                        acc[4 * i] += u * dr; acc[4 * i + 1] += u * dg; acc[4 * i + 2] += u * db; acc[4 * i + 3] += u * da;
                        acc[4 * i + 4] += w * dr; acc[4 * i + 5] += w * dg; acc[4 * i + 6] += w * db; acc[4 * i + 7] += w * da;
                        // w = (t - o_i) / (o_{i+1} - o_i)
                        const float *off = B.stop_offsets + 4 * (size_t)j;
                        const float span = off[i + 1] - off[i];
                        if (span > 0.0f) {
                            const float4 *sc = reinterpret_cast<const float4 *>(B.stop_colors) + 4 * (size_t)j;
                            const float4 c0 = sc[i], c1 = sc[i + 1];
                            const float dw = dr * (c1.x - c0.x) + dg * (c1.y - c0.y) + db * (c1.z - c0.z) + da * (c1.w - c0.w);
                            const float inv2 = 1.0f / (span * span);
                            acc[16 + i] += dw * (po.t - off[i + 1]) * inv2;
                            acc[16 + i + 1] += -dw * (po.t - off[i]) * inv2;
                        }
                    }
                    gC[k].x *= 1.0f - c * po.a;
                    gC[k].y *= 1.0f - c * po.a;
                    gC[k].z *= 1.0f - c * po.a;
                    gC[k].w *= 1.0f - c * po.a;
                    const float dcA = (fabsf(A) < 1.0f) ? (A > 0.0f ? 1.0f : (A < 0.0f ? -1.0f : 0.0f)) : 0.0f;
                    dA = dc * dcA;
                }
                if (x < W) areaS[si] = dA;
            }
            // reduce the paint gradients of this path over the row
            if (tid < kAcc) pacc[tid] = 0.0f;
            __syncthreads();
            const int nq = is_grad ? kAcc : 5;  // solid: colour channels 0..3, then the opacity
#pragma unroll
            for (int q = 0; q < kAcc; q++) {
                if (q >= nq) break;
                const int qi = (!is_grad && q == 4) ? 20 : q;
                const float v = warp_sum(acc[qi]);
                if (lane == 0 && v != 0.0f) atomicAdd(&pacc[qi], v);
            }
            __syncthreads();
            if (tid < kAcc && pacc[tid] != 0.0f) {
                if (tid == 20) { if (G.opacity) atomicAdd(&G.opacity[j], pacc[20]); }
                else if (!is_grad) atomicAdd(&G.colors[4 * (size_t)j + tid], pacc[tid]);
                else if (tid < 16) atomicAdd(&G.stop_colors[16 * (size_t)j + tid], pacc[tid]);
                else atomicAdd(&G.stop_offsets[4 * (size_t)j + (tid - 16)], pacc[tid]);
            }
            __syncthreads();
        }
        // line gradients: for each path, dA over the row, suffix sums, duals over crossing lines
        for (uint32_t p = 0; p < P; p++) {
            const uint32_t j = s * P + p;
            // dA of this path -> shared (by pixel x), then suffix sums S(x) = sum_{q >= x} dA(q)
#pragma unroll
            for (int k = 0; k < kMaxPx; k++) {
                const size_t si = ((size_t)p * kMaxPx + k) * kThreads + tid;
                const int x = tid + k * kThreads;
                sh.dbuf[x] = x < W ? areaS[si] : 0.0f;
            }
            __syncthreads();
            suffix_sums(sh, W);
            gather_crossings(sh, verts, path_vbase(B, j), path_nverts(B, j), (float)py);
            auto S = [&](int x) -> float { return x >= W ? 0.0f : sh.sbuf[max(x, 0)]; };
            const uint32_t vb = path_vbase(B, j), nv = path_nverts(B, j);
            for (int ci = warp; ci < sh.ncross; ci += kThreads / 32) {
                const float4 cr = sh.cross[ci];
                const uint32_t li = __float_as_uint(cr.w);
                const uint32_t ia = vb + li, ib = vb + (li + 1 < nv ? li + 1 : 0);
                const float2 a = verts[ia], b = verts[ib];
                const float xmin = fminf(cr.x, cr.y), xmax = fmaxf(cr.x, cr.y);
                int x_lo = (int)floorf(xmin), x_hi = (int)ceilf(xmax) - 1;  // pixels with fractional coverage
                x_lo = max(x_lo, 0);
                x_hi = min(x_hi, W - 1);
                float g[4] = {0.f, 0.f, 0.f, 0.f};
                // the line clipped to the row, with derivatives in its end
                // coordinates (the same for every pixel of the row)
                D4 X0 = mk(a.x), Y0 = mk(a.y), X1 = mk(b.x), Y1 = mk(b.y);
                X0.d[0] = 1.f; Y0.d[1] = 1.f; X1.d[2] = 1.f; Y1.d[3] = 1.f;
                D4 xl, xh, sdy;
                const bool crosses = clip_row<D4>(X0, Y0, X1, Y1, (float)py, &xl, &xh, &sdy);
                if (crosses)
                    for (int x = x_lo + lane; x <= x_hi; x += 32) {
                        const float d = sh.dbuf[x];
                        if (d == 0.0f) continue;
                        const D4 v = sdy * mean_right<D4>(xl - (float)x, xh - (float)x);
#pragma unroll
                        for (int q = 0; q < 4; q++) g[q] += d * v.d[q];
                    }
                // pixels right of the line: area = sdy, weighted by the suffix sum
                const int xr = max((int)ceilf(xmax), 0);
                if (crosses && lane == 0 && xr < W) {
                    const float sr = S(xr);
                    if (sr != 0.0f) {
#pragma unroll
                        for (int q = 0; q < 4; q++) g[q] += sr * sdy.d[q];
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; q++) g[q] = warp_sum(g[q]);
                if (lane == 0) {
                    if (g[0] != 0.0f) atomicAdd(&vgrad[ia].x, g[0]);
                    if (g[1] != 0.0f) atomicAdd(&vgrad[ia].y, g[1]);
                    if (g[2] != 0.0f) atomicAdd(&vgrad[ib].x, g[2]);
                    if (g[3] != 0.0f) atomicAdd(&vgrad[ib].y, g[3]);
                }
            }
            __syncthreads();
        }
    }
}

__global__ void k_mse(const float *a, const float *b, size_t n, float scale, float *loss, float *grad) {
    __shared__ float red[32];
    float sum = 0.0f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float d = a[i] - b[i];
        sum += d * d;
        if (grad) grad[i] = 2.0f * d * scale;
    }
    sum = warp_sum(sum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int i = 0; i < (int)(blockDim.x / 32); i++) t += red[i];
        atomicAdd(loss, t * scale);
    }
}

// ---- host side: cached work buffers
struct Buf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
};
std::mutex g_mu;
Buf g_verts, g_vgrad, g_tmp0, g_tmp1, g_tmp2, g_area, g_col, g_flags;

bool valid(const rgpu_soft_batch *b) {
    return b && b->scenes && b->width && b->height && b->paths_per_scene && b->seg_offset && b->points &&
           b->paint_kind && b->colors && b->stop_offsets && b->stop_colors && b->grad_line && b->sigma &&
           b->width <= (uint32_t)(kThreads * kMaxPx) && b->total_segments;
}

int fail(cudaError_t e) {
    set_last_error_message(cudaGetErrorString(e));
    return RGPU_ERR_CUDA;
}

cudaError_t flatten(const rgpu_soft_batch &b, cudaStream_t s) {
    const uint32_t npaths = b.scenes * b.paths_per_scene;
    const size_t nverts = (size_t)kFlat * b.total_segments;
    cudaError_t e = g_verts.ensure(nverts * sizeof(float2));
    if (e != cudaSuccess) return e;
    dim3 grid(1, npaths);
    k_flatten<<<grid, 256, 0, s>>>(b, npaths, (float2 *)g_verts.p);
    return cudaGetLastError();
}

cudaError_t blur(const float4 *in, float4 *out, float4 *tmp, const rgpu_soft_batch &b, cudaStream_t s) {
    dim3 blk(32, 8), grid((b.width + 31) / 32, (b.height + 7) / 8, b.scenes);
    k_blur<<<grid, blk, 0, s>>>(in, tmp, b.sigma, b.width, b.height, 1, 0);
    k_blur<<<grid, blk, 0, s>>>(tmp, out, b.sigma, b.width, b.height, 0, 0);
    return cudaGetLastError();
}

}  // namespace
}  // namespace soft
}  // namespace rgpu

using namespace rgpu::soft;

extern "C" int rgpu_soft_forward(const rgpu_soft_batch *b, float *image, float *blurred, void *stream) {
    rgpu::set_last_error_message("");
    if (!valid(b) || !image || !blurred) {
        rgpu::set_last_error_message("invalid arguments (canvas width is limited to 1024)");
        return RGPU_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = flatten(*b, s);
    if (e == cudaSuccess) e = g_flags.ensure(16);
    if (e == cudaSuccess) e = g_tmp0.ensure((size_t)b->scenes * b->width * b->height * sizeof(float4));
    if (e != cudaSuccess) return fail(e);
    cudaMemsetAsync(g_flags.p, 0, 16, s);
    k_forward<<<b->scenes * b->height, kThreads, 0, s>>>(*b, (const float2 *)g_verts.p, (float4 *)image,
                                                         (uint32_t *)g_flags.p);
    e = blur((const float4 *)image, (float4 *)blurred, (float4 *)g_tmp0.p, *b, s);
    uint32_t ovf = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ovf, g_flags.p, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(e);
    if (ovf) {
        rgpu::set_last_error_message("more than 512 lines of one path cross a pixel row");
        return RGPU_ERR_CAPACITY;
    }
    return RGPU_OK;
}

extern "C" int rgpu_soft_backward(const rgpu_soft_batch *b, const float *image, const float *grad_blurred,
                                  rgpu_soft_grads *g, void *stream) {
    rgpu::set_last_error_message("");
    if (!valid(b) || !image || !grad_blurred || !g || !g->points || !g->colors || !g->stop_offsets ||
        !g->stop_colors || !g->sigma) {
        rgpu::set_last_error_message("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t npaths = b->scenes * b->paths_per_scene;
    const size_t npx = (size_t)b->scenes * b->width * b->height;
    const size_t nverts = (size_t)kFlat * b->total_segments;
    const size_t npts = 3 * (size_t)b->total_segments;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // persistent CTAs taking rows from a counter: as many as fit on the GPU at once
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_backward, kThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 2;
    const uint32_t ctas = (uint32_t)std::max(1, sms) * (uint32_t)per_sm;
    cudaError_t e = flatten(*b, s);
    if (e == cudaSuccess) e = g_vgrad.ensure(nverts * sizeof(float2));
    if (e == cudaSuccess) e = g_tmp0.ensure(npx * sizeof(float4));
    if (e == cudaSuccess) e = g_tmp1.ensure(npx * sizeof(float4));
    if (e == cudaSuccess) e = g_tmp2.ensure(npx * sizeof(float4));
    if (e == cudaSuccess) e = g_area.ensure((size_t)ctas * b->paths_per_scene * kThreads * kMaxPx * sizeof(float));
    if (e == cudaSuccess) e = g_col.ensure((size_t)ctas * b->paths_per_scene * kThreads * kMaxPx * sizeof(float4));
    if (e == cudaSuccess) e = g_flags.ensure(16);
    if (e != cudaSuccess) return fail(e);
    // gradients are overwritten
    cudaMemsetAsync(g->points, 0, npts * sizeof(float2), s);
    cudaMemsetAsync(g->colors, 0, (size_t)npaths * 16, s);
    cudaMemsetAsync(g->stop_offsets, 0, (size_t)npaths * 16, s);
    cudaMemsetAsync(g->stop_colors, 0, (size_t)npaths * 64, s);
    cudaMemsetAsync(g->sigma, 0, (size_t)b->scenes * 4, s);
    if (g->opacity) cudaMemsetAsync(g->opacity, 0, (size_t)npaths * 4, s);
    cudaMemsetAsync(g_vgrad.p, 0, nverts * sizeof(float2), s);
    cudaMemsetAsync(g_flags.p, 0, 16, s);
    const dim3 blk(32, 8), grid((b->width + 31) / 32, (b->height + 7) / 8, b->scenes);
    float4 *gI = (float4 *)g_tmp0.p, *H = (float4 *)g_tmp1.p, *T = (float4 *)g_tmp2.p;
    const float4 *gB = (const float4 *)grad_blurred, *I = (const float4 *)image;
    // blurred = Kv(Kh I): dsigma = <gB, dKv (Kh I)> + <Kv gB, dKh I>; gI = Kh(Kv gB)
    k_blur<<<grid, blk, 0, s>>>(I, H, b->sigma, b->width, b->height, 1, 0);
    k_dsigma<<<grid, blk, 0, s>>>(gB, H, b->sigma, b->width, b->height, 0, g->sigma);
    k_blur<<<grid, blk, 0, s>>>(gB, T, b->sigma, b->width, b->height, 0, 0);
    k_dsigma<<<grid, blk, 0, s>>>(T, I, b->sigma, b->width, b->height, 1, g->sigma);
    k_blur<<<grid, blk, 0, s>>>(T, gI, b->sigma, b->width, b->height, 1, 0);
    // rows (counter lives in the flags word 1)
    k_backward<<<ctas, kThreads, 0, s>>>(*b, *g, (const float2 *)g_verts.p, gI, (float *)g_area.p, (float4 *)g_col.p,
                                         (float2 *)g_vgrad.p, (uint32_t *)g_flags.p + 1, (uint32_t *)g_flags.p);
    dim3 ug(1, npaths);
    k_unflatten<<<ug, 256, 0, s>>>(*b, npaths, (const float2 *)g_vgrad.p, g->points);
    uint32_t ovf = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ovf, g_flags.p, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(e);
    if (ovf) {
        rgpu::set_last_error_message("more than 512 lines of one path cross a pixel row");
        return RGPU_ERR_CAPACITY;
    }
    return RGPU_OK;
}

extern "C" int rgpu_soft_mse(const float *blurred, const float *target, size_t count, float *loss,
                             float *grad_blurred, void *stream) {
    rgpu::set_last_error_message("");
    if (!blurred || !target || !loss || !count) {
        rgpu::set_last_error_message("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(loss, 0, 4, s);
    k_mse<<<1024, 256, 0, s>>>(blurred, target, count, 1.0f / (float)count, loss, grad_blurred);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? RGPU_OK : fail(e);
}
