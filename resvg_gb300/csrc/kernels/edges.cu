// Geometry kernels: per-draw setup, per-segment edge building, exclusive scans
// and row-band binning.
//
// Pipeline for one submission (all draws of all streams):
//   k_draw_setup   thread/draw:    transform points, bounds, scan ranges
//                                  (tiny-skia painter.rs fill_path + scan/path_aa.rs
//                                  fill_path), segment slots (path.rs PathEdgeIter)
//   k_edges<false> thread/segment: count line edges
//   scan           exclusive prefix sum -> edge offsets
//   k_edges<true>  thread/segment: write line edges (edge_builder.rs)
//   k_draw_edges   thread/draw:    edge range; paths with < 2 edges are dropped
//   k_bin<false>   thread/edge:    count (band, draw) bin sizes
//   scan           -> bin offsets
//   k_bin<true>    thread/edge:    copy edges into their bands
#include <cuda_runtime.h>
#include <stdint.h>
#include "edge_build.cuh"
#include "kernels.h"

namespace rgpu {
namespace {

using dev::Pt;

__device__ __forceinline__ bool nearly_zero(float v) { return fabsf(v) <= (1.0f / 4096.0f); }

__global__ void k_draw_setup(DrawRec *draws, uint32_t ndraws, const uint8_t *scene_verbs, const float *scene_pts,
                             const uint8_t *stroke_verbs, const float *stroke_pts, Pt *tpts, SegRec *segs) {
    uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndraws) return;
    DrawRec dr = draws[d];
    // a stroke outline built on the device lives in the stroke arrays
    const bool stroked = (dr.flags & DRAW_STROKED) != 0;
    const uint8_t *verbs = stroked ? stroke_verbs : scene_verbs;
    const float *pts = stroked ? stroke_pts : scene_pts;
    dr.valid = 0;
    dr.edge_base = 0;
    dr.edge_count = 0;
    // segment slots default to empty
    for (uint32_t i = 0; i <= dr.verb_cnt; i++) segs[dr.seg_base + i] = SegRec{d, 0, 0, 0};
    if (dr.flags & 0x80000000u) { draws[d] = dr; return; }  // host-side skip
    // ---- transform (tiny-skia Transform::map_points branches)
    float sx = dr.ts[0], ky = dr.ts[1], kx = dr.ts[2], sy = dr.ts[3], tx = dr.ts[4], ty = dr.ts[5];
    bool ident = sx == 1 && ky == 0 && kx == 0 && sy == 1 && tx == 0 && ty == 0;
    bool skew = kx != 0 || ky != 0;
    bool scale = sx != 1 || sy != 1;
    float l = 0, t = 0, r = 0, b = 0;
    bool finite = true;
    for (uint32_t i = 0; i < dr.pt_cnt; i++) {
        float x = pts[2 * (dr.pt_off + i)], y = pts[2 * (dr.pt_off + i) + 1];
        float nx, ny;
        if (ident) { nx = x; ny = y; }
        else if (!skew && !scale) { nx = x + tx; ny = y + ty; }
        else if (!skew) { nx = x * sx + tx; ny = y * sy + ty; }
        else { nx = x * sx + y * kx + tx; ny = x * ky + y * sy + ty; }
        if (!ident && (!isfinite(nx) || !isfinite(ny))) finite = false;
        tpts[dr.tpt_base + i] = Pt{nx, ny};
        if (i == 0) { l = r = nx; t = b = ny; }
        else { l = fminf(l, nx); r = fmaxf(r, nx); t = fminf(t, ny); b = fmaxf(b, ny); }
    }
    if (!finite || dr.pt_cnt == 0) { draws[d] = dr; return; }
    if (nearly_zero(r - l) || nearly_zero(b - t)) { draws[d] = dr; return; }
    const float lim = 3.4028235e38f * 0.25f;
    if (!(l >= -lim && t >= -lim && r <= lim && b <= lim)) { draws[d] = dr; return; }
    int32_t cw = dr.clip_w, ch = dr.clip_h;
    bool aa = (dr.flags & DRAW_AA) != 0;
    if (aa) {
        float fl = floorf(l), ft = floorf(t), fr = ceilf(r), fb = ceilf(b);
        int32_t ix = dev::sat_i32(fl), iy = dev::sat_i32(ft);
        int32_t iw = max(1, dev::sat_i32(fr - fl)), ih = max(1, dev::sat_i32(fb - ft));
        int32_t sl = max(ix, 0), st = max(iy, 0), sr = min(ix + iw, cw), sb = min(iy + ih, ch);
        if (sr <= sl || sb <= st) { draws[d] = dr; return; }
        bool ovf = sl > 8191 || st > 8191 || sr > 8191 || sb > 8191 || sl < -8192 || st < -8192;
        if (ovf) aa = false;  // supersampled coordinates would overflow i16: aliased fill
        else {
            if (cw > 32767 || ch > 32767) { draws[d] = dr; return; }
            bool contained = ix >= 0 && iy >= 0 && ix + iw <= cw && iy + ih <= ch;
            dr.shift = 2;
            dr.contained = contained;
            dr.sect_l = sl; dr.sect_t = st; dr.sect_r = sr; dr.sect_b = sb;
            int32_t sy0 = iy << 2, sy1 = (iy + ih) << 2;
            if (!contained) { sy0 = max(sy0, 0); sy1 = min(sy1, ch << 2); }
            dr.start_y = sy0; dr.stop_y = sy1;
            dr.right_clip = cw << 2;
            dr.super_left = sl << 2;
            dr.valid = 1;
        }
    }
    if (!aa) {
        const double bias = 0.5 + 1.5 / 64.0;
        int32_t il = dev::sat_i32((float)ceil((double)l - bias));
        int32_t it = dev::sat_i32((float)ceil((double)t - bias));
        int32_t ir = dev::sat_i32((float)floor((double)r + bias));
        int32_t ib = dev::sat_i32((float)floor((double)b + bias));
        if (ir <= il || ib <= it) { draws[d] = dr; return; }
        bool contained = il >= 0 && it >= 0 && ir <= cw && ib <= ch;
        int32_t y0 = it, y1 = ib;
        if (!contained) { y0 = max(y0, 0); y1 = min(y1, ch); }
        if (y0 >= y1) { draws[d] = dr; return; }
        dr.shift = 0;
        dr.contained = contained;
        dr.sect_l = 0; dr.sect_t = 0; dr.sect_r = cw; dr.sect_b = ch;
        dr.start_y = y0; dr.stop_y = y1;
        dr.right_clip = cw;
        dr.super_left = INT32_MIN;
        dr.valid = 1;
    }
    // ---- segments (PathEdgeIter with implicit close lines)
    // validate the verb/point structure first: every drawing verb needs a
    // current point and its points must exist
    {
        uint32_t need = 0;
        bool have_cur = false, ok = true;
        for (uint32_t vi = 0; vi < dr.verb_cnt && ok; vi++) {
            uint8_t v = verbs[dr.verb_off + vi];
            if (v == RGPU_MOVE) { need += 1; have_cur = true; }
            else if (v == RGPU_LINE || v == RGPU_QUAD || v == RGPU_CUBIC) {
                if (!have_cur) ok = false;
                need += v == RGPU_LINE ? 1 : (v == RGPU_QUAD ? 2 : 3);
            } else if (v != RGPU_CLOSE) ok = false;
        }
        if (!ok || need > dr.pt_cnt) { dr.valid = 0; draws[d] = dr; return; }
    }
    uint32_t pi = 0, move_to = 0, ns = 0;
    bool needs_close = false;
    uint32_t base = dr.tpt_base;
    for (uint32_t vi = 0; vi < dr.verb_cnt; vi++) {
        uint8_t v = verbs[dr.verb_off + vi];
        if (v == RGPU_MOVE) {
            if (needs_close) { segs[dr.seg_base + ns++] = SegRec{d, 1, base + pi - 1, base + move_to}; needs_close = false; }
            move_to = pi; pi += 1;
        } else if (v == RGPU_CLOSE) {
            if (needs_close) { segs[dr.seg_base + ns++] = SegRec{d, 1, base + pi - 1, base + move_to}; needs_close = false; }
        } else if (v == RGPU_LINE) {
            needs_close = true;
            segs[dr.seg_base + ns++] = SegRec{d, 1, base + pi - 1, base + pi};
            pi += 1;
        } else if (v == RGPU_QUAD) {
            needs_close = true;
            segs[dr.seg_base + ns++] = SegRec{d, 2, base + pi - 1, 0};
            pi += 2;
        } else if (v == RGPU_CUBIC) {
            needs_close = true;
            segs[dr.seg_base + ns++] = SegRec{d, 3, base + pi - 1, 0};
            pi += 3;
        }
    }
    if (needs_close) segs[dr.seg_base + ns++] = SegRec{d, 1, base + pi - 1, base + move_to};
    draws[d] = dr;
}

template <bool EMIT>
__global__ void k_edges(const SegRec *segs, uint32_t nsegs, const DrawRec *draws, const Pt *tpts, uint32_t *counts,
                        const uint32_t *offsets, EdgeRec *edges, uint32_t *edge_draw, uint32_t edge_cap) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsegs) return;
    SegRec sg = segs[s];
    dev::EdgeSink sink{nullptr, 0, 0};
    if (sg.kind != 0) {
        const DrawRec &dr = draws[sg.draw];
        if (dr.valid) {
            Pt p[4];
            if (sg.kind == 1) { p[0] = tpts[sg.p0]; p[1] = tpts[sg.p1]; }
            else { for (uint32_t k = 0; k <= sg.kind; k++) p[k] = tpts[sg.p0 + k]; }
            dev::ClipR clip{0.0f, 0.0f, (float)dr.clip_w, (float)dr.clip_h};
            if (EMIT) {
                uint32_t off = offsets[s];
                uint32_t cap = off < edge_cap ? edge_cap - off : 0;
                sink = dev::EdgeSink{edges + off, 0, min(cap, counts[s])};
            }
            dev::build_segment(sink, (int)sg.kind, p, dr.contained != 0, clip, dr.shift);
            if (EMIT) {
                uint32_t off = offsets[s];
                for (uint32_t k = 0; k < sink.n && off + k < edge_cap; k++) edge_draw[off + k] = sg.draw;
            }
        }
    }
    if (!EMIT) counts[s] = sink.n;
}

__global__ void k_draw_edges(DrawRec *draws, uint32_t ndraws, const uint32_t *seg_offsets) {
    uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndraws) return;
    DrawRec &dr = draws[d];
    uint32_t b = seg_offsets[dr.seg_base], e = seg_offsets[dr.seg_base + dr.verb_cnt + 1];
    dr.edge_base = b;
    dr.edge_count = e - b;
    if (dr.valid && e - b < 2) dr.valid = 0;
}

template <bool SCATTER>
__global__ void k_bin(const EdgeRec *edges, const uint32_t *edge_draw, uint32_t nedges, const DrawRec *draws,
                      const StreamRec *streams, uint32_t *bin_counts, const uint32_t *bin_offsets, uint32_t bin_cap,
                      uint32_t *err, EdgeRec *bins) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedges) return;
    uint32_t d = edge_draw[e];
    const DrawRec &dr = draws[d];
    if (!dr.valid) return;
    const StreamRec &st = streams[dr.stream];
    EdgeRec er = edges[e];
    int32_t last_y = er.first_y + (er.hw >> 8);
    int32_t y0 = max(er.first_y, dr.start_y), y1 = min(last_y, dr.stop_y - 1);
    if (y1 < y0) return;
    int32_t r0 = (y0 >> dr.shift) + dr.oy, r1 = (y1 >> dr.shift) + dr.oy;
    int32_t bh = (int32_t)st.band_rows;
    int32_t b0 = r0 >= 0 ? r0 / bh : -((-r0 + bh - 1) / bh);
    int32_t b1 = r1 >= 0 ? r1 / bh : -((-r1 + bh - 1) / bh);
    b0 = max(b0, 0);
    b1 = min(b1, (int32_t)st.nbands - 1);
    uint32_t ld = d - st.draw_off;
    for (int32_t b = b0; b <= b1; b++) {
        uint32_t slot = st.bin_off + (uint32_t)b * st.draw_cnt + ld;
        uint32_t k = atomicAdd(&bin_counts[slot], 1u);
        if (SCATTER) {
            uint32_t pos = bin_offsets[slot] + k;
            if (pos < bin_cap) bins[pos] = er;
            else atomicOr(err, 1u);
        }
    }
}

// ---- exclusive scan (three passes, 1024-element tiles)
constexpr int SCAN_T = 256;
constexpr int SCAN_PER = 4;
constexpr int SCAN_TILE = SCAN_T * SCAN_PER;

__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t *sh, uint32_t *total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < (SCAN_T / 32) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (SCAN_T / 32)) sh[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = wid ? sh[wid - 1] : 0;
    *total = sh[SCAN_T / 32 - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void k_scan_reduce(const uint32_t *in, uint64_t n, uint32_t *block_sums) {
    __shared__ uint32_t sh[32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
    for (int k = 0; k < SCAN_PER; k++) {
        uint64_t i = base + (uint64_t)threadIdx.x * SCAN_PER + k;
        if (i < n) s += in[i];
    }
    uint32_t total;
    block_exclusive(s, sh, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}
__global__ void k_scan_blocks(uint32_t *block_sums, uint32_t nblocks, uint32_t *total_out) {
    __shared__ uint32_t sh[32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nblocks; base += SCAN_T) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < nblocks ? block_sums[i] : 0;
        uint32_t tot;
        uint32_t ex = block_exclusive(v, sh, &tot);
        if (i < nblocks) block_sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total_out = carry;
}
__global__ void k_scan_down(const uint32_t *in, uint64_t n, const uint32_t *block_sums, uint32_t *out) {
    __shared__ uint32_t sh[32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t v[SCAN_PER];
    uint32_t s = 0;
    for (int k = 0; k < SCAN_PER; k++) {
        uint64_t i = base + (uint64_t)threadIdx.x * SCAN_PER + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    uint32_t total;
    uint32_t ex = block_exclusive(s, sh, &total) + block_sums[blockIdx.x];
    for (int k = 0; k < SCAN_PER; k++) {
        uint64_t i = base + (uint64_t)threadIdx.x * SCAN_PER + k;
        if (i < n) out[i] = ex;
        ex += v[k];
    }
}

inline uint32_t blocks_for(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------- host launchers
cudaError_t launch_draw_setup(DrawRec *draws, uint32_t ndraws, const uint8_t *verbs, const float *pts,
                              const uint8_t *stroke_verbs, const float *stroke_pts, void *tpts, SegRec *segs,
                              cudaStream_t s) {
    if (!ndraws) return cudaSuccess;
    k_draw_setup<<<blocks_for(ndraws, 128), 128, 0, s>>>(draws, ndraws, verbs, pts, stroke_verbs, stroke_pts,
                                                         (Pt *)tpts, segs);
    return cudaGetLastError();
}
cudaError_t launch_edges(bool emit, const SegRec *segs, uint32_t nsegs, const DrawRec *draws, const void *tpts,
                         uint32_t *counts, const uint32_t *offsets, EdgeRec *edges, uint32_t *edge_draw,
                         uint32_t edge_cap, cudaStream_t s) {
    if (!nsegs) return cudaSuccess;
    if (emit)
        k_edges<true><<<blocks_for(nsegs, 128), 128, 0, s>>>(segs, nsegs, draws, (const Pt *)tpts, counts, offsets,
                                                              edges, edge_draw, edge_cap);
    else
        k_edges<false><<<blocks_for(nsegs, 128), 128, 0, s>>>(segs, nsegs, draws, (const Pt *)tpts, counts, offsets,
                                                               edges, edge_draw, edge_cap);
    return cudaGetLastError();
}
cudaError_t launch_draw_edges(DrawRec *draws, uint32_t ndraws, const uint32_t *seg_offsets, cudaStream_t s) {
    if (!ndraws) return cudaSuccess;
    k_draw_edges<<<blocks_for(ndraws, 256), 256, 0, s>>>(draws, ndraws, seg_offsets);
    return cudaGetLastError();
}
cudaError_t launch_bin(bool scatter, const EdgeRec *edges, const uint32_t *edge_draw, uint32_t nedges,
                       const DrawRec *draws, const StreamRec *streams, uint32_t *bin_counts,
                       const uint32_t *bin_offsets, uint32_t bin_cap, uint32_t *err, EdgeRec *bins, cudaStream_t s) {
    if (!nedges) return cudaSuccess;
    if (scatter)
        k_bin<true><<<blocks_for(nedges, 256), 256, 0, s>>>(edges, edge_draw, nedges, draws, streams, bin_counts,
                                                             bin_offsets, bin_cap, err, bins);
    else
        k_bin<false><<<blocks_for(nedges, 256), 256, 0, s>>>(edges, edge_draw, nedges, draws, streams, bin_counts,
                                                              bin_offsets, bin_cap, err, bins);
    return cudaGetLastError();
}
size_t scan_scratch_words(uint64_t n) { return (size_t)blocks_for(n ? n : 1, SCAN_TILE) + 1; }
// out[i] = sum(in[0..i)), *total = sum(in); `scratch` holds scan_scratch_words(n) words.
cudaError_t launch_exclusive_scan(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *scratch, uint32_t *total,
                                  cudaStream_t s) {
    if (n == 0) return cudaMemsetAsync(total, 0, 4, s);
    uint32_t nb = blocks_for(n, SCAN_TILE);
    k_scan_reduce<<<nb, SCAN_T, 0, s>>>(in, n, scratch);
    k_scan_blocks<<<1, SCAN_T, 0, s>>>(scratch, nb, total);
    k_scan_down<<<nb, SCAN_T, 0, s>>>(in, n, scratch, out);
    return cudaGetLastError();
}

}  // namespace rgpu
