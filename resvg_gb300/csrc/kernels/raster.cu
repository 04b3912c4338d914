// The band VM: one persistent kernel renders every work item (a band of output
// rows, optionally an x-chunk of it) by executing its stream's command list.
//
// Coverage follows tiny-skia's supersampling scan converter (scan/path_aa.rs:
// SHIFT = 2, 4 sub-scanlines x 4 sub-columns per pixel; SkScan_AntiPath):
//   phase A  (one thread per (draw, sub-scanline)): gather the crossings of the
//            draw's binned edges with the sub-scanline, sort them by x, and walk
//            them with the fill rule (scan/path.rs walk_edges) into spans
//            [L, R) of sub-columns, applying the super_left clamp and the
//            right-clip span of an unclosed winding;
//   phase B  (one thread per PX consecutive pixels): per pixel, each span adds
//            16 per covered sub-column, or 64 (63 on the 4th sub-scanline) when
//            it covers the whole pixel (SuperBlitter::blit_h's max_value), and
//            the sum is capped at 255 (SkAlphaRuns catch-overflow).  The pixel
//            is then shaded and blended in registers (lowp or highp pipeline).
// Phase A is batched over the next K fill commands so all 256 threads work.
// The top layer of the command stream's layer stack lives in registers; pushed
// layers spill to per-CTA global scratch (L2 resident).
#include <cuda_runtime.h>
#include <stdint.h>
#include "kernels.h"
#include "pipeline.cuh"

namespace rgpu {
namespace {

constexpr int kThreads = 256;
constexpr int kXCap = 40;        // crossings held per thread before the exact slow path
constexpr int kSpanCap = 12;     // spans per (slot, sub-scanline) kept in shared memory
constexpr int kMaxDepth = 48;    // layer stack depth

struct VmShared {
    int32_t win_first;           // first command index of the prepared window
    int32_t win_last;            // one past the last command index covered by the window
    int32_t nslots;
    int32_t slot_cmd[kThreads];  // command index per slot
    uint16_t span_cnt[kThreads];
    int2 spans[kThreads * kSpanCap];
    int32_t item;
};

__device__ __forceinline__ int32_t round16(int32_t x) { return (int32_t)((uint32_t)x + 0x8000u) >> 16; }

// Exact slow path: the crossings in (x, position) order by repeated minimum
// search when a sub-scanline has more than kXCap crossings.
struct Crossing { int32_t x; int32_t w; };

__device__ void store_span(VmShared &sh, int2 *ovf, uint32_t ovf_cap, int slot_j, int idx, int32_t L, int32_t R,
                           uint32_t *err) {
    if (idx < kSpanCap) sh.spans[slot_j * kSpanCap + idx] = make_int2(L, R);
    else if ((uint32_t)(idx - kSpanCap) < ovf_cap) ovf[(size_t)slot_j * ovf_cap + (idx - kSpanCap)] = make_int2(L, R);
    else atomicOr(err, 2u);
}
__device__ __forceinline__ int2 load_span(const VmShared &sh, const int2 *ovf, uint32_t ovf_cap, int slot_j, int idx) {
    return idx < kSpanCap ? sh.spans[slot_j * kSpanCap + idx] : ovf[(size_t)slot_j * ovf_cap + (idx - kSpanCap)];
}

// Phase A for one (draw, scanline): spans into slot `sj`.
__device__ void phase_a(VmShared &sh, int sj, const DrawRec &dr, int32_t y, const EdgeRec *bl, uint32_t nb,
                        int2 *ovf, uint32_t ovf_cap, uint32_t *err) {
    int nspans = 0;
    if (!dr.valid || y < dr.start_y || y >= dr.stop_y || nb == 0) { sh.span_cnt[sj] = 0; return; }
    int32_t mask = (dr.flags & DRAW_EVENODD) ? 1 : -1;
    // gather + insertion sort (key: x, then bin position)
    Crossing xs[kXCap];
    int n = 0;
    bool overflow = false;
    for (uint32_t i = 0; i < nb; i++) {
        EdgeRec e = bl[i];
        int32_t h = e.hw >> 8;
        if (y < e.first_y || y > e.first_y + h) continue;
        int32_t X = (int32_t)((uint32_t)e.x + (uint32_t)(y - e.first_y) * (uint32_t)e.dx);
        int32_t w = (int32_t)(int8_t)(e.hw & 0xff);
        if (n == kXCap) { overflow = true; break; }
        int k = n++;
        while (k > 0 && (xs[k - 1].x > X || (xs[k - 1].x == X && xs[k - 1].w > w))) { xs[k] = xs[k - 1]; k--; }
        xs[k] = Crossing{X, w};
    }
    int32_t right_clip = dr.right_clip, super_left = dr.super_left;
    auto emit = [&](int32_t L, int32_t R) {
        if (L < super_left) L = super_left;
        if (R <= L) return;
        store_span(sh, ovf, ovf_cap, sj, nspans, L, R, err);
        nspans++;
    };
    int32_t w = 0, left = 0;
    if (!overflow) {
        for (int i = 0; i < n; i++) {
            int32_t x = dr.shift ? round16(xs[i].x) : round16(xs[i].x);
            if ((w & mask) == 0) left = x;
            w += xs[i].w;
            if ((w & mask) == 0 && x > left) emit(left, x);
        }
    } else {
        // repeated minimum over (x, bin position)
        int32_t last_x = INT32_MIN;
        int32_t last_i = -1, last_w = -128;
        for (;;) {
            int32_t bx = INT32_MAX, bi = -1, bw = 127;
            for (uint32_t i = 0; i < nb; i++) {
                EdgeRec e = bl[i];
                int32_t h = e.hw >> 8;
                if (y < e.first_y || y > e.first_y + h) continue;
                int32_t X = (int32_t)((uint32_t)e.x + (uint32_t)(y - e.first_y) * (uint32_t)e.dx);
                int32_t ew = (int32_t)(int8_t)(e.hw & 0xff);
                // order key (x, winding, bin position); equal (x, winding) pairs commute
                bool after = X > last_x || (X == last_x && (ew > last_w || (ew == last_w && (int32_t)i > last_i)));
                bool better = X < bx || (X == bx && (ew < bw || (ew == bw && (int32_t)i < bi)));
                if (after && better) { bx = X; bi = (int32_t)i; bw = ew; }
            }
            if (bi < 0) break;
            last_x = bx; last_i = bi; last_w = bw;
            int32_t x = round16(bx);
            if ((w & mask) == 0) left = x;
            w += bw;
            if ((w & mask) == 0 && x > left) emit(left, x);
        }
    }
    if ((w & mask) != 0 && right_clip > left) emit(left, right_clip);
    sh.span_cnt[sj] = (uint16_t)min(nspans, kSpanCap + (int)ovf_cap);
}

template <int PX>
__global__ void __launch_bounds__(kThreads, 2)
k_raster(const StreamRec *streams, const WorkItem *items, uint32_t nitems, uint32_t *item_counter, const Cmd *cmds,
         const DrawRec *draws, const PaintRec *paints, const GradRec *grads, const LayerRec *layers,
         const EdgeRec *bins, const uint32_t *bin_offsets, const uint32_t *bin_counts, uint32_t *stack_scratch,
         uint32_t stack_depth, int2 *span_ovf, uint32_t ovf_cap, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VmShared &sh = *reinterpret_cast<VmShared *>(smem_raw);
    const int tid = threadIdx.x;
    uint32_t *stack = stack_scratch + (size_t)blockIdx.x * stack_depth * kThreads * PX;
    int2 *ovf = span_ovf + (size_t)blockIdx.x * kThreads * ovf_cap;

    for (;;) {
        if (tid == 0) sh.item = (int32_t)atomicAdd(item_counter, 1u);
        __syncthreads();
        int32_t item_idx = sh.item;
        __syncthreads();
        if (item_idx >= (int32_t)nitems) break;
        const WorkItem wi = items[item_idx];
        const StreamRec st = streams[wi.stream];
        const int BH = (int)st.band_rows;
        const int S = 4 * BH;                 // scanline slots per draw (sub-scanlines for AA)
        const int K = kThreads / S;           // draws per phase-A window
        const int tpr = kThreads / BH;        // threads per pixel row
        const int row = tid / tpr;
        const int32_t cy = (int32_t)wi.band * BH + row;
        const int32_t cx0 = wi.x0 + (tid % tpr) * PX;
        const bool row_ok = cy < st.out_h;
        uint8_t *out = (uint8_t *)(uintptr_t)st.out_ptr;

        uint32_t px[PX];
#pragma unroll
        for (int i = 0; i < PX; i++) {
            int32_t x = cx0 + i;
            px[i] = (row_ok && x < st.out_w && x < wi.x1) ? *(const uint32_t *)(out + (size_t)cy * st.out_stride + 4 * (size_t)x) : 0u;
        }
        // layer stack: rect of each level in output space
        int32_t depth = 0;
        int32_t top_x = 0, top_y = 0, top_w = st.out_w, top_h = st.out_h;
        int32_t rect_x[kMaxDepth], rect_y[kMaxDepth], rect_w[kMaxDepth], rect_h[kMaxDepth];

        if (tid == 0) { sh.win_first = 0; sh.win_last = 0; sh.nslots = 0; }
        __syncthreads();
        int32_t slot_next = 0;

        for (uint32_t ci = 0; ci < st.cmd_cnt; ci++) {
            const Cmd c = cmds[st.cmd_off + ci];
            if (c.op == CMD_FILL || c.op == CMD_APPLY_REGION) {
                if ((int32_t)ci >= sh.win_last) {
                    // ---- prepare a new phase-A window starting at this command
                    __syncthreads();
                    if (tid == 0) {
                        int ns = 0;
                        uint32_t cj = ci;
                        for (; cj < st.cmd_cnt && ns < K; cj++) {
                            uint32_t op = cmds[st.cmd_off + cj].op;
                            if (op == CMD_FILL || op == CMD_APPLY_REGION) sh.slot_cmd[ns++] = (int32_t)cj;
                        }
                        sh.win_first = (int32_t)ci;
                        sh.win_last = (int32_t)cj;
                        sh.nslots = ns;
                    }
                    __syncthreads();
                    slot_next = 0;
                    int k = tid / S, j = tid % S;
                    if (k < sh.nslots) {
                        const Cmd fc = cmds[st.cmd_off + sh.slot_cmd[k]];
                        const DrawRec dr = draws[fc.a];
                        uint32_t ld = fc.a - st.draw_off;
                        uint32_t slot = st.bin_off + wi.band * st.draw_cnt + ld;
                        // scanline for (draw, j): layer row of this band's first row
                        int32_t lrow0 = (int32_t)wi.band * BH - dr.oy;
                        int32_t y;
                        bool ok;
                        if (dr.shift) { y = lrow0 * 4 + j; ok = true; }
                        else { y = lrow0 + j; ok = j < BH; }
                        if (ok && dr.valid) phase_a(sh, tid, dr, y, bins + bin_offsets[slot], bin_counts[slot], ovf, ovf_cap, err);
                        else sh.span_cnt[tid] = 0;
                    }
                    __syncthreads();
                }
                // ---- phase B for this command's slot
                const int slot = slot_next++;
                const DrawRec dr = draws[c.a];
                uint32_t cov[PX];
#pragma unroll
                for (int i = 0; i < PX; i++) cov[i] = 0;
                const int32_t ly = cy - dr.oy;
                const int32_t lx0 = cx0 - dr.ox;
                if (dr.valid && row_ok && ly >= dr.sect_t && ly < dr.sect_b) {
                    const int32_t lrow0 = (int32_t)wi.band * BH - dr.oy;
                    if (dr.shift) {
                        for (int s = 0; s < 4; s++) {
                            const int j = (ly - lrow0) * 4 + s;
                            const int sj = slot * S + j;
                            const int n = sh.span_cnt[sj];
                            const uint32_t maxv = s == 3 ? 63u : 64u;
                            const int32_t a0 = lx0 << 2, a1 = (lx0 + PX) << 2;
                            for (int q = 0; q < n; q++) {
                                int2 sp = load_span(sh, ovf, ovf_cap, sj, q);
                                if (sp.y <= a0) continue;
                                if (sp.x >= a1) break;
#pragma unroll
                                for (int i = 0; i < PX; i++) {
                                    int32_t p0 = (lx0 + i) << 2;
                                    int32_t ov = min(sp.y, p0 + 4) - max(sp.x, p0);
                                    if (ov > 0) cov[i] += ov == 4 ? maxv : (uint32_t)ov * 16u;
                                }
                            }
                        }
                    } else {
                        const int j = ly - lrow0;
                        const int sj = slot * S + j;
                        const int n = sh.span_cnt[sj];
                        for (int q = 0; q < n; q++) {
                            int2 sp = load_span(sh, ovf, ovf_cap, sj, q);
#pragma unroll
                            for (int i = 0; i < PX; i++) {
                                int32_t x = lx0 + i;
                                if (x >= sp.x && x < sp.y) cov[i] = 255;
                            }
                        }
                    }
                }
                const PaintRec pr = paints[dr.paint];
#pragma unroll
                for (int i = 0; i < PX; i++) {
                    int32_t lx = lx0 + i;
                    uint32_t cv = min(cov[i], 255u);
                    if (lx < dr.sect_l || lx >= dr.sect_r) cv = 0;
                    if (c.op == CMD_FILL) {
                        if (cv && !(pr.flags & PAINT_SKIP)) px[i] = dev::shade_pixel(pr, grads, lx, ly, cv, px[i]);
                    } else {
                        // region mask: Mask::fill_path coverage (lerp 0 -> 255), then apply_mask
                        int32_t x = cx0 + i;
                        bool in_top = row_ok && x >= top_x && x < top_x + top_w && cy >= top_y && cy < top_y + top_h;
                        if (in_top) {
                            uint32_t m = cv == 255 ? 255u
                                                   : (uint32_t)dev::div255((uint32_t)dev::sat_u16(((float)cv * dev::kInv255) * 255.0f + 0.5f) * 255u);
                            px[i] = dev::mask_pixel(px[i], m);
                        }
                    }
                }
            } else if (c.op == CMD_PUSH) {
                if (depth + 1 >= kMaxDepth || (uint32_t)depth >= stack_depth) { atomicOr(err, 4u); break; }
                uint32_t *lvl = stack + (size_t)depth * kThreads * PX + (size_t)tid * PX;
#pragma unroll
                for (int i = 0; i < PX; i++) lvl[i] = px[i];
                rect_x[depth] = top_x; rect_y[depth] = top_y; rect_w[depth] = top_w; rect_h[depth] = top_h;
                depth++;
                const LayerRec L = layers[st.layer_off + c.a];
                top_x = L.x; top_y = L.y; top_w = L.w; top_h = L.h;
                uint32_t init = c.b == 1 ? 0xFF000000u : 0u;
#pragma unroll
                for (int i = 0; i < PX; i++) {
                    int32_t x = cx0 + i;
                    bool in = x >= top_x && x < top_x + top_w && cy >= top_y && cy < top_y + top_h;
                    px[i] = in ? init : 0u;
                }
            } else if (c.op == CMD_POP_COMPOSITE || c.op == CMD_POP_CLIP || c.op == CMD_POP_MASK) {
                if (depth == 0) { atomicOr(err, 4u); break; }
                depth--;
                const uint32_t *lvl = stack + (size_t)depth * kThreads * PX + (size_t)tid * PX;
                int32_t px0 = rect_x[depth], py0 = rect_y[depth], pw = rect_w[depth], ph = rect_h[depth];
#pragma unroll
                for (int i = 0; i < PX; i++) {
                    int32_t x = cx0 + i;
                    uint32_t parent = lvl[i];
                    bool in_child = x >= top_x && x < top_x + top_w && cy >= top_y && cy < top_y + top_h;
                    bool in_parent = x >= px0 && x < px0 + pw && cy >= py0 && cy < py0 + ph;
                    if (in_child && in_parent) {
                        if (c.op == CMD_POP_COMPOSITE) parent = dev::composite_pixel(px[i], parent, c.f, c.b);
                        else if (c.op == CMD_POP_CLIP) parent = dev::mask_pixel(parent, 255u - dev::ch(px[i], 3));
                        else parent = dev::mask_pixel(parent, dev::mask_value(px[i], c.b == 0));
                    }
                    px[i] = parent;
                }
                top_x = px0; top_y = py0; top_w = pw; top_h = ph;
            } else if (c.op == CMD_CLEAR) {
#pragma unroll
                for (int i = 0; i < PX; i++) {
                    int32_t x = cx0 + i;
                    bool in = x >= top_x && x < top_x + top_w && cy >= top_y && cy < top_y + top_h;
                    if (in) px[i] = 0u;
                }
            } else if (c.op == CMD_END) {
                break;
            }
        }
        // ---- write back the root layer
        if (depth != 0) atomicOr(err, 8u);
#pragma unroll
        for (int i = 0; i < PX; i++) {
            int32_t x = cx0 + i;
            if (row_ok && x < st.out_w && x < wi.x1) *(uint32_t *)(out + (size_t)cy * st.out_stride + 4 * (size_t)x) = px[i];
        }
        __syncthreads();
    }
}

}  // namespace

size_t raster_smem_bytes() { return sizeof(VmShared); }
size_t raster_stack_words_per_cta(int px) { return (size_t)kMaxDepth * kThreads * px; }
int raster_threads() { return kThreads; }

cudaError_t launch_raster(int px, uint32_t grid, uint32_t stack_depth, const StreamRec *streams, const WorkItem *items, uint32_t nitems,
                          uint32_t *item_counter, const Cmd *cmds, const DrawRec *draws, const PaintRec *paints,
                          const GradRec *grads, const LayerRec *layers, const EdgeRec *bins,
                          const uint32_t *bin_offsets, const uint32_t *bin_counts, uint32_t *stack, int2 *span_ovf,
                          uint32_t ovf_cap, uint32_t *err, cudaStream_t s) {
    size_t smem = sizeof(VmShared);
    cudaError_t e;
    switch (px) {
    case 4:
        e = cudaFuncSetAttribute(k_raster<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_raster<4><<<grid, kThreads, smem, s>>>(streams, items, nitems, item_counter, cmds, draws, paints, grads, layers,
                                                  bins, bin_offsets, bin_counts, stack, stack_depth, span_ovf, ovf_cap, err);
        break;
    case 8:
        e = cudaFuncSetAttribute(k_raster<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_raster<8><<<grid, kThreads, smem, s>>>(streams, items, nitems, item_counter, cmds, draws, paints, grads, layers,
                                                  bins, bin_offsets, bin_counts, stack, stack_depth, span_ovf, ovf_cap, err);
        break;
    default:
        e = cudaFuncSetAttribute(k_raster<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_raster<16><<<grid, kThreads, smem, s>>>(streams, items, nitems, item_counter, cmds, draws, paints, grads,
                                                   layers, bins, bin_offsets, bin_counts, stack, stack_depth, span_ovf, ovf_cap, err);
        break;
    }
    return cudaGetLastError();
}

}  // namespace rgpu

namespace rgpu {
int raster_max_blocks_per_sm(int px) {
    int n = 0;
    size_t smem = raster_smem_bytes();
    cudaError_t e;
    if (px == 4) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster<4>, raster_threads(), smem);
    else if (px == 8) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster<8>, raster_threads(), smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster<16>, raster_threads(), smem);
    if (e != cudaSuccess || n < 1) n = 1;
    return n;
}
}  // namespace rgpu
