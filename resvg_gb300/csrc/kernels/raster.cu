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

constexpr int kThreads = 256;    // consumer threads: they own the band's pixels
constexpr int kProducers = 128;  // producer threads: phase A and the run merge of the next window
constexpr int kBlock = kThreads + kProducers;
constexpr int kXCap = 40;        // crossings held per thread before the exact slow path
constexpr int kSpanCap = 8;      // spans per (slot, sub-scanline) kept in shared memory
constexpr int kSpanStride = kSpanCap + 1;  // padded: neighbouring lists start in different banks
constexpr int kMaxDepth = 48;    // layer stack depth

constexpr int kMaxSlots = 32;   // draws per phase-A window
constexpr uint32_t kWinBufs = 3;  // window buffers: the producers run up to two windows ahead
constexpr int kMaxPairs = kThreads / 4;  // (slot, row) pairs per window: K x BH <= kThreads / 4
constexpr int kRunCap = 32;     // alpha runs per (slot, row) kept in shared memory
constexpr int kRunStride = kRunCap + 1;

// A work item taken from the queue, with its stream (idx >= the item count:
// the queue is empty and both roles stop).
struct ItemInfo {
    int32_t idx;
    int32_t _pad[3];
    WorkItem wi;
    StreamRec st;
};

// One phase-A window as the consumers read it: the window's paints and draw
// origins, and per (slot, row) the alpha runs.  kWinBufs of them rotate: the
// producers fill the next ones while the consumers shade from the oldest.
struct WinBuf {
    // alpha runs per (slot, row), including the closing sentinel; the upper
    // half stays zero: a consumer that gave up on a window reads its counts there
    uint16_t run_cnt[2 * kMaxPairs];
    int2 run_ext[kMaxPairs];      // [first, last) layer x with non-zero coverage per (slot, row)
    int2 runs[kMaxPairs * kRunStride];
    PaintRec paint[kMaxSlots + 1];   // paints of the window's draws; [kMaxSlots] of buffer 0: the hairline's
    int4 slot_geo[kMaxSlots];    // (unused, ox, oy, unused) per slot

};
struct VmShared {
    uint16_t span_cnt[kThreads];  // producer-private: spans per (slot, sub-scanline) task
    int2 spans[kThreads * kSpanStride];
    WinBuf win[kWinBufs];
    unsigned long long mb_ready[kWinBufs];  // mbarriers: window in buffer b produced (kProducers arrivals)
    unsigned long long mb_free[kWinBufs];   // buffer b consumed (kThreads arrivals)
    int32_t abort;                   // set on an error: the rest of the launch skips work and waits
    int32_t cabort;                  // consumers only: set (for good) by a consumer that has seen an abort
    unsigned long long mb_item_ready[2];  // item ring entry filled (1 arrival: producer 0)
    unsigned long long mb_item_free[2];   // item ring entry done with (kThreads arrivals)
    int4 rects[kMaxDepth];       // layer-stack rects (x, y, w, h) by depth, the top one at [depth]
    ItemInfo items[2];           // ring of work items: producers fetch ahead of the consumers
    ItemInfo cur;                // the consumers' current item (a copy: the ring entry is released early)
    // followed by the top layer: kThreads * px uint32 pixels (dynamic)
};

// ---- producer / consumer hand-off (mbarriers, every wait bounded)
// try_wait rounds before a wait is declared stuck (the launch's wait_limit
// argument; rgpu_set_wait_limit changes it)
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mb_init(unsigned long long *mb, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mb)), "r"(count) : "memory");
}
__device__ __forceinline__ void mb_arrive(unsigned long long *mb) {
    asm volatile("{ .reg .b64 st; mbarrier.arrive.shared::cta.b64 st, [%0]; }" ::"r"(smem_addr(mb)) : "memory");
}
// Waits for the phase of parity `parity` to complete; false (and error bit 16)
// when it does not within `limit` rounds, or at once when the CTA has aborted.
// The caller proceeds either way, so every thread still reaches every later
// barrier; after an abort no window is read and no pixel is written.
__device__ __forceinline__ bool mb_wait(unsigned long long *mb, uint32_t parity, uint32_t *err,
                                        const volatile int32_t *abort, uint32_t limit) {
    const uint32_t a = smem_addr(mb);
    for (uint32_t it = 0; it < limit; it++) {
        if ((it & 255u) == 0u && *abort) return false;
        uint32_t ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    atomicOr(err, 16u);
    *const_cast<volatile int32_t *>(abort) = 1;
    return false;
}
// barriers of the consumer threads only (named barrier 1) and of the producer
// threads only (named barrier 2)
__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kThreads) : "memory"); }
__device__ __forceinline__ void producer_sync() { asm volatile("bar.sync 2, %0;" ::"n"(kProducers) : "memory"); }

__device__ __forceinline__ int32_t round16(int32_t x) { return (int32_t)((uint32_t)x + 0x8000u) >> 16; }

// Exact slow path: the crossings in (x, position) order by repeated minimum
// search when a sub-scanline has more than kXCap crossings.
struct Crossing { int32_t x; int32_t w; };

// Spans of one (slot, scanline) live in shared memory while they fit; a
// longer list moves as a whole to the per-CTA global overflow area.
__device__ void store_span(VmShared &sh, int2 *ovf, uint32_t ovf_cap, int slot_j, int idx, int32_t L, int32_t R,
                           uint32_t *err) {
    int2 *o = ovf + (size_t)slot_j * ovf_cap;
    if (idx < kSpanCap) {
        sh.spans[slot_j * kSpanStride + idx] = make_int2(L, R);
        return;
    }
    if (idx == kSpanCap)
        for (int k = 0; k < kSpanCap; k++) o[k] = sh.spans[slot_j * kSpanStride + k];
    if ((uint32_t)idx < ovf_cap) o[idx] = make_int2(L, R);
    else atomicOr(err, 2u);
}
__device__ __forceinline__ const int2 *span_base(const VmShared &sh, const int2 *ovf, uint32_t ovf_cap, int slot_j,
                                                 int n) {
    return n <= kSpanCap ? &sh.spans[slot_j * kSpanStride] : ovf + (size_t)slot_j * ovf_cap;
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
    EdgeRec en = bl[0];  // the next edge, loaded one iteration ahead
    for (uint32_t i = 0; i < nb; i++) {
        const EdgeRec e = en;
        if (i + 1 < nb) en = bl[i + 1];
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
    sh.span_cnt[sj] = (uint16_t)min(nspans, (int)ovf_cap);
}


// Coverage contribution of one scanline's spans to pixel sub-column range
// [p0, p0+4), for the warp window [w0, w1); `q` is a cursor past spans that
// end left of the window (windows advance left to right).
__device__ __forceinline__ uint32_t span_cov(const int2 *L, int n, int &q, int32_t w0, int32_t w1, int32_t p0,
                                             uint32_t maxv) {
    while (q < n && L[q].y <= w0) q++;
    uint32_t cov = 0;
    for (int k = q; k < n; k++) {
        const int2 a = L[k];
        if (a.x >= w1) break;
        const int32_t ov = min(a.y, p0 + 4) - max(a.x, p0);
        if (ov > 0) cov += ov == 4 ? maxv : (uint32_t)ov * 16u;
    }
    return cov;
}

// Alpha runs of one (slot, row): entries (end, alpha), alpha covering the
// layer pixels [previous end, end), the list closed by (INT32_MAX, 0), so a
// pixel's coverage is the alpha of the first entry whose end exceeds it.  The
// pixel coverage is SuperBlitter's (scan/path_aa.rs): over the row's 4
// sub-scanlines, 16 per covered sub-column, or 64 (63 on the 4th) for a fully
// covered pixel, capped at 255; aliased spans are whole pixels at 255.  Only
// [lo, hi) (the draw's coverage rect, the work item) can be non-zero.
struct RunWriter {
    int2 *sm, *gl;
    uint32_t gcap;
    int n;
    int32_t alpha;        // alpha from the last stored end onwards
    int32_t first, last;  // extent of the non-zero coverage
    __device__ void put(int32_t end, int32_t a, uint32_t *err) {
        if (n < kRunCap) sm[n] = make_int2(end, a);
        else {
            if (n == kRunCap)
                for (int k = 0; k < kRunCap; k++) gl[k] = sm[k];
            // the last entry that fits stays a sentinel, so readers always stop
            if ((uint32_t)n + 1 < gcap) gl[n] = make_int2(end, a);
            else { gl[gcap - 1] = make_int2(INT32_MAX, 0); if (end != INT32_MAX) atomicOr(err, 2u); }
        }
        n++;
    }
    // coverage changes to `a` at pixel x
    __device__ __forceinline__ void set(int32_t x, int32_t a, uint32_t *err) {
        if (a != alpha) {
            if (alpha == 0) first = min(first, x);
            else if (a == 0) last = x;
            put(x, alpha, err);
            alpha = a;
        }
    }
};

__device__ void merge_runs(VmShared &sh, WinBuf &wb, const int2 *ovf, uint32_t ovf_cap, int2 *rovf, uint32_t rovf_cap,
                           int pair, int sj, bool aa, int32_t lo, int32_t hi, uint32_t *err) {
    RunWriter w{&wb.runs[pair * kRunStride], rovf + (size_t)pair * rovf_cap, rovf_cap, 0, 0, INT32_MAX, INT32_MIN};
    if (aa) {
        const int2 *L[4];
        int n[4], q[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            n[j] = sh.span_cnt[sj + j];
            L[j] = span_base(sh, ovf, ovf_cap, sj + j, n[j]);
            q[j] = 0;
        }
        int32_t x = lo;
        while (x < hi) {
            int32_t nxt = hi;
            uint32_t sum = 0;
            const int32_t p0 = x << 2;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                while (q[j] < n[j] && L[j][q[j]].y <= p0) q[j]++;
                for (int k = q[j]; k < n[j]; k++) {
                    const int2 a = L[j][k];
                    if (a.x >= p0 + 4) { nxt = min(nxt, a.x >> 2); break; }
                    const int32_t ov = min(a.y, p0 + 4) - max(a.x, p0);
                    if (ov == 4) {  // full from here up to the pixel holding the span's end
                        sum += j == 3 ? 63u : 64u;
                        nxt = min(nxt, a.y >> 2);
                    } else {
                        sum += (uint32_t)ov * 16u;
                        nxt = min(nxt, x + 1);
                    }
                }
            }
            w.set(x, (int32_t)min(sum, 255u), err);
            x = nxt;
        }
    } else {
        const int n0 = sh.span_cnt[sj];
        const int2 *L0 = span_base(sh, ovf, ovf_cap, sj, n0);
        for (int k = 0; k < n0; k++) {
            const int2 a = L0[k];
            const int32_t x0 = max(a.x, lo), x1 = min(a.y, hi);
            if (x0 >= x1) continue;
            w.set(x0, 255, err);
            w.set(x1, 0, err);
        }
    }
    w.set(hi, 0, err);
    w.put(INT32_MAX, 0, err);
    wb.run_cnt[pair] = (uint16_t)min(w.n, (int)rovf_cap);
    wb.run_ext[pair] = make_int2(w.first, w.last);
}

// The anti-aliased merge of one (slot, row) by the two neighbouring producer
// lanes that ran its phase A: each lane walks two of the row's four
// sub-scanline span lists (`half` 0: sub-scanlines 0, 1; 1: 2, 3), and at
// every coverage change the lanes add their partial coverage and take the
// nearer next change through shuffles, so both step through the same
// positions; the even lane writes the runs.  The result is the one-lane
// merge's (the sum of the four lists' contributions and the minimum of their
// next changes do not depend on the split).
__device__ void merge_runs_aa2(VmShared &sh, WinBuf &wb, const int2 *ovf, uint32_t ovf_cap, int2 *rovf,
                               uint32_t rovf_cap, int pair, int sj0, int half, int32_t lo, int32_t hi, uint32_t *err) {
    const unsigned mask = 3u << ((threadIdx.x & 31u) & ~1u);
    RunWriter w{&wb.runs[pair * kRunStride], rovf + (size_t)pair * rovf_cap, rovf_cap, 0, 0, INT32_MAX, INT32_MIN};
    const int2 *L[2];
    int n[2], q[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        n[j] = sh.span_cnt[sj0 + 2 * half + j];
        L[j] = span_base(sh, ovf, ovf_cap, sj0 + 2 * half + j, n[j]);
        q[j] = 0;
    }
    int32_t x = lo;
    while (x < hi) {
        int32_t nxt = hi;
        uint32_t sum = 0;
        const int32_t p0 = x << 2;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            while (q[j] < n[j] && L[j][q[j]].y <= p0) q[j]++;
            for (int k = q[j]; k < n[j]; k++) {
                const int2 a = L[j][k];
                if (a.x >= p0 + 4) { nxt = min(nxt, a.x >> 2); break; }
                const int32_t ov = min(a.y, p0 + 4) - max(a.x, p0);
                if (ov == 4) {  // full from here up to the pixel holding the span's end
                    sum += (half == 1 && j == 1) ? 63u : 64u;
                    nxt = min(nxt, a.y >> 2);
                } else {
                    sum += (uint32_t)ov * 16u;
                    nxt = min(nxt, x + 1);
                }
            }
        }
        sum += __shfl_xor_sync(mask, sum, 1);
        nxt = min(nxt, __shfl_xor_sync(mask, nxt, 1));
        if (half == 0) w.set(x, (int32_t)min(sum, 255u), err);
        x = nxt;
    }
    if (half == 0) {
        w.set(hi, 0, err);
        w.put(INT32_MAX, 0, err);
        wb.run_cnt[pair] = (uint16_t)min(w.n, (int)rovf_cap);
        wb.run_ext[pair] = make_int2(w.first, w.last);
    }
}

__device__ __forceinline__ const int2 *run_base(const WinBuf &wb, const int2 *rovf, uint32_t rovf_cap, int pair) {
    return wb.run_cnt[pair] <= kRunCap ? &wb.runs[pair * kRunStride] : rovf + (size_t)pair * rovf_cap;
}

// Coverage of layer pixel (px, py) from one hairline span (tiny-skia
// scan/hairline_aa.rs: the step k on the pixel's major coordinate, the two
// pixels its blitter touches, alpha scaled by the end-cap fraction); 0 = no
// blit.  A vline whose two columns coincide (x in [0, 1)) blits each pixel
// twice: the host emits it as two spans, the second (HAIR_SECOND) carrying
// only the second blit.
static_assert(sizeof(HairSpan) == 32, "a hairline span is two int4: setup, then its pixel rect");

// A read-only 16-byte load the compiler keeps in place: hoisting a span's
// fields out of the per-pixel loop would hold eight more registers across it.
__device__ __forceinline__ int4 ld_span(const int4 *p) {
    int4 r;
    asm volatile("ld.global.nc.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p));
    return r;
}

__device__ __forceinline__ uint32_t hair_cov(const HairSpan *hsp, int32_t px, int32_t py) {
    const int4 r = ld_span(reinterpret_cast<const int4 *>(hsp) + 1);
    if (px < r.x || py < r.y || px >= r.z || py >= r.w) return 0u;
    const int4 q = ld_span(reinterpret_cast<const int4 *>(hsp));
    const int32_t istart = q.x, f0 = q.y, slope = q.z;
    const uint32_t pack = (uint32_t)q.w, kind = pack & 3u;
    const int32_t n = (int32_t)(pack >> 16);
    const int32_t k = (kind < 2 ? px : py) - istart, minor = kind < 2 ? py : px;
    const int32_t cv = slope >= 0 ? max(f0, 0) + k * slope : max(f0 + k * slope, 0);
    const int32_t hi = cv >> 16;
    const uint32_t a = (uint32_t)(cv >> 8) & 0xFFu;
    const uint32_t stop = (pack >> 9) & 127u;
    const uint32_t mod = k == 0 ? ((pack >> 2) & 127u) : ((k == n - 1 && stop > 0) ? stop : 64u);
    const uint32_t sa = (a * mod) >> 6, sna = ((255u - a) * mod) >> 6;
    const int32_t lo = max(hi, 1) - 1;
    if (kind == 0) {  // hline: row hi, then row hi - 1 (when hi >= 1)
        if (minor == hi) return sa;
        return (hi >= 1 && minor == hi - 1) ? sna : 0u;
    }
    if (kind == 2) {  // vline: column hi, then column max(hi, 1) - 1
        if (pack & HAIR_SECOND) return minor == lo ? sna : 0u;
        if (minor == hi) return sa;
        return (minor == lo && lo != hi) ? sna : 0u;
    }
    // horish / vertish: lo then lo + 1
    return minor == lo ? sna : (minor == lo + 1 ? sa : 0u);
}

// One phase-A window by the producer threads (pt = 0 .. kProducers-1) into
// buffer wb: stage the window's paints and draw origins, run phase
// A for two (slot, sub-scanline) tasks per thread, then merge each (slot, row)
// into alpha runs (a row's tasks sit in one warp, so a warp barrier orders
// them).
__device__ __forceinline__ void produce_window(VmShared &sh, const ItemInfo &itm, WinBuf &wb, int pt, uint32_t wfirst,
                                               const Cmd *cmds,
                                               const uint32_t *fill_cmds, const DrawRec *draws,
                                               const PaintRec *paints, const EdgeRec *bins,
                                               const uint32_t *bin_offsets, const uint32_t *bin_counts, int2 *ovf,
                                               uint32_t ovf_cap, int2 *rovf, uint32_t rovf_cap, uint32_t *err) {
    const WorkItem &wi = itm.wi;
    const StreamRec &st = itm.st;
    const int BH = (int)st.band_rows;
    const int S = 4 * BH;
    const int K = min(kThreads / S, kMaxSlots);
    const uint32_t nsl = min((uint32_t)K, st.fill_cnt - wfirst);
    const uint32_t *flist = fill_cmds + st.fill_off + wfirst;
    const int pw = pt >> 5, lane = pt & 31;
    // lane j fetches slot j's draw and paint indices (one wave of dependent
    // loads per warp instead of one per slot); the slots' users shuffle them
    uint32_t my_di = 0, my_pi = 0;
    if (lane < (int)nsl) {
        my_di = cmds[st.cmd_off + flist[lane]].a;
        my_pi = draws[my_di].paint;
    }
    for (uint32_t k = (uint32_t)pw; k < nsl; k += kProducers / 32) {
        const uint32_t di = __shfl_sync(0xffffffffu, my_di, (int)k);
        const uint32_t pi = __shfl_sync(0xffffffffu, my_pi, (int)k);
        if (lane < (int)(sizeof(PaintRec) / 4))
            ((uint32_t *)&wb.paint[k])[lane] = ((const uint32_t *)&paints[pi])[lane];
        if (lane == 0) wb.slot_geo[k] = make_int4(0, draws[di].ox, draws[di].oy, 0);
    }
    // tasks 2 pt and 2 pt + 1: the same slot (S = 4 x band rows, a power of two)
    const int Sshift = 31 - __clz(S);
    const int u0 = 2 * pt, k = u0 >> Sshift, j0 = u0 & (S - 1);
    const uint32_t kdi = __shfl_sync(0xffffffffu, my_di, k & 31);
    DrawRec dr;
    if (k < (int)nsl) {
        const uint32_t di = kdi;
        dr = draws[di];
        const uint32_t slot = st.bin_off + wi.band * st.draw_cnt + (di - st.draw_off);
        const EdgeRec *bl = bins + bin_offsets[slot];
        const uint32_t nb = bin_counts[slot];
        const int32_t lrow0 = (int32_t)wi.band * BH - dr.oy;
        for (int h = 0; h < 2; h++) {
            const int j = j0 + h;
            int32_t y;
            bool ok;
            if (dr.shift) { y = lrow0 * 4 + j; ok = true; }
            else { y = lrow0 + j; ok = j < BH; }
            if (ok && dr.valid) phase_a(sh, u0 + h, dr, y, bl, nb, ovf, ovf_cap, err);
            else sh.span_cnt[u0 + h] = 0;
        }
    }
    __syncwarp();
    if (k < (int)nsl) {
        // row r2's four sub-scanlines are tasks 4 r2 .. 4 r2 + 3: two lanes
        const int r2 = j0 >> 2;
        const int32_t ly = (int32_t)wi.band * BH + r2 - dr.oy;
        int32_t lo = max(dr.sect_l, wi.x0 - dr.ox), hi = min(dr.sect_r, wi.x1 - dr.ox);
        if (!dr.valid || ly < dr.sect_t || ly >= dr.sect_b || (int32_t)wi.band * BH + r2 >= st.out_h) hi = lo;
        if (dr.shift)
            merge_runs_aa2(sh, wb, ovf, ovf_cap, rovf, rovf_cap, k * BH + r2, k * S + (j0 & ~3), (j0 >> 1) & 1, lo,
                           hi, err);
        else if ((j0 & 3) == 0 && r2 < BH)
            merge_runs(sh, wb, ovf, ovf_cap, rovf, rovf_cap, k * BH + r2, k * S + r2, false, lo, hi, err);
    }
    __syncwarp();  // the merge has read the spans before the next window's phase A overwrites them
}

__global__ void __launch_bounds__(kBlock, 2)
k_raster(int PX, const StreamRec *streams, const WorkItem *items, uint32_t nitems, uint32_t *item_counter,
         const Cmd *cmds, const uint32_t *fill_cmds, const DrawRec *draws, const PaintRec *paints, const GradRec *grads, const LayerRec *layers,
         const EdgeRec *bins, const uint32_t *bin_offsets, const uint32_t *bin_counts, uint32_t *stack_scratch,
         uint32_t stack_depth, int2 *span_ovf, uint32_t ovf_cap, int2 *run_ovf, uint32_t rovf_cap, const HairRec *hairs,
         const HairSpan *hair_spans, uint32_t *err, uint32_t wait_limit, uint32_t withhold) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VmShared &sh = *reinterpret_cast<VmShared *>(smem_raw);
    uint32_t *layer = reinterpret_cast<uint32_t *>(smem_raw + ((sizeof(VmShared) + 15) & ~(size_t)15));
    const int tid = threadIdx.x;
    uint32_t *stack = stack_scratch + (size_t)blockIdx.x * stack_depth * kThreads * PX;
    int2 *ovf = span_ovf + (size_t)blockIdx.x * kThreads * ovf_cap;
    // two run-overflow areas per CTA, one per window buffer
    int2 *rovf = run_ovf + (size_t)blockIdx.x * kWinBufs * kMaxPairs * rovf_cap;
    if (tid == 0) {
        for (uint32_t b = 0; b < kWinBufs; b++) {
            mb_init(&sh.mb_ready[b], kProducers);
            mb_init(&sh.mb_free[b], kThreads);
        }
        mb_init(&sh.mb_item_ready[0], 1);
        mb_init(&sh.mb_item_ready[1], 1);
        mb_init(&sh.mb_item_free[0], kThreads);
        mb_init(&sh.mb_item_free[1], kThreads);
        sh.abort = 0;
        sh.cabort = 0;
    }
    if (tid < (int)kWinBufs * kMaxPairs) sh.win[tid / kMaxPairs].run_cnt[kMaxPairs + tid % kMaxPairs] = 0;
    __syncthreads();
    uint32_t win_base = 0;  // windows produced and consumed by this CTA so far

    if (tid >= kThreads) {
        // ---- producers: take items from the queue (up to two ahead of the
        // consumers) and build each item's windows in order (two buffers ahead)
        const int pt = tid - kThreads;
        for (uint32_t seq = 0;; seq++) {
            const uint32_t is = seq & 1u;
            if (pt == 0) {
                if (seq >= 2) mb_wait(&sh.mb_item_free[is], ((seq >> 1) - 1u) & 1u, err, &sh.abort, wait_limit);
                // a wait that returned because of an abort is ordered before the
                // entry is overwritten: a consumer that sees part of the new
                // entry also sees the abort
                __threadfence_block();
                ItemInfo &w = sh.items[is];
                const int32_t idx = (int32_t)atomicAdd(item_counter, 1u);
                w.idx = idx;
                if (idx < (int32_t)nitems) {
                    w.wi = items[idx];
                    w.st = streams[w.wi.stream];
                }
            }
            producer_sync();
            if (pt == 0) mb_arrive(&sh.mb_item_ready[is]);
            const ItemInfo &itm = sh.items[is];
            if (itm.idx >= (int32_t)nitems) break;
            const int S = 4 * (int)itm.st.band_rows;
            const int K = min(kThreads / S, kMaxSlots);
            const uint32_t nwin = (itm.st.fill_cnt + (uint32_t)K - 1) / (uint32_t)K;
            for (uint32_t w = 0; w < nwin; w++) {
                const uint32_t gw = win_base + w, b = gw % kWinBufs;
                if (gw >= kWinBufs) mb_wait(&sh.mb_free[b], (gw / kWinBufs - 1u) & 1u, err, &sh.abort, wait_limit);
                // one decision per warp: produce_window synchronises its warps
                const bool skip = __any_sync(0xffffffffu, *(volatile int32_t *)&sh.abort != 0);
                if (!skip)
                    produce_window(sh, itm, sh.win[b], pt, w * (uint32_t)K, cmds, fill_cmds, draws, paints,
                                   bins, bin_offsets, bin_counts, ovf, ovf_cap,
                                   rovf + (size_t)b * kMaxPairs * rovf_cap, rovf_cap, err);
                // failure-detection test hook: CTA 0 never completes its first
                // window, so its consumers' bounded wait must run out
                if (!(withhold && blockIdx.x == 0 && gw == 0)) mb_arrive(&sh.mb_ready[b]);
            }
            win_base += nwin;
        }
        return;
    }

    // After an abort (a wait that ran out sets `abort`, and every later wait
    // returns at once) a window buffer may hold a window that was not
    // produced.  A consumer that sees the abort at a window reads that
    // window's run counts from the zero half of `run_cnt`, so every fill is
    // skipped without touching the window, and stores no pixel; it runs the
    // command list like the others so the consumer barriers still match.  At
    // the next item every consumer stops: the decision is taken at the item
    // barrier from `cabort`, which only consumers write, only before that
    // barrier, and never clear, so all of them read the same value.
    for (uint32_t seq = 0;; seq++) {
        const uint32_t is = seq & 1u;
        mb_wait(&sh.mb_item_ready[is], (seq >> 1) & 1u, err, &sh.abort, wait_limit);
        if (tid == 0) {
            sh.cur = sh.items[is];
            sh.rects[0] = make_int4(0, 0, sh.cur.st.out_w, sh.cur.st.out_h);
            __threadfence_block();  // the copy, then the abort flag (see the producers' fence)
        }
        if (*(volatile int32_t *)&sh.abort != 0) *(volatile int32_t *)&sh.cabort = 1;
        consumer_sync();
        const bool stop = *(volatile int32_t *)&sh.cabort != 0;
        mb_arrive(&sh.mb_item_free[is]);  // the entry is copied: the producers may refill it
        // After an abort the producers stop waiting for ring entries to be
        // released, so the copy may mix two items: nobody uses it.  The
        // producers' remaining waits return at once, so the launch ends.
        if (stop || sh.cur.idx >= (int32_t)nitems) break;
        const WorkItem &wi = sh.cur.wi;
        const StreamRec &st = sh.cur.st;
        const int BH = (int)st.band_rows;
        const int S = 4 * BH;                 // scanline slots per draw (sub-scanlines for AA)
        const int K = min(kThreads / S, kMaxSlots);  // a power of two: 8, 16 or 32
        const int Kshift = 31 - __clz(K);
        const uint32_t nwin = (st.fill_cnt + (uint32_t)K - 1) >> Kshift;
        // ---- consumers
        const int tpr = kThreads / BH;        // threads per pixel row
        const int row = tid / tpr;
        const int lr = tid % tpr;             // lane within the row: pixel x = x0 + i*tpr + lr
        // Lane-interleaved pixels: at each step i the 32 lanes of a warp shade 32
        // neighbouring pixels, which mostly share a run and take the same branches.
        const int tpr_sh = 31 - __clz(tpr);    // tpr is a power of two
        const int32_t cy = (int32_t)wi.band * BH + row;
        const bool row_ok = cy < st.out_h;
        uint8_t *out = (uint8_t *)(uintptr_t)st.out_ptr;
        // pixel (i) of this thread lives in layer[i * kThreads + tid]
        for (int i = 0; i < PX; i++) {
            int32_t x = wi.x0 + i * tpr + lr;
            layer[i * kThreads + tid] =
                (row_ok && x < wi.x1) ? *(const uint32_t *)(out + (size_t)cy * st.out_stride + 4 * (size_t)x) : 0u;
        }
        int32_t depth = 0;
        int32_t slot_next = 0;
        uint32_t cur_b = 0;      // window buffer of the current fills
        int32_t cnt_off = 0;     // kMaxPairs after an abort: run counts from the zero half
        uint32_t fill_seen = 0;  // fill commands of the stream before the current one

        for (uint32_t ci = 0; ci < st.cmd_cnt; ci++) {
            const Cmd c = cmds[st.cmd_off + ci];
            if (c.op == CMD_FILL || c.op == CMD_APPLY_REGION || c.op == CMD_HAIR) {
                if (c.op != CMD_HAIR && (fill_seen & (uint32_t)(K - 1)) == 0) {
                    // ---- the next window: release the previous buffer, wait for this one
                    const uint32_t gw = win_base + (fill_seen >> Kshift);
                    if (fill_seen) mb_arrive(&sh.mb_free[(gw - 1u) % kWinBufs]);
                    mb_wait(&sh.mb_ready[gw % kWinBufs], (gw / kWinBufs) & 1u, err, &sh.abort, wait_limit);
                    // a failed wait sets `abort`; producers skip windows after
                    // an abort but still arrive
                    cur_b = gw % kWinBufs;
                    cnt_off = *(volatile int32_t *)&sh.abort != 0 ? kMaxPairs : 0;
                    slot_next = 0;
                }
                // ---- phase B: coverage + shading, one pixel per (thread, i).  A hairline
                // (CMD_HAIR) runs its spans in order through the same loop, each thread
                // for its own pixels, so blits to one pixel keep their order.
                const bool hair = c.op == CMD_HAIR;
                int32_t ox, oy;
                int slot;
                // coverage source: alpha runs of a fill (rp, cursor q), or for a
                // hairline its span list (hs, hn), the chunk of 32 being walked (hq)
                // and the chunk's spans that meet this work item (hm)
                const int2 *rp = nullptr;
                int q = 0;
                int i_lo = 0, i_hi = PX;  // this thread's pixels that can be covered
                int hs = 0, hn = 0, hq = -32;
                uint32_t hm = 0;
                if (hair) {
                    // stage the hairline's paint in the spare slot (uniform across the CTA)
                    const HairRec hr = hairs[c.a];
                    {
                        const int32_t lx0 = wi.x0 - hr.ox, ly0 = (int32_t)wi.band * BH - hr.oy;
                        if (hr.x1 <= lx0 || hr.x0 >= wi.x1 - hr.ox || hr.y1 <= ly0 || hr.y0 >= ly0 + BH) continue;
                    }
                    consumer_sync();  // the previous hairline's pixels are done with the slot
                    slot = kMaxSlots;  // the spare slot of buffer 0 (producers never write it)
                    if (tid == 0) sh.win[0].paint[slot] = paints[hr.paint];
                    consumer_sync();
                    if (sh.win[0].paint[slot].flags & PAINT_SKIP) continue;
                    ox = hr.ox; oy = hr.oy;
                    hs = (int)hr.span_off;
                    hn = (int)hr.span_cnt;
                } else {
                    fill_seen++;
                    slot = slot_next++;
                    const int pair = slot * BH + row;
                    // one entry: the closing sentinel alone, nothing covered on this
                    // row; none: the window is not read after an abort
                    const WinBuf &wb = sh.win[cur_b];
                    const uint32_t rc = wb.run_cnt[pair + cnt_off];
                    if (rc == 0u || (rc == 1u && c.op == CMD_FILL)) continue;
                    const int4 geo = wb.slot_geo[slot];
                    ox = geo.y; oy = geo.z;
                    rp = run_base(wb, rovf + (size_t)cur_b * kMaxPairs * rovf_cap, rovf_cap, pair);
                    if (c.op == CMD_FILL) {
                        // pixel i sits at layer x = x0 - ox + lr + i * tpr; only
                        // [first, last) of the row has coverage
                        const int2 e = wb.run_ext[pair];
                        const int32_t b0 = wi.x0 - ox + lr;
                        const int32_t n0 = e.x - b0, n1 = e.y - b0;
                        i_lo = n0 <= 0 ? 0 : (n0 + tpr - 1) >> tpr_sh;
                        i_hi = n1 <= 0 ? 0 : min(PX, (n1 + tpr - 1) >> tpr_sh);
                    }
                }
                const WinBuf &pb = sh.win[hair ? 0u : cur_b];
                const PaintRec &pr = pb.paint[slot];
                // gradient and image records are read from global memory through the
                // read-only path: not staging them leaves the producers less work and
                // shared memory for a third window buffer
                const GradRec *gr = grads + pr.grad;
                const int32_t ly = cy - oy;
                const int32_t lrow0 = (int32_t)wi.band * BH - oy;
#pragma unroll 1
                for (;;) {
                    int hcur = 0;
                    if (hair) {
                        // the next span that meets this work item, in order: each warp
                        // tests 32 span rects at a time (the same answer in every warp)
                        while (hm == 0) {
                            hq += 32;
                            if (hq >= hn) break;
                            const int j = hq + (tid & 31);
                            bool meets = false;
                            if (j < hn) {
                                const int4 r = __ldg(reinterpret_cast<const int4 *>(hair_spans + hs + j) + 1);
                                meets = !(r.z <= wi.x0 - ox || r.x >= wi.x1 - ox || r.w <= lrow0 || r.y >= lrow0 + BH);
                            }
                            hm = __ballot_sync(0xffffffffu, meets);
                        }
                        if (hm == 0) break;
                        hcur = hs + hq + __ffs(hm) - 1;  // the span to draw
                        hm &= hm - 1;
                    }
#pragma unroll 1
                    for (int i = i_lo; i < i_hi; i++) {
                        const int32_t x = wi.x0 + i * tpr + lr;
                        const int32_t lx = x - ox;
                        uint32_t cv = 0;
                        if (hair) {
                            if (row_ok && x < wi.x1) cv = hair_cov(hair_spans + hcur, lx, ly);
                        } else {
                            while (rp[q].x <= lx) q++;
                            cv = (uint32_t)rp[q].y;
                        }
                        uint32_t &px = layer[i * kThreads + tid];
                        if (c.op != CMD_APPLY_REGION) {
                            if (cv && !(pr.flags & PAINT_SKIP)) px = dev::shade_pixel(pr, gr, lx, ly, cv, px);
                        } else {
                            // region mask: Mask::fill_path coverage (lerp 0 -> 255), then apply_mask
                            const int4 t = sh.rects[depth];
                            const bool in_top = row_ok && x < wi.x1 && x >= t.x && x < t.x + t.z && cy >= t.y &&
                                                cy < t.y + t.w;
                            if (in_top) {
                                uint32_t m = cv == 255 ? 255u
                                                       : (uint32_t)dev::div255((uint32_t)dev::sat_u16(((float)cv * dev::kInv255) * 255.0f + 0.5f) * 255u);
                                px = dev::mask_pixel(px, m);
                            }
                        }
                    }
                    if (!hair) break;
                }
            } else if (c.op == CMD_PUSH) {
                consumer_sync();
                if (depth + 1 >= kMaxDepth || (uint32_t)depth >= stack_depth) {
                    atomicOr(err, 4u);
                    sh.abort = 1;
                    break;
                }
                uint32_t *lvl = stack + (size_t)depth * kThreads * PX;
                for (int i = 0; i < PX; i++) lvl[i * kThreads + tid] = layer[i * kThreads + tid];
                depth++;
                const LayerRec L = layers[st.layer_off + c.a];
                const uint32_t init = c.b == 1 ? 0xFF000000u : 0u;
                const bool row_in = cy >= L.y && cy < L.y + L.h;
                const uint32_t *src = (c.b == 2 && L.buf) ? (const uint32_t *)(uintptr_t)L.buf : nullptr;
                for (int i = 0; i < PX; i++) {
                    const int32_t x = wi.x0 + i * tpr + lr;
                    uint32_t v = 0u;
                    if (row_in && x >= L.x && x < L.x + L.w)
                        v = src ? src[(size_t)(cy - L.y) * L.w + (x - L.x)] : init;
                    layer[i * kThreads + tid] = v;
                }
                if (tid == 0) sh.rects[depth] = make_int4(L.x, L.y, L.w, L.h);
                consumer_sync();
            } else if (c.op == CMD_POP_COMPOSITE || c.op == CMD_POP_CLIP || c.op == CMD_POP_MASK) {
                if (depth == 0) {
                    atomicOr(err, 4u);
                    sh.abort = 1;
                    break;
                }
                consumer_sync();
                depth--;
                const uint32_t *lvl = stack + (size_t)depth * kThreads * PX;
                const int4 p4 = sh.rects[depth], t = sh.rects[depth + 1];
                const bool in_child_row = cy >= t.y && cy < t.y + t.w;
                const bool in_parent_row = cy >= p4.y && cy < p4.y + p4.w;
                for (int i = 0; i < PX; i++) {
                    const int32_t x = wi.x0 + i * tpr + lr;
                    uint32_t parent = lvl[i * kThreads + tid];
                    const uint32_t child = layer[i * kThreads + tid];
                    const bool in_child = in_child_row && x >= t.x && x < t.x + t.z;
                    const bool in_parent = in_parent_row && x >= p4.x && x < p4.x + p4.z;
                    if (in_child && in_parent) {
                        if (c.op == CMD_POP_COMPOSITE) parent = dev::composite_pixel(child, parent, c.f, c.b);
                        else if (c.op == CMD_POP_CLIP) parent = dev::mask_pixel(parent, 255u - dev::ch(child, 3));
                        else parent = dev::mask_pixel(parent, dev::mask_value(child, c.b == 0));
                    }
                    layer[i * kThreads + tid] = parent;
                }
            } else if (c.op == CMD_CLEAR) {
                const int4 t = sh.rects[depth];
                const bool row_in = cy >= t.y && cy < t.y + t.w;
                for (int i = 0; i < PX; i++) {
                    const int32_t x = wi.x0 + i * tpr + lr;
                    if (row_in && x >= t.x && x < t.x + t.z) layer[i * kThreads + tid] = 0u;
                }
            } else if (c.op == CMD_END) {
                break;
            }
        }
        if (nwin) mb_arrive(&sh.mb_free[(win_base + nwin - 1u) % kWinBufs]);
        win_base += nwin;
        if (depth != 0) atomicOr(err, 8u);
        if (*(volatile int32_t *)&sh.abort == 0)
            for (int i = 0; i < PX; i++) {
                const int32_t x = wi.x0 + i * tpr + lr;
                if (row_ok && x < wi.x1) *(uint32_t *)(out + (size_t)cy * st.out_stride + 4 * (size_t)x) = layer[i * kThreads + tid];
            }
        consumer_sync();  // every consumer is done with the item copy and the layer stack
    }
}

// launch arguments of the failure-detection controls (read at launch time; a
// captured graph keeps the values it was captured with)
constexpr uint32_t kDefaultWaitLimit = 1u << 22;
uint32_t g_wait_limit = kDefaultWaitLimit;
uint32_t g_withhold = 0;

}  // namespace

size_t raster_smem_bytes_px(int px) { return ((sizeof(VmShared) + 15) & ~(size_t)15) + (size_t)kThreads * px * 4; }
size_t raster_smem_bytes() { return raster_smem_bytes_px(16); }
size_t raster_stack_words_per_cta(int px) { return (size_t)kMaxDepth * kThreads * px; }
int raster_threads() { return kThreads; }
int raster_max_pairs() { return kMaxPairs; }
int raster_window_buffers() { return (int)kWinBufs; }

cudaError_t raster_init() {
    return cudaFuncSetAttribute(k_raster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)raster_smem_bytes_px(16));
}

cudaError_t launch_raster(int px, uint32_t grid, uint32_t stack_depth, const StreamRec *streams, const WorkItem *items,
                          uint32_t nitems, uint32_t *item_counter, const Cmd *cmds, const uint32_t *fill_cmds, const DrawRec *draws,
                          const PaintRec *paints, const GradRec *grads, const LayerRec *layers, const EdgeRec *bins,
                          const uint32_t *bin_offsets, const uint32_t *bin_counts, uint32_t *stack, int2 *span_ovf,
                          uint32_t ovf_cap, int2 *run_ovf, uint32_t run_ovf_cap, const HairRec *hairs, const HairSpan *hair_spans, uint32_t *err,
                          cudaStream_t s) {
    k_raster<<<grid, kBlock, raster_smem_bytes_px(px), s>>>(px, streams, items, nitems, item_counter, cmds, fill_cmds, draws, paints,
                                                              grads, layers, bins, bin_offsets, bin_counts, stack,
                                                              stack_depth, span_ovf, ovf_cap, run_ovf, run_ovf_cap, hairs,
                                                              hair_spans, err, g_wait_limit, g_withhold);
    return cudaGetLastError();
}

void raster_set_wait_limit(uint32_t rounds) { g_wait_limit = rounds ? rounds : kDefaultWaitLimit; }
uint32_t raster_wait_limit() { return g_wait_limit; }
void raster_set_withhold(bool on) { g_withhold = on ? 1u : 0u; }

int raster_max_blocks_per_sm(int px) {
    int n = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster, kBlock, raster_smem_bytes_px(px));
    if (e != cudaSuccess || n < 1) { cudaGetLastError(); n = 1; }
    return n;
}

}  // namespace rgpu
