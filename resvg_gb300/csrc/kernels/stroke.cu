// Device-side stroking: tiny-skia's Path::stroke (stroke_core.h, the same
// source the host compiles) run by one thread per stroked path.
//
//   k_stroke  thread/job: build the source path's segments (auto-close), run
//             the stroker into the job's outline slice, write the outline's
//             verb and point counts into its DrawRec
//   k_draw_sizes / scans: segment-slot and transformed-point bases per draw
//             (a stroke outline's size is known only on the device)
//
// A job's builders live in fixed slices of device memory: the outline in the
// stroke arrays, the inner offset path and the cusp circles in scratch
// arrays twice that size.  The outline only grows while it is built and the
// inner path and cusp circles are copied into it, so a slice as large as the
// finished outline holds every builder.  A builder that outgrows its slice
// stops writing, raises the job's status word and keeps counting; the host
// then gives that job a larger slice and strokes it again.
#include <cuda_runtime.h>
#include <stdint.h>
#include "kernels.h"
#include "../host/dash_core.h"

namespace rgpu {
namespace {

// std::vector-like storage over a fixed slice (writes past the end are
// dropped and flagged; reads are clamped into the slice)
template <class T> struct SliceVec {
    T *p = nullptr;
    uint32_t n = 0, cap = 0;
    uint32_t *ovf = nullptr;
    __host__ __device__ size_t size() const { return n; }
    __host__ __device__ bool empty() const { return n == 0; }
    __host__ __device__ void clear() { n = 0; }
    __host__ __device__ void push_back(const T &v) {
        if (n < cap) p[n] = v;
        else *ovf = 1u;
        n++;
    }
    __host__ __device__ T &back() { return p[n == 0 ? 0 : (n <= cap ? n : cap) - 1]; }
    __host__ __device__ const T &back() const { return p[n == 0 ? 0 : (n <= cap ? n : cap) - 1]; }
    __host__ __device__ T &operator[](size_t i) { return p[i < cap ? i : cap - 1]; }
    __host__ __device__ const T &operator[](size_t i) const { return p[i < cap ? i : cap - 1]; }
};

struct SliceTraits {
    template <class T> using Vec = SliceVec<T>;
};
using DevStroker = sk::StrokerT<SliceTraits>;

// Device-side arrays a stroke job works in (the job holds its slices).
struct StrokeArrays {
    const uint8_t *src_verbs;
    const float *src_pts;
    const float *dashes;
    uint8_t *out_verbs;
    float *out_pts;
    uint8_t *scr_verbs;   // inner offset path + cusp circles: twice the outline slice
    float *scr_pts;
    sk::Seg *segs;
    uint8_t *dash_verbs;  // the dashed path
    float *dash_pts;
    sk::MSeg *msegs;      // one measured contour
    float *mpts;
    DrawRec *draws;
    uint32_t *status;
};

template <class T> __device__ __forceinline__ void bind_vec(SliceVec<T> &v, T *p, uint32_t cap, uint32_t *ovf) {
    v.p = p;
    v.cap = cap;
    v.ovf = ovf;
    v.n = 0;
}

__global__ void __launch_bounds__(128) k_stroke(const StrokeJob *jobs, uint32_t njobs, StrokeArrays a) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    const StrokeJob jb = jobs[j];
    uint32_t ovf = 0;
    uint32_t nv = 0, np = 0;
    // slices of at least one entry: the builders' back() needs one
    if (jb.verb_cap > 0 && jb.pt_cap > 0) {
        // the path to stroke: the source, or its dashed copy (dash.rs)
        const uint8_t *pv = a.src_verbs + jb.src_verb_off;
        const float *pp = a.src_pts + 2 * (size_t)jb.src_pt_off;
        size_t pnv = jb.src_verb_cnt;
        bool any = true;
        if (jb.dash_cnt > 0 && jb.dverb_cap > 0 && jb.dpt_cap > 0 && jb.mseg_cap > 0 && jb.mpt_cap > 0) {
            sk::ContourT<SliceTraits> c;
            bind_vec(c.segs, a.msegs + jb.mseg_off, jb.mseg_cap, &ovf);
            bind_vec(c.pts, reinterpret_cast<sk::Pt *>(a.mpts) + jb.mpt_off, jb.mpt_cap, &ovf);
            sk::BuilderT<SliceTraits> db;
            bind_vec(db.verbs, a.dash_verbs + jb.dverb_off, jb.dverb_cap, &ovf);
            bind_vec(db.pts, reinterpret_cast<sk::Pt *>(a.dash_pts) + jb.dpt_off, jb.dpt_cap, &ovf);
            const int r = sk::dash_run(pv, pnv, pp, a.dashes + jb.dash_off, jb.dash_cnt, jb.dash_phase, jb.res_scale, c,
                                       db);
            if (r == 0) {
                any = false;  // dashing left nothing, or gave up: nothing is drawn
            } else if (r > 0) {
                pv = db.verbs.p;
                pp = reinterpret_cast<const float *>(db.pts.p);
                pnv = db.verbs.n;
            }
        }
        // a path of n verbs makes at most 2n segments
        if (any && !ovf && 2 * pnv + 1 > jb.seg_cap) ovf = 1u;
        if (any && !ovf) {
            const long ns = sk::build_segments(pv, pnv, pp, a.segs + jb.seg_off);
            if (ns >= 0) {
                DevStroker skr;
                auto bind = [&](sk::BuilderT<SliceTraits> &bd, uint8_t *v, float *p) {
                    bind_vec(bd.verbs, v, jb.verb_cap, &ovf);
                    bind_vec(bd.pts, reinterpret_cast<sk::Pt *>(p), jb.pt_cap, &ovf);
                };
                bind(skr.outer, a.out_verbs + jb.verb_off, a.out_pts + 2 * (size_t)jb.pt_off);
                bind(skr.inner, a.scr_verbs + 2 * (size_t)jb.verb_off, a.scr_pts + 4 * (size_t)jb.pt_off);
                bind(skr.cusper, a.scr_verbs + 2 * (size_t)jb.verb_off + jb.verb_cap,
                     a.scr_pts + 4 * (size_t)jb.pt_off + 2 * (size_t)jb.pt_cap);
                sk::StrokeParams sp;
                sp.width = jb.width;
                sp.miter_limit = jb.miter_limit;
                sp.cap = jb.cap_join & 0xFFu;
                sp.join = jb.cap_join >> 8;
                sp.res_scale = jb.res_scale;
                if (sk::stroke_segments(skr, a.segs + jb.seg_off, (size_t)ns, sp)) {
                    nv = skr.outer.verbs.n;
                    np = skr.outer.pts.n;
                }
            }
        }
    }
    // the outline's size; after an overflow only a flag (the counts ran on
    // clamped reads) and the host grows the slices
    a.status[2 * j] = ovf ? (nv | 0x80000000u) : nv;
    a.status[2 * j + 1] = np;
    DrawRec &d = a.draws[jb.draw];
    d.verb_off = jb.verb_off;
    d.pt_off = jb.pt_off;
    d.verb_cnt = ovf ? 0u : nv;
    d.pt_cnt = ovf ? 0u : np;
}

// per draw: segment slots (verbs + 1) and transformed points, for the scans
// that place them
__global__ void k_draw_sizes(const DrawRec *draws, uint32_t ndraws, uint32_t *seg_sizes, uint32_t *tpt_sizes) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndraws) return;
    seg_sizes[d] = draws[d].verb_cnt + 1;
    tpt_sizes[d] = draws[d].pt_cnt;
}

__global__ void k_draw_bases(DrawRec *draws, uint32_t ndraws, const uint32_t *seg_base, const uint32_t *tpt_base) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndraws) return;
    draws[d].seg_base = seg_base[d];
    draws[d].tpt_base = tpt_base[d];
}

// Moves each finished outline from its sizing slice to its exact slice in
// the other pair of arrays (one warp per job) and points its DrawRec there.
__global__ void k_stroke_gather(const StrokeMove *moves, uint32_t n, const uint8_t *src_verbs, const float *src_pts,
                                uint8_t *dst_verbs, float *dst_pts, DrawRec *draws) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (w >= n) return;
    const StrokeMove m = moves[w];
    for (uint32_t i = lane; i < m.verbs; i += 32) dst_verbs[m.dst_verb + i] = src_verbs[m.src_verb + i];
    const float2 *sp = reinterpret_cast<const float2 *>(src_pts) + m.src_pt;
    float2 *dp = reinterpret_cast<float2 *>(dst_pts) + m.dst_pt;
    for (uint32_t i = lane; i < m.pts; i += 32) dp[i] = sp[i];
    if (lane == 0) {
        draws[m.draw].verb_off = m.dst_verb;
        draws[m.draw].pt_off = m.dst_pt;
    }
}

}  // namespace

size_t stroke_seg_bytes() { return sizeof(sk::Seg); }
size_t stroke_mseg_bytes() { return sizeof(sk::MSeg); }

// One launch of k_stroke over an empty job at start-up: the kernel's 6.5 KB of
// per-thread local memory is reserved then, not inside the first render.
cudaError_t stroke_warmup(cudaStream_t s) {
    void *mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, sizeof(StrokeJob) + sizeof(DrawRec) + 64);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(mem, 0, sizeof(StrokeJob) + sizeof(DrawRec) + 64, s);
    StrokeJob *job = reinterpret_cast<StrokeJob *>(mem);
    DrawRec *draw = reinterpret_cast<DrawRec *>(reinterpret_cast<char *>(mem) + sizeof(StrokeJob));
    uint32_t *status = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(mem) + sizeof(StrokeJob) + sizeof(DrawRec));
    if (e == cudaSuccess) {
        // verb_cap = 0: the thread strokes nothing and writes empty counts
        StrokeArrays a{};
        a.draws = draw;
        a.status = status;
        k_stroke<<<1, 32, 0, s>>>(job, 1, a);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(mem);
    return e != cudaSuccess ? e : e2;
}

cudaError_t launch_stroke_gather(const StrokeMove *moves, uint32_t n, const uint8_t *src_verbs, const float *src_pts,
                                 uint8_t *dst_verbs, float *dst_pts, DrawRec *draws, cudaStream_t s) {
    if (!n) return cudaSuccess;
    k_stroke_gather<<<(n + 7) / 8, 256, 0, s>>>(moves, n, src_verbs, src_pts, dst_verbs, dst_pts, draws);
    return cudaGetLastError();
}

cudaError_t launch_stroke(const StrokeJob *jobs, uint32_t njobs, const StrokeBuffers &b, cudaStream_t s) {
    if (!njobs) return cudaSuccess;
    StrokeArrays a;
    a.src_verbs = b.src_verbs;
    a.src_pts = b.src_pts;
    a.dashes = b.dashes;
    a.out_verbs = b.out_verbs;
    a.out_pts = b.out_pts;
    a.scr_verbs = b.scr_verbs;
    a.scr_pts = b.scr_pts;
    a.segs = reinterpret_cast<sk::Seg *>(b.segs);
    a.dash_verbs = b.dash_verbs;
    a.dash_pts = b.dash_pts;
    a.msegs = reinterpret_cast<sk::MSeg *>(b.msegs);
    a.mpts = b.mpts;
    a.draws = b.draws;
    a.status = b.status;
    // one warp per block: the jobs of a warp diverge, so a small pass spreads its warps over the SMs
    k_stroke<<<(njobs + 31) / 32, 32, 0, s>>>(jobs, njobs, a);
    return cudaGetLastError();
}

cudaError_t launch_draw_sizes(const DrawRec *draws, uint32_t ndraws, uint32_t *seg_sizes, uint32_t *tpt_sizes,
                              cudaStream_t s) {
    if (!ndraws) return cudaSuccess;
    k_draw_sizes<<<(ndraws + 255) / 256, 256, 0, s>>>(draws, ndraws, seg_sizes, tpt_sizes);
    return cudaGetLastError();
}

cudaError_t launch_draw_bases(DrawRec *draws, uint32_t ndraws, const uint32_t *seg_base, const uint32_t *tpt_base,
                              cudaStream_t s) {
    if (!ndraws) return cudaSuccess;
    k_draw_bases<<<(ndraws + 255) / 256, 256, 0, s>>>(draws, ndraws, seg_base, tpt_base);
    return cudaGetLastError();
}

}  // namespace rgpu
