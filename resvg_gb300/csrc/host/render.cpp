// Render orchestration and the C ABI render entry points (include/resvg_gpu.h).
//
// One submission = one SceneBuild (one or many trees, one output stream each):
// upload records and geometry, run the geometry kernels, size the edge and bin
// buffers from two device-side totals, then one persistent raster kernel over
// all work items.  Device buffers grow monotonically and are reused across
// calls; host staging is pinned.  There is no CPU rendering path: without a
// usable device the call fails with RGPU_ERR_NO_DEVICE.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include "../kernels/kernels.h"
#include "filter_exec.h"
#include "flatten.h"
#include "resvg_gpu.h"
#include "tree.h"

struct rgpu_tree : rgpu::Tree {};

namespace rgpu {
namespace {

thread_local std::string g_last_error;
thread_local std::string g_last_warning;
thread_local rgpu_stats g_stats{};

// Warnings of the current call: parts of the tree that the reference skips or
// clears with a log message (a failing filter clears its layer,
// crates/resvg/src/filter/mod.rs:343-354) while the render goes on.
void add_warning(const std::string &w) {
    if (w.empty()) return;
    if (!g_last_warning.empty()) g_last_warning += "; ";
    g_last_warning += w;
}

void set_error(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

// Failure-detection test hook: the next this-many device or pinned host
// allocations of the library fail as if memory were exhausted.
std::atomic<uint32_t> g_fail_allocs{0};
bool forced_alloc_failure() {
    uint32_t n = g_fail_allocs.load();
    while (n && !g_fail_allocs.compare_exchange_weak(n, n - 1)) {}
    return n != 0;
}

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max(bytes, (size_t)4096);
        want = want + want / 4;
        if (forced_alloc_failure()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T> T *as() const { return (T *)p; }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max(bytes, (size_t)4096) * 5 / 4;
        if (forced_alloc_failure()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

struct Tuning {
    uint32_t band_rows = 0;  // 0: automatic (the table, else a rule on the stream width)
    uint32_t px = 0;         // pixels per thread: 0 automatic, else 4/8/16
    std::vector<rgpu_tuning_entry> table;  // band rows by (stream width, stream draws) bucket
};

struct Buffers {
    DevBuf verbs, pts, draws, paints, grads, layers, cmds, streams, items;
    DevBuf tpts, segs, seg_counts, seg_offsets, scan_scratch, totals;
    DevBuf edges, edge_draw, bin_counts, bin_offsets, bins;
    DevBuf stack, span_ovf, run_ovf, err, counter, fill_cmds;
    DevBuf hairs, hair_spans;
    // device stroking: jobs, outlines, builder scratch, segment scratch,
    // per-job status, per-draw sizes and bases
    DevBuf sjobs, sverbs, spts, sscr_verbs, sscr_pts, ssegs, sstatus, dsizes, dbases;
    DevBuf sdash, sdverbs, sdpts, smsegs, smpts;  // dash intervals, dashed paths, measured contours
    DevBuf smoves;                                // the sizing run's outline moves
    std::vector<DevBuf> surf, img;   // internal surfaces (filter content/results) and filter images
    DevBuf plane;                    // f64 plane of the IIR blur
    void release() {
        DevBuf *all[] = {&verbs, &pts, &draws, &paints, &grads, &layers, &cmds, &streams, &items, &tpts, &segs,
                         &seg_counts, &seg_offsets, &scan_scratch, &totals, &edges, &edge_draw, &bin_counts,
                         &bin_offsets, &bins, &stack, &span_ovf, &run_ovf, &err, &counter, &fill_cmds, &plane, &hairs, &hair_spans,
                         &sjobs, &sverbs, &spts, &sscr_verbs, &sscr_pts, &ssegs, &sstatus, &dsizes, &dbases,
                         &sdash, &sdverbs, &sdpts, &smsegs, &smpts, &smoves};
        for (DevBuf *b : all) b->release();
        for (auto &b : surf) b.release();
        for (auto &b : img) b.release();
        surf.clear();
        img.clear();
    }
};

struct BufScratch : FilterScratch {
    Buffers &b;
    cudaError_t e = cudaSuccess;
    explicit BufScratch(Buffers &bb) : b(bb) {}
    uint32_t *image(uint32_t idx, size_t pixels) override {
        if (b.img.size() <= idx) b.img.resize(idx + 1);
        cudaError_t x = b.img[idx].ensure(pixels * 4);
        if (x != cudaSuccess) e = x;
        return b.img[idx].as<uint32_t>();
    }
    double *plane(size_t n) override {
        cudaError_t x = b.plane.ensure(n * 8);
        if (x != cudaSuccess) e = x;
        return b.plane.as<double>();
    }
};

// rgpu_render_batch pipelines batches of at least this many scenes in this many chunks.
constexpr uint32_t kPipeMinScenes = 64;
constexpr uint32_t kPipeChunks = 8;

// A flattened submission with its work decomposition.
constexpr uint32_t kSpanOvf = 64;  // spans one sub-scanline of one draw may hold in the raster kernel

struct Plan {
    SceneBuild sb;
    std::vector<WorkItem> items;
    std::vector<uint32_t> level_off, level_cnt;  // work items per dependency level
    uint32_t px = 8;
    uint64_t nbins = 0;
    uint32_t max_depth = 1;
    uint32_t grid = 1;
    uint32_t run_cap = 0;              // alpha-run overflow entries per (draw, row) pair
    uint32_t nedges = 0, nbinned = 0;  // known after the first (sizing) run
    // segment slots and transformed points: the build's own counts, or with
    // device-stroked paths the device's totals (known after the sizing run)
    uint64_t nsegs = 0, ntpts = 0;
    // device stroking: per job the outline slice (verbs, points); the layout's
    // totals in the stroke arrays and the segment scratch
    std::vector<uint32_t> svcap, spcap;
    std::vector<uint32_t> sscale;  // per job: growth of its slices (1, 4, 16, ...)
    uint64_t sverbs = 0, spts = 0, ssegs = 0, sdverbs = 0, sdpts = 0, smsegs = 0, smpts = 0;
    // the outlines, their DrawRec counts and the draws' bases are in device
    // memory since the last upload: renders (and graph replays) reuse them
    bool strokes_ready = false;
    bool sized = false;
};

// CUDA events around the raster launch of each dependency level (created on
// first use); the raster time of a render is the sum over its levels.
struct RasterTimer {
    static constexpr int kPairs = 16;
    cudaEvent_t start[kPairs] = {}, stop[kPairs] = {};
    int used = 0;
    bool made = false;
    cudaError_t ensure() {
        if (made) return cudaSuccess;
        for (int k = 0; k < kPairs; k++) {
            cudaError_t e = cudaEventCreate(&start[k]);
            if (e == cudaSuccess) e = cudaEventCreate(&stop[k]);
            if (e != cudaSuccess) return e;
        }
        made = true;
        return cudaSuccess;
    }
    ~RasterTimer() {
        for (int k = 0; k < kPairs; k++) {
            if (start[k]) cudaEventDestroy(start[k]);
            if (stop[k]) cudaEventDestroy(stop[k]);
        }
    }
};

// One stage of rgpu_render_batch's pipeline: while the device renders the
// chunk in one slot, the host flattens and uploads the next into the other.
struct PipeSlot {
    Buffers buf;
    HostBuf staging;
    RasterTimer timer;
    cudaEvent_t done = nullptr;  // the slot's uploads and kernels have run
};

struct Context {
    std::mutex mu;
    int device = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    RasterTimer timer;
    Buffers buf;
    DevBuf surface;
    HostBuf staging;
    Tuning tuning;
    PipeSlot pipe[2];
    HostBuf pipe_err;            // error words of the pipelined chunks, read back asynchronously
    uint32_t batch_chunks = 0;   // 0: automatic; else the chunk count of rgpu_render_batch
};

Context &ctx() {
    static Context c;
    return c;
}

// Outline-cache writebacks run on their own threads while the device works
// on; every render entry point joins them before it returns (so a tree is
// never written after the call that stroked it).
std::mutex g_wb_mu;
std::vector<std::thread> g_writebacks;
void join_writebacks() {
    std::vector<std::thread> ts;
    {
        std::lock_guard<std::mutex> g(g_wb_mu);
        ts.swap(g_writebacks);
    }
    for (auto &t : ts) t.join();
}
struct WritebackJoin {
    ~WritebackJoin() { join_writebacks(); }
};

#define CK(expr)                                                                                  \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            set_error("%s: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, __LINE__);       \
            return _e == cudaErrorMemoryAllocation ? RGPU_ERR_OUT_OF_MEMORY : RGPU_ERR_CUDA;     \
        }                                                                                         \
    } while (0)

int ensure_device(Context &c) {
    if (c.device >= 0) return RGPU_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return RGPU_ERR_NO_DEVICE;
    }
    int dev = 0;
    CK(cudaSetDevice(dev));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, dev));
    if (prop.major < 10) {
        set_error("device %s (sm_%d%d) is not a Blackwell GPU; this build targets sm_103a", prop.name, prop.major,
                  prop.minor);
        return RGPU_ERR_NO_DEVICE;
    }
    c.sms = prop.multiProcessorCount;
    CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    CK(raster_init());
    CK(stroke_warmup(c.stream));
    c.device = dev;
    return RGPU_OK;
}

template <class T>
int upload(HostBuf &staging, DevBuf &d, const std::vector<T> &v, size_t &stage_off, cudaStream_t s) {
    size_t bytes = v.size() * sizeof(T);
    CK(d.ensure(bytes ? bytes : 16));
    if (!bytes) return RGPU_OK;
    std::memcpy((char *)staging.p + stage_off, v.data(), bytes);
    CK(cudaMemcpyAsync(d.p, (char *)staging.p + stage_off, bytes, cudaMemcpyHostToDevice, s));
    stage_off += (bytes + 255) & ~(size_t)255;
    g_stats.h2d_bytes += bytes;
    return RGPU_OK;
}

uint32_t pick_px(const SceneBuild &sb, const Tuning &tu) {
    if (tu.px) return tu.px;
    int32_t maxw = 0;
    for (auto &s : sb.streams) maxw = std::max(maxw, s.out_w);
    return maxw <= 512 ? 4 : (maxw <= 1024 ? 8 : 16);
}
uint32_t pick_bh(int32_t w, uint32_t draws, uint32_t px, const Tuning &tu) {
    if (tu.band_rows) return tu.band_rows;
    for (const auto &e : tu.table)
        if ((uint32_t)w <= e.max_width && draws <= e.max_draws) {
            if (e.band_rows) return e.band_rows;
            break;
        }
    uint32_t bh = 1;
    while (bh < 8 && (256 / (bh * 2)) * px >= (uint32_t)w) bh *= 2;
    return bh;
}

// Host-side work decomposition of a flattened submission.
// First slice sizes of a job at growth `sc`: outlines measured on the
// benchmark scenes average 15 verbs and 12 points per source verb and point
// (at most 29 and 24); a dashed path is sized from the source too, and its
// outline from the dashed path.  A job that outgrows a slice is given four
// times the room by the sizing run.
void first_slices(const StrokeJob &j, uint32_t sc, uint32_t *vcap, uint32_t *pcap) {
    uint64_t v = 32ull * j.src_verb_cnt + 64, q = 32ull * j.src_pt_cnt + 128;
    if (j.dash_cnt) {
        v = 16ull * (64ull * j.src_verb_cnt + 256);
        q = 16ull * (64ull * j.src_pt_cnt + 512);
    }
    *vcap = (uint32_t)std::min<uint64_t>(v * sc, 0x10000000ull);
    *pcap = (uint32_t)std::min<uint64_t>(q * sc, 0x10000000ull);
}

// Places each stroke job's slices (outline: p.svcap / p.spcap; the rest from
// the job's growth p.sscale) in the stroke arrays.
int layout_strokes(Plan &p) {
    uint64_t v = 0, q = 0, g = 0, dv = 0, dq = 0, ms = 0, mq = 0;
    auto &jobs = p.sb.stroke_jobs;
    for (size_t i = 0; i < jobs.size(); i++) {
        StrokeJob &j = jobs[i];
        const uint64_t sc = p.sscale[i];
        j.verb_off = (uint32_t)v;
        j.verb_cap = p.svcap[i];
        j.pt_off = (uint32_t)q;
        j.pt_cap = p.spcap[i];
        uint64_t seg_cap = 2ull * j.src_verb_cnt + 1;
        j.dverb_off = (uint32_t)dv; j.dpt_off = (uint32_t)dq;
        j.mseg_off = (uint32_t)ms; j.mpt_off = (uint32_t)mq;
        j.dverb_cap = j.dpt_cap = j.mseg_cap = j.mpt_cap = 0;
        if (j.dash_cnt) {
            j.dverb_cap = (uint32_t)std::min<uint64_t>((64ull * j.src_verb_cnt + 256) * sc, 0x10000000ull);
            j.dpt_cap = (uint32_t)std::min<uint64_t>((64ull * j.src_pt_cnt + 512) * sc, 0x10000000ull);
            j.mseg_cap = (uint32_t)std::min<uint64_t>((64ull * j.src_verb_cnt + 64) * sc, 0x10000000ull);
            j.mpt_cap = j.src_pt_cnt + 2;  // a contour's points and its closing point
            seg_cap = std::max<uint64_t>(seg_cap, 2ull * j.dverb_cap + 1);
        }
        j.seg_off = (uint32_t)g;
        j.seg_cap = (uint32_t)seg_cap;
        v += j.verb_cap;
        q += j.pt_cap;
        g += seg_cap;
        dv += j.dverb_cap;
        dq += j.dpt_cap;
        ms += j.mseg_cap;
        mq += j.mpt_cap;
        if (v > 0x7FFFFFFFull || q > 0x3FFFFFFFull || g > 0x7FFFFFFFull || dv > 0x7FFFFFFFull ||
            dq > 0x3FFFFFFFull || ms > 0x3FFFFFFFull || mq > 0x3FFFFFFFull) {
            set_error("stroke outlines exceed the stroke arrays' index range");
            return RGPU_ERR_CAPACITY;
        }
    }
    p.sverbs = v;
    p.spts = q;
    p.ssegs = g;
    p.sdverbs = dv;
    p.sdpts = dq;
    p.smsegs = ms;
    p.smpts = mq;
    return RGPU_OK;
}

int plan_scene(Context &c, Plan &p) {
    SceneBuild &sb = p.sb;
    if (sb.stroke_jobs.empty()) {
        p.nsegs = sb.nsegs;
        p.ntpts = sb.ntpts;
    }
    if (!sb.stroke_jobs.empty() && p.svcap.size() != sb.stroke_jobs.size()) {
        // one thread strokes one path, so the 32 paths of a warp run in step
        // only as far as their control flow agrees: order the jobs by source
        // verb count and cap / join (each keeps its draw and cache entry)
        {
            const size_t nj = sb.stroke_jobs.size();
            std::vector<uint32_t> ord(nj);
            for (size_t i = 0; i < nj; i++) ord[i] = (uint32_t)i;
            auto key = [&](uint32_t i) {
                const StrokeJob &j = sb.stroke_jobs[i];
                return ((uint64_t)j.src_verb_cnt << 32) | j.cap_join;
            };
            std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return key(a) < key(b); });
            std::vector<StrokeJob> jobs(nj);
            for (size_t i = 0; i < nj; i++) jobs[i] = sb.stroke_jobs[ord[i]];
            sb.stroke_jobs.swap(jobs);
            if (sb.stroke_keys.size() == nj) {
                std::vector<StrokeKey> keys(nj);
                for (size_t i = 0; i < nj; i++) keys[i] = sb.stroke_keys[ord[i]];
                sb.stroke_keys.swap(keys);
            }
        }
        // first slices: outlines measured on the benchmark scenes average 15
        // verbs and 12 points per source verb and point (at most 29 and 24);
        // a larger outline is given a larger slice by the sizing run
        p.svcap.resize(sb.stroke_jobs.size());
        p.spcap.resize(sb.stroke_jobs.size());
        p.sscale.assign(sb.stroke_jobs.size(), 1u);
        for (size_t i = 0; i < sb.stroke_jobs.size(); i++) first_slices(sb.stroke_jobs[i], 1, &p.svcap[i], &p.spcap[i]);
        p.sized = false;
    }
    if (!sb.stroke_jobs.empty()) {
        int r = layout_strokes(p);
        if (r) return r;
    }
    p.px = pick_px(sb, c.tuning);
    p.items.clear();
    p.nbins = 0;
    p.max_depth = 1;
    sb.fill_cmds.clear();
    for (uint32_t si = 0; si < sb.streams.size(); si++) {
        StreamRec &st = sb.streams[si];
        // the raster kernel's phase-A windows take the stream's fill commands in order
        st.fill_off = (uint32_t)sb.fill_cmds.size();
        for (uint32_t ci = 0; ci < st.cmd_cnt; ci++) {
            const uint32_t op = sb.cmds[st.cmd_off + ci].op;
            if (op == CMD_FILL || op == CMD_APPLY_REGION) sb.fill_cmds.push_back(ci);
        }
        st.fill_cnt = (uint32_t)sb.fill_cmds.size() - st.fill_off;
        uint32_t bh = pick_bh(st.out_w, st.draw_cnt, p.px, c.tuning);
        st.band_rows = bh;
        st.nbands = (uint32_t)((st.out_h + (int32_t)bh - 1) / (int32_t)bh);
        st.bin_off = (uint32_t)p.nbins;
        p.nbins += (uint64_t)st.nbands * st.draw_cnt;
        p.max_depth = std::max(p.max_depth, st.max_depth + 1);
    }
    p.level_off.assign(sb.max_level + 1, 0);
    p.level_cnt.assign(sb.max_level + 1, 0);
    for (uint32_t lv = 0; lv <= sb.max_level; lv++) {
        p.level_off[lv] = (uint32_t)p.items.size();
        for (uint32_t si = 0; si < sb.streams.size(); si++) {
            const StreamRec &st = sb.streams[si];
            if (st.level != lv) continue;
            int32_t cw = (int32_t)((256 / st.band_rows) * p.px);
            for (uint32_t b = 0; b < st.nbands; b++)
                for (int32_t x0 = 0; x0 < st.out_w; x0 += cw)
                    p.items.push_back(WorkItem{si, b, x0, std::min(x0 + cw, st.out_w)});
        }
        p.level_cnt[lv] = (uint32_t)p.items.size() - p.level_off[lv];
        // the persistent kernel takes items in order: heaviest first (draws x
        // pixels) shortens the tail when scenes of very different cost share
        // a launch
        auto cost = [&](const WorkItem &it) {
            const StreamRec &st = sb.streams[it.stream];
            return (uint64_t)st.draw_cnt * (uint64_t)(it.x1 - it.x0) * st.band_rows;
        };
        std::stable_sort(p.items.begin() + p.level_off[lv], p.items.end(),
                         [&](const WorkItem &a, const WorkItem &b) { return cost(a) > cost(b); });
    }
    if (p.nbins > 0xF0000000ull) { set_error("too many (band, draw) bins"); return RGPU_ERR_CAPACITY; }
    // a pair's runs cover at most its work item's width, one entry per pixel
    // step, or two per aliased span (kSpanOvf spans a scanline at most)
    uint32_t item_w = 0;
    for (const auto &st : sb.streams) item_w = std::max(item_w, (256 / st.band_rows) * p.px);
    p.run_cap = std::max(item_w, 2 * kSpanOvf) + 2;
    uint32_t per_sm = (uint32_t)raster_max_blocks_per_sm((int)p.px);
    p.grid = std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)p.items.size(), (uint32_t)c.sms * per_sm));
    return RGPU_OK;
}

int ensure_stroke_buffers(Buffers &b, Plan &p) {
    if (p.sb.stroke_jobs.empty()) return RGPU_OK;
    const size_t nd = p.sb.draws.size();
    CK(b.sverbs.ensure(std::max<uint64_t>(p.sverbs, 1)));
    CK(b.spts.ensure(std::max<uint64_t>(p.spts, 1) * 8));
    CK(b.sscr_verbs.ensure(std::max<uint64_t>(2 * p.sverbs, 1)));
    CK(b.sscr_pts.ensure(std::max<uint64_t>(2 * p.spts, 1) * 8));
    CK(b.ssegs.ensure(std::max<uint64_t>(p.ssegs, 1) * stroke_seg_bytes()));
    CK(b.sdash.ensure(std::max<size_t>(p.sb.dashes.size(), 1) * 4));
    CK(b.sdverbs.ensure(std::max<uint64_t>(p.sdverbs, 1)));
    CK(b.sdpts.ensure(std::max<uint64_t>(p.sdpts, 1) * 8));
    CK(b.smsegs.ensure(std::max<uint64_t>(p.smsegs, 1) * stroke_mseg_bytes()));
    CK(b.smpts.ensure(std::max<uint64_t>(p.smpts, 1) * 8));
    CK(b.sstatus.ensure(p.sb.stroke_jobs.size() * 8));
    CK(b.dsizes.ensure((nd + 1) * 8));
    CK(b.dbases.ensure((nd + 1) * 8));
    return RGPU_OK;
}

int ensure_segment_buffers(Buffers &b, Plan &p) {
    const uint64_t nsegs = p.nsegs;
    CK(b.tpts.ensure(std::max<uint64_t>(p.ntpts, 1) * 8));
    CK(b.segs.ensure(std::max<uint64_t>(nsegs, 1) * sizeof(SegRec)));
    CK(b.seg_counts.ensure((nsegs + 1) * 4));
    CK(b.seg_offsets.ensure((nsegs + 1) * 4));
    CK(b.scan_scratch.ensure(scan_scratch_words(std::max<uint64_t>({nsegs + 1, p.nbins + 1, p.sb.draws.size() + 1})) * 4));
    return RGPU_OK;
}

// One device stroking pass: every job's outline into its slice (the counts
// into its DrawRec), then the per-draw segment and point bases.
int stroke_pass(Buffers &b, Plan &p, cudaStream_t s) {
    SceneBuild &sb = p.sb;
    const uint32_t nj = (uint32_t)sb.stroke_jobs.size(), nd = (uint32_t)sb.draws.size();
    uint32_t *totals = b.totals.as<uint32_t>();
    uint32_t *sz = b.dsizes.as<uint32_t>(), *bs = b.dbases.as<uint32_t>();
    StrokeBuffers sbuf;
    sbuf.src_verbs = b.verbs.as<uint8_t>();
    sbuf.src_pts = b.pts.as<float>();
    sbuf.dashes = b.sdash.as<float>();
    sbuf.out_verbs = b.sverbs.as<uint8_t>();
    sbuf.out_pts = b.spts.as<float>();
    sbuf.scr_verbs = b.sscr_verbs.as<uint8_t>();
    sbuf.scr_pts = b.sscr_pts.as<float>();
    sbuf.segs = b.ssegs.p;
    sbuf.dash_verbs = b.sdverbs.as<uint8_t>();
    sbuf.dash_pts = b.sdpts.as<float>();
    sbuf.msegs = b.smsegs.p;
    sbuf.mpts = b.smpts.as<float>();
    sbuf.draws = b.draws.as<DrawRec>();
    sbuf.status = b.sstatus.as<uint32_t>();
    CK(launch_stroke(b.sjobs.as<StrokeJob>(), nj, sbuf, s));
    CK(launch_draw_sizes(b.draws.as<DrawRec>(), nd, sz, sz + (nd + 1), s));
    CK(launch_exclusive_scan(sz, bs, nd, b.scan_scratch.as<uint32_t>(), totals + 2, s));
    CK(launch_exclusive_scan(sz + (nd + 1), bs + (nd + 1), nd, b.scan_scratch.as<uint32_t>(), totals + 3, s));
    CK(launch_draw_bases(b.draws.as<DrawRec>(), nd, bs, bs + (nd + 1), s));
    g_stats.kernel_launches += 5;
    return RGPU_OK;
}

// Copies the outlines the device built into their trees' outline caches, so
// that flattening the same trees again reuses them instead of new jobs.
int cache_outlines(Buffers &b, Plan &p, cudaStream_t s) {
    SceneBuild &sb = p.sb;
    const size_t nj = sb.stroke_jobs.size();
    if (sb.stroke_keys.size() != nj) return RGPU_OK;
    auto hv = std::make_shared<std::vector<uint8_t>>(p.sverbs);
    auto hp = std::make_shared<std::vector<float>>(2 * p.spts);
    if (p.sverbs) CK(cudaMemcpyAsync(hv->data(), b.sverbs.p, p.sverbs, cudaMemcpyDeviceToHost, s));
    if (p.spts) CK(cudaMemcpyAsync(hp->data(), b.spts.p, p.spts * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    g_stats.d2h_bytes += p.sverbs + p.spts * 8;
    // the slices and keys the inserts need, copied: the plan lives on
    struct Slice { uint32_t vo, vn, po, pn; };
    auto slices = std::make_shared<std::vector<Slice>>(nj);
    auto keys = std::make_shared<std::vector<StrokeKey>>(sb.stroke_keys);
    for (size_t j = 0; j < nj; j++) {
        const StrokeJob &jb = sb.stroke_jobs[j];
        (*slices)[j] = Slice{jb.verb_off, jb.verb_cap, jb.pt_off, jb.pt_cap};
    }
    auto store = [hv, hp, slices, keys](size_t a, size_t e) {
        for (size_t j = a; j < e; j++) {
            const Slice &sl = (*slices)[j];
            std::shared_ptr<PathData> out;
            if (sl.vn > 1) {
                out = std::make_shared<PathData>();
                out->verbs.assign(hv->begin() + sl.vo, hv->begin() + sl.vo + sl.vn);
                out->pts.assign(hp->begin() + 2 * (size_t)sl.po, hp->begin() + 2 * ((size_t)sl.po + sl.pn));
            }
            const StrokeKey &k = (*keys)[j];
            k.tree->store_stroke_outline(k.path, k.res_scale, std::move(out));
        }
    };
    // contiguous ranges: a tree's jobs are adjacent, so threads rarely share a cache
    const size_t nt = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency() / 2), nj / 4096 + 1);
    std::lock_guard<std::mutex> g(g_wb_mu);
    for (size_t k = 0; k < nt; k++) g_writebacks.emplace_back(store, nj * k / nt, nj * (k + 1) / nt);
    return RGPU_OK;
}

// Device stroking with the sizing run: outlines that outgrow their slice are
// stroked again with four times the room until all fit, then every slice is
// cut to its outline's exact size and the outlines are built once more in
// that layout, which later renders (and graph replays) reuse.
int run_strokes(Buffers &b, Plan &p, cudaStream_t s) {
    int r;
    if (p.sized) return stroke_pass(b, p, s);
    SceneBuild &sb = p.sb;
    const size_t nj = sb.stroke_jobs.size();
    std::vector<uint32_t> st(2 * nj);
    auto reupload = [&]() -> int {
        int rr = layout_strokes(p);
        if (rr) return rr;
        if ((rr = ensure_stroke_buffers(b, p))) return rr;
        CK(b.sjobs.ensure(nj * sizeof(StrokeJob)));
        CK(cudaMemcpyAsync(b.sjobs.p, sb.stroke_jobs.data(), nj * sizeof(StrokeJob), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        return RGPU_OK;
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const bool timed = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    for (int round = 0;; round++) {
        if (timed && round == 0) CK(cudaEventRecord(e0, s));
        if ((r = stroke_pass(b, p, s))) return r;
        if (timed && round == 0) CK(cudaEventRecord(e1, s));
        CK(cudaMemcpyAsync(st.data(), b.sstatus.p, nj * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        bool grow = false;
        for (size_t j = 0; j < nj; j++)
            if (st[2 * j] & 0x80000000u) {
                grow = true;
                p.sscale[j] = (uint32_t)std::min<uint64_t>(4ull * p.sscale[j], 1u << 24);
                first_slices(sb.stroke_jobs[j], p.sscale[j], &p.svcap[j], &p.spcap[j]);
            }
        if (!grow) break;
        if (round >= 6) {
            set_error("a stroke outline outgrew its slice after repeated growth");
            return RGPU_ERR_CAPACITY;
        }
        if ((r = reupload())) return r;
    }
    // every outline fits: move each to a slice of its exact size in the
    // scratch arrays, which then become the outline arrays
    std::vector<StrokeMove> moves(nj);
    for (size_t j = 0; j < nj; j++) {
        moves[j].src_verb = sb.stroke_jobs[j].verb_off;
        moves[j].src_pt = sb.stroke_jobs[j].pt_off;
        moves[j].verbs = st[2 * j];
        moves[j].pts = st[2 * j + 1];
        moves[j].draw = sb.stroke_jobs[j].draw;
        p.svcap[j] = st[2 * j];
        p.spcap[j] = st[2 * j + 1];
    }
    if ((r = layout_strokes(p))) return r;
    for (size_t j = 0; j < nj; j++) {
        moves[j].dst_verb = sb.stroke_jobs[j].verb_off;
        moves[j].dst_pt = sb.stroke_jobs[j].pt_off;
    }
    CK(b.smoves.ensure(nj * sizeof(StrokeMove)));
    // pageable sources: the copies are staged before the calls return
    CK(cudaMemcpyAsync(b.smoves.p, moves.data(), nj * sizeof(StrokeMove), cudaMemcpyHostToDevice, s));
    CK(launch_stroke_gather(b.smoves.as<StrokeMove>(), (uint32_t)nj, b.sverbs.as<uint8_t>(), b.spts.as<float>(),
                            b.sscr_verbs.as<uint8_t>(), b.sscr_pts.as<float>(), b.draws.as<DrawRec>(), s));
    CK(cudaMemcpyAsync(b.sjobs.p, sb.stroke_jobs.data(), nj * sizeof(StrokeJob), cudaMemcpyHostToDevice, s));
    std::swap(b.sverbs, b.sscr_verbs);
    std::swap(b.spts, b.sscr_pts);
    if ((r = ensure_stroke_buffers(b, p))) return r;
    uint32_t tot[2] = {0, 0};
    CK(cudaMemcpyAsync(tot, b.totals.as<uint32_t>() + 2, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    p.nsegs = tot[0];
    p.ntpts = tot[1];
    g_stats.stroke_jobs += nj;
    if (timed) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) g_stats.stroke_ms += ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaGetLastError();
    if ((r = cache_outlines(b, p, s))) return r;
    return ensure_segment_buffers(b, p);
}

int upload_plan(Context &c, Buffers &b, Plan &p, cudaStream_t s, HostBuf *staging_buf = nullptr) {
    HostBuf &staging = staging_buf ? *staging_buf : c.staging;
    SceneBuild &sb = p.sb;
    if (b.surf.size() < sb.surfaces.size()) b.surf.resize(sb.surfaces.size());
    for (size_t i = 0; i < sb.surfaces.size(); i++) {
        CK(b.surf[i].ensure((size_t)sb.surfaces[i].w * sb.surfaces[i].h * 4));
        if (sb.surfaces[i].init)
            CK(cudaMemcpyAsync(b.surf[i].p, sb.surfaces[i].init, (size_t)sb.surfaces[i].w * sb.surfaces[i].h * 4,
                               cudaMemcpyHostToDevice, s));
    }
    for (auto &st : sb.streams)
        if (st.surface >= 0) st.out_ptr = (uint64_t)(uintptr_t)b.surf[st.surface].p;
    for (auto &L : sb.layers)
        if (L.surf >= 0) L.buf = (uint64_t)(uintptr_t)b.surf[L.surf].p;
    for (const auto &q : sb.patterns) {
        ImageRec im{(uint64_t)(uintptr_t)b.surf[q.shade].p, q.bx, q.by, q.bw, q.bh};
        std::memcpy(&sb.grads[q.grad], &im, sizeof(im));
    }
    auto rup = [](size_t n) { return (n + 255) & ~(size_t)255; };
    size_t stage = rup(sb.verbs.size()) + rup(sb.pts.size() * 4) + rup(sb.draws.size() * sizeof(DrawRec)) +
                   rup(sb.paints.size() * sizeof(PaintRec)) + rup(sb.grads.size() * sizeof(GradRec)) +
                   rup(sb.layers.size() * sizeof(LayerRec)) + rup(sb.cmds.size() * sizeof(Cmd)) +
                   rup(sb.streams.size() * sizeof(StreamRec)) + rup(p.items.size() * sizeof(WorkItem)) +
                   rup(sb.hairs.size() * sizeof(HairRec)) + rup(sb.hair_spans.size() * sizeof(HairSpan)) +
                   rup(sb.fill_cmds.size() * 4) + rup(sb.stroke_jobs.size() * sizeof(StrokeJob)) +
                   rup(sb.dashes.size() * 4) + 4096;
    CK(staging.ensure(stage));
    size_t off = 0;
    int r;
    if ((r = upload(staging, b.verbs, sb.verbs, off, s))) return r;
    if ((r = upload(staging, b.pts, sb.pts, off, s))) return r;
    if ((r = upload(staging, b.draws, sb.draws, off, s))) return r;
    if ((r = upload(staging, b.paints, sb.paints, off, s))) return r;
    if ((r = upload(staging, b.grads, sb.grads, off, s))) return r;
    if ((r = upload(staging, b.layers, sb.layers, off, s))) return r;
    if ((r = upload(staging, b.cmds, sb.cmds, off, s))) return r;
    if ((r = upload(staging, b.streams, sb.streams, off, s))) return r;
    if ((r = upload(staging, b.items, p.items, off, s))) return r;
    if ((r = upload(staging, b.hairs, sb.hairs, off, s))) return r;
    if ((r = upload(staging, b.hair_spans, sb.hair_spans, off, s))) return r;
    if ((r = upload(staging, b.fill_cmds, sb.fill_cmds, off, s))) return r;
    if ((r = upload(staging, b.sjobs, sb.stroke_jobs, off, s))) return r;
    if ((r = upload(staging, b.sdash, sb.dashes, off, s))) return r;
    if ((r = ensure_stroke_buffers(b, p))) return r;
    p.strokes_ready = false;  // the draws just uploaded carry no outline counts
    // fixed-size work buffers (with device-stroked paths the segment counts
    // are the device's, so these follow the sizing run)
    if (sb.stroke_jobs.empty() || p.sized)
        if ((r = ensure_segment_buffers(b, p))) return r;
    CK(b.totals.ensure(64));
    CK(b.scan_scratch.ensure(scan_scratch_words(std::max<uint64_t>({p.nsegs + 1, p.nbins + 1, sb.draws.size() + 1})) * 4));
    CK(b.bin_counts.ensure((p.nbins + 1) * 4));
    CK(b.bin_offsets.ensure((p.nbins + 1) * 4));
    size_t stack_words = (size_t)p.max_depth * raster_threads() * p.px;
    CK(b.stack.ensure((size_t)p.grid * stack_words * 4));
    CK(b.span_ovf.ensure((size_t)p.grid * raster_threads() * kSpanOvf * 8));
    CK(b.run_ovf.ensure((size_t)p.grid * raster_window_buffers() * raster_max_pairs() * p.run_cap * 8));
    CK(b.err.ensure(16));
    CK(b.counter.ensure(4 * (sb.max_level + 1)));
    return RGPU_OK;
}

// Enqueues the device pipeline.  Without known sizes it synchronises twice to
// read the edge and bin totals; with known sizes (a prepared scene rendered
// before) it is fully asynchronous and capturable into a CUDA graph.
int enqueue_plan(Context &c, Buffers &b, Plan &p, cudaStream_t s, RasterTimer *tm) {
    SceneBuild &sb = p.sb;
    uint32_t ndraws = (uint32_t)sb.draws.size();
    if (!sb.stroke_jobs.empty() && !p.strokes_ready) {
        int r = run_strokes(b, p, s);
        if (r) return r;
        p.strokes_ready = true;
    }
    uint64_t nsegs = p.nsegs;
    uint32_t *totals = b.totals.as<uint32_t>();
    CK(launch_draw_setup(b.draws.as<DrawRec>(), ndraws, b.verbs.as<uint8_t>(), b.pts.as<float>(),
                         b.sverbs.as<uint8_t>(), b.spts.as<float>(), b.tpts.p, b.segs.as<SegRec>(), s));
    CK(cudaMemsetAsync(b.seg_counts.p, 0, (nsegs + 1) * 4, s));
    CK(launch_edges(false, b.segs.as<SegRec>(), (uint32_t)nsegs, b.draws.as<DrawRec>(), b.tpts.p,
                    b.seg_counts.as<uint32_t>(), nullptr, nullptr, nullptr, 0, s));
    CK(launch_exclusive_scan(b.seg_counts.as<uint32_t>(), b.seg_offsets.as<uint32_t>(), nsegs + 1,
                             b.scan_scratch.as<uint32_t>(), totals, s));
    if (!p.sized) {
        uint32_t tot = 0;
        CK(cudaMemcpyAsync(&tot, totals, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        p.nedges = tot;
        CK(b.edges.ensure(std::max<uint32_t>(tot, 1) * sizeof(EdgeRec)));
        CK(b.edge_draw.ensure(std::max<uint32_t>(tot, 1) * 4));
    }
    uint32_t nedges = p.nedges;
    g_stats.edges += nedges;
    CK(launch_edges(true, b.segs.as<SegRec>(), (uint32_t)nsegs, b.draws.as<DrawRec>(), b.tpts.p,
                    b.seg_counts.as<uint32_t>(), b.seg_offsets.as<uint32_t>(), b.edges.as<EdgeRec>(),
                    b.edge_draw.as<uint32_t>(), nedges, s));
    CK(launch_draw_edges(b.draws.as<DrawRec>(), ndraws, b.seg_offsets.as<uint32_t>(), s));
    CK(cudaMemsetAsync(b.bin_counts.p, 0, (p.nbins + 1) * 4, s));
    CK(launch_bin(false, b.edges.as<EdgeRec>(), b.edge_draw.as<uint32_t>(), nedges, b.draws.as<DrawRec>(),
                  b.streams.as<StreamRec>(), b.bin_counts.as<uint32_t>(), nullptr, 0, nullptr, nullptr, s));
    CK(launch_exclusive_scan(b.bin_counts.as<uint32_t>(), b.bin_offsets.as<uint32_t>(), p.nbins + 1,
                             b.scan_scratch.as<uint32_t>(), totals + 1, s));
    if (!p.sized) {
        uint32_t tot = 0;
        CK(cudaMemcpyAsync(&tot, totals + 1, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        p.nbinned = tot;
        CK(b.bins.ensure(std::max<uint32_t>(tot, 1) * sizeof(EdgeRec)));
        p.sized = true;
    }
    CK(cudaMemsetAsync(b.bin_counts.p, 0, (p.nbins + 1) * 4, s));
    CK(cudaMemsetAsync(b.err.p, 0, 4, s));
    CK(launch_bin(true, b.edges.as<EdgeRec>(), b.edge_draw.as<uint32_t>(), nedges, b.draws.as<DrawRec>(),
                  b.streams.as<StreamRec>(), b.bin_counts.as<uint32_t>(), b.bin_offsets.as<uint32_t>(), p.nbinned,
                  b.err.as<uint32_t>(), b.bins.as<EdgeRec>(), s));
    CK(cudaMemsetAsync(b.counter.p, 0, 4 * (sb.max_level + 1), s));
    for (const auto &st : sb.streams)
        if (st.surface >= 0) CK(cudaMemsetAsync(b.surf[st.surface].p, 0, (size_t)st.out_w * st.out_h * 4, s));
    BufScratch scratch(b);
    if (tm) {
        CK(tm->ensure());
        tm->used = 0;
    }
    for (uint32_t lv = 0; lv <= sb.max_level; lv++) {
        const bool timed = tm && p.level_cnt[lv] && tm->used < RasterTimer::kPairs;
        if (timed) CK(cudaEventRecord(tm->start[tm->used], s));
        if (p.level_cnt[lv])
            CK(launch_raster((int)p.px, p.grid, p.max_depth, b.streams.as<StreamRec>(),
                             b.items.as<WorkItem>() + p.level_off[lv], p.level_cnt[lv], b.counter.as<uint32_t>() + lv,
                             b.cmds.as<Cmd>(), b.fill_cmds.as<uint32_t>(), b.draws.as<DrawRec>(), b.paints.as<PaintRec>(), b.grads.as<GradRec>(),
                             b.layers.as<LayerRec>(), b.bins.as<EdgeRec>(), b.bin_offsets.as<uint32_t>(),
                             b.bin_counts.as<uint32_t>(), b.stack.as<uint32_t>(), b.span_ovf.as<int2>(), kSpanOvf,
                             b.run_ovf.as<int2>(), p.run_cap, b.hairs.as<HairRec>(), b.hair_spans.as<HairSpan>(), b.err.as<uint32_t>(), s));
        if (timed) CK(cudaEventRecord(tm->stop[tm->used++], s));
        for (const auto &q : sb.patterns) {
            if (q.level != lv) continue;
            const float inv[6] = {q.inv.sx, q.inv.ky, q.inv.kx, q.inv.sy, q.inv.tx, q.inv.ty};
            CK(filter_pattern_shade(b.surf[q.tile].as<uint32_t>(), q.tw, q.th, (float *)b.surf[q.shade].p, q.bx, q.by,
                                    q.bw, q.bh, inv, q.quality, q.repeat != 0, q.opacity, s));
        }
        for (const auto &job : sb.jobs) {
            if (job.level != lv) continue;
            std::string ferr;
            std::vector<FeImageSurface> ims;
            for (uint32_t k = 0; k < job.image_count; k++) {
                const FeImageReq &q = sb.fe_images[job.image_first + k];
                ims.push_back(FeImageSurface{q.prim, b.surf[q.surface].as<uint32_t>()});
            }
            int r = run_filter_job(job, b.surf[job.content].as<uint32_t>(), b.surf[job.result].as<uint32_t>(), scratch,
                                   s, ferr, &ims);
            if (scratch.e != cudaSuccess) CK(scratch.e);
            if (r) { set_error("filter: %s", ferr.c_str()); return r; }
            if (!ferr.empty()) add_warning("filter: " + ferr + " (layer cleared)");
        }
    }
    g_stats.draws += ndraws;
    g_stats.work_items += p.items.size();
    g_stats.kernel_launches += 13;
    return RGPU_OK;
}

int check_err(Buffers &b, cudaStream_t s, RasterTimer *tm) {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, b.err.p, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (tm && tm->used) {
        // the raster launches of every dependency level, summed
        float total = 0.0f;
        for (int k = 0; k < tm->used; k++) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, tm->start[k], tm->stop[k]) == cudaSuccess) total += ms;
        }
        g_stats.raster_ms = total;
        cudaGetLastError();  // never leave a pending error behind for the caller
    }
    if (e) {
        set_error("raster kernel reported error flags 0x%x", e);
        return RGPU_ERR_DEVICE_FAULT;
    }
    return RGPU_OK;
}

int render_host(const rgpu_tree *tree, const resvg_transform &ts, uint32_t w, uint32_t h, char *pixmap,
                int node_kind = -1, uint32_t node_index = 0) {
    g_last_error.clear();
    g_last_warning.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!tree || !pixmap || w == 0 || h == 0 || w > 32767 || h > 32767) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    WritebackJoin writebacks;  // joined before the lock is released
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = c.stream;
    size_t bytes = (size_t)w * h * 4;
    CK(c.surface.ensure(bytes));
    Plan p;
    rgpu_tree *tr = const_cast<rgpu_tree *>(tree);
    if (!tr->finalized) tr->finalize();
    const Xf xts = Xf::row(ts.a, ts.b, ts.c, ts.d, ts.e, ts.f);
    const int added = node_kind < 0 ? p.sb.add_tree(*tr, xts, (int32_t)w, (int32_t)h, (uint64_t)(uintptr_t)c.surface.p, w * 4)
                                    : p.sb.add_node(*tr, (uint32_t)node_kind, node_index, xts, (int32_t)w, (int32_t)h,
                                                    (uint64_t)(uintptr_t)c.surface.p, w * 4);
    if (added < 0) {
        set_error("%s", p.sb.error.c_str());
        return RGPU_ERR_UNSUPPORTED;
    }
    CK(c.staging.ensure(bytes));
    std::memcpy(c.staging.p, pixmap, bytes);
    CK(cudaMemcpyAsync(c.surface.p, c.staging.p, bytes, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // staging is reused for the records
    g_stats.h2d_bytes += bytes;
    if ((r = plan_scene(c, p))) return r;
    if ((r = upload_plan(c, c.buf, p, s))) return r;
    if ((r = enqueue_plan(c, c.buf, p, s, &c.timer))) return r;
    if ((r = check_err(c.buf, s, &c.timer))) return r;
    CK(c.staging.ensure(bytes));
    CK(cudaMemcpyAsync(c.staging.p, c.surface.p, bytes, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::memcpy(pixmap, c.staging.p, bytes);
    g_stats.d2h_bytes += bytes;
    return RGPU_OK;
}

}  // namespace

// Sets the calling thread's rgpu_last_error() text (for entry points in other
// translation units).
void set_last_error_message(const char *msg) { g_last_error = msg ? msg : ""; }

}  // namespace rgpu

using namespace rgpu;

extern "C" {

int rgpu_init(int device) {
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    if (device != 0) {
        set_error("only device 0 is used by this build");
        return RGPU_ERR_INVALID_ARG;
    }
    return ensure_device(c);
}

const char *rgpu_last_error(void) { return g_last_error.c_str(); }
const char *rgpu_last_warning(void) { return g_last_warning.c_str(); }

void resvg_render(const resvg_render_tree *tree, resvg_transform transform, uint32_t width, uint32_t height,
                  char *pixmap) {
    int r = render_host(tree, transform, width, height, pixmap);
    if (r != RGPU_OK) fprintf(stderr, "resvg_render: %s\n", g_last_error.c_str());
}

bool resvg_render_node(const resvg_render_tree *tree, const char *id, resvg_transform transform, uint32_t width,
                       uint32_t height, char *pixmap) {
    // resvg::render_node (crates/resvg/src/lib.rs:55-70) behind the C API's
    // id lookup (crates/c-api/lib.rs:908-942): the node's absolute layer
    // bounding box moves to the pixmap origin (transform.pre_translate(-x, -y))
    // and the node renders with only its own transform on top of that.
    g_last_error.clear();
    if (!tree || !pixmap || !width || !height) { set_error("invalid arguments"); return false; }
    if (!id || !*id) { set_error("resvg_render_node: empty id"); return false; }
    rgpu_tree *tr = const_cast<rgpu_tree *>(tree);
    if (!tr->finalized) tr->finalize();
    const rgpu_tree_view &t = *tr->get_view();
    // tree.node_by_id(id) (crates/c-api/lib.rs:931)
    uint32_t kind = 0, idx = 0;
    if (!tr->node_by_id(id, &kind, &idx)) {
        set_error("resvg_render_node: no node with id '%s'", id);
        return false;
    }
    const bool is_path = kind == RGPU_NODE_PATH;
    // parents, then the absolute transform (parent_abs.pre_concat(own))
    std::vector<int32_t> group_parent(t.group_count, -1), path_parent(t.path_count, -1);
    for (uint32_t g = 0; g < t.group_count; g++)
        for (uint32_t k = 0; k < t.groups[g].child_count; k++) {
            const rgpu_node &n = t.children[t.groups[g].child_offset + k];
            if (n.kind == RGPU_NODE_GROUP) group_parent[n.index] = (int32_t)g;
            else path_parent[n.index] = (int32_t)g;
        }
    Xf abs = is_path ? Xf() : Xf::of(t.groups[idx].transform);
    for (int32_t g = is_path ? path_parent[idx] : group_parent[idx]; g >= 0; g = group_parent[g])
        abs = concat(Xf::of(t.groups[g].transform), abs);
    float r[4];
    if (is_path) {
        const rgpu_path &p = t.paths[idx];
        r[0] = p.bbox_x; r[1] = p.bbox_y; r[2] = p.bbox_x + p.bbox_w; r[3] = p.bbox_y + p.bbox_h;
    } else {
        const rgpu_group &g = t.groups[idx];
        if (!g.has_layer_bbox) { set_error("resvg_render_node: the node has no bounding box"); return false; }
        r[0] = g.layer_x; r[1] = g.layer_y; r[2] = g.layer_x + g.layer_w; r[3] = g.layer_y + g.layer_h;
    }
    float bb[4];
    if (!(r[2] > r[0] && r[3] > r[1]) || !map_rect(abs, r[0], r[1], r[2], r[3], bb)) {
        set_error("resvg_render_node: the node has a zero-sized bounding box");
        return false;
    }
    const Xf ts = concat(Xf::row(transform.a, transform.b, transform.c, transform.d, transform.e, transform.f),
                         Xf::translate(-bb[0], -bb[1]));
    const resvg_transform rt{ts.sx, ts.ky, ts.kx, ts.sy, ts.tx, ts.ty};
    const int rr = render_host(tree, rt, width, height, pixmap, is_path ? RGPU_NODE_PATH : RGPU_NODE_GROUP,
                               (uint32_t)idx);
    if (rr != RGPU_OK) fprintf(stderr, "resvg_render_node: %s\n", g_last_error.c_str());
    return rr == RGPU_OK;
}

}  // extern "C"

// Prepared scene: flattened records resident on the device with their own
// work buffers; renders after the first are asynchronous and replay a
// captured CUDA graph.
struct rgpu_scene {
    Plan plan;
    Buffers buf;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
    cudaStream_t last_stream = nullptr;
    bool timing = false;        // un-captured renders with events around the raster kernel
    bool timed_valid = false;
    RasterTimer timer;
    ~rgpu_scene() {
        if (graph) cudaGraphExecDestroy(graph);
        buf.release();
    }
};

// Flattens a batch of trees into one SceneBuild.  Trees are flattened (and
// their strokes outlined) on host threads, in contiguous chunks that are then
// appended in order, so the records equal a one-thread flatten of the batch.
static int build_batch(Plan &p, const resvg_render_tree *const *trees, const resvg_transform *transforms,
                       uint32_t count, const uint32_t *widths, const uint32_t *heights, uint8_t *const *ptrs,
                       const uint32_t *strides) {
    for (uint32_t i = 0; i < count; i++) {
        rgpu_tree *tr = const_cast<rgpu_tree *>(trees[i]);
        if (!tr || !ptrs[i] || !widths[i] || !heights[i] || widths[i] > 32767 || heights[i] > 32767) {
            set_error("invalid batch entry %u", i);
            return RGPU_ERR_INVALID_ARG;
        }
        uint32_t stride = strides ? strides[i] : widths[i] * 4;
        if (stride < widths[i] * 4) { set_error("invalid stride for entry %u", i); return RGPU_ERR_INVALID_ARG; }
        // finalised here, on one thread: the flatten threads only read trees
        if (!tr->finalized) tr->finalize();
    }
    auto flatten_range = [&](SceneBuild &sb, uint32_t a, uint32_t b, uint32_t *failed) {
        for (uint32_t i = a; i < b; i++) {
            rgpu_tree *tr = const_cast<rgpu_tree *>(trees[i]);
            const resvg_transform &ts = transforms[i];
            const uint32_t stride = strides ? strides[i] : widths[i] * 4;
            if (sb.add_tree(*tr, Xf::row(ts.a, ts.b, ts.c, ts.d, ts.e, ts.f), (int32_t)widths[i], (int32_t)heights[i],
                            (uint64_t)(uintptr_t)ptrs[i], stride) < 0) {
                *failed = i;
                return false;
            }
        }
        return true;
    };
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t nthreads = std::min<uint32_t>(hw, 64);
    if (count < 16 || nthreads == 1) {
        uint32_t failed = 0;
        if (!flatten_range(p.sb, 0, count, &failed)) {
            set_error("entry %u: %s", failed, p.sb.error.c_str());
            return RGPU_ERR_UNSUPPORTED;
        }
        return RGPU_OK;
    }
    const uint32_t nchunks = std::min<uint32_t>(count, 8 * nthreads);
    std::vector<SceneBuild> parts(nchunks);
    std::vector<uint32_t> fail_at(nchunks, UINT32_MAX);
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        for (;;) {
            const uint32_t c = next.fetch_add(1);
            if (c >= nchunks) return;
            const uint32_t a = (uint32_t)((uint64_t)count * c / nchunks), b = (uint32_t)((uint64_t)count * (c + 1) / nchunks);
            uint32_t failed = 0;
            if (!flatten_range(parts[c], a, b, &failed)) fail_at[c] = failed;
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t k = 1; k < std::min(nthreads, nchunks); k++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    for (uint32_t c = 0; c < nchunks; c++)
        if (fail_at[c] != UINT32_MAX) {
            set_error("entry %u: %s", fail_at[c], parts[c].error.c_str());
            return RGPU_ERR_UNSUPPORTED;
        }
    p.sb.merge(parts, nthreads);
    return RGPU_OK;
}

extern "C" {

int rgpu_render_device(const resvg_render_tree *tree, resvg_transform ts, uint32_t w, uint32_t h,
                       uint8_t *device_pixmap, uint32_t stride, void *stream) {
    g_last_error.clear();
    g_last_warning.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!tree || !device_pixmap || w == 0 || h == 0 || stride < w * 4) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    WritebackJoin writebacks;  // joined before the lock is released
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    Plan p;
    if ((r = build_batch(p, &tree, &ts, 1, &w, &h, &device_pixmap, &stride))) return r;
    if ((r = plan_scene(c, p))) return r;
    if ((r = upload_plan(c, c.buf, p, s))) return r;
    if ((r = enqueue_plan(c, c.buf, p, s, &c.timer))) return r;
    return check_err(c.buf, s, &c.timer);
}

int rgpu_render_batch(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                      const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps, void *stream) {
    g_last_error.clear();
    g_last_warning.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!trees || !transforms || !widths || !heights || !device_pixmaps) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    WritebackJoin writebacks;  // joined before the lock is released
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    uint32_t nch = c.batch_chunks ? c.batch_chunks : (count >= kPipeMinScenes ? kPipeChunks : 1u);
    nch = std::min(nch, count);
    if (nch <= 1) {
        Plan p;
        if ((r = build_batch(p, trees, transforms, count, widths, heights, device_pixmaps, nullptr))) return r;
        if ((r = plan_scene(c, p))) return r;
        if ((r = upload_plan(c, c.buf, p, s))) return r;
        if ((r = enqueue_plan(c, c.buf, p, s, &c.timer))) return r;
        return check_err(c.buf, s, &c.timer);
    }
    // Pipelined: the batch is cut into `nch` contiguous chunks of about equal
    // estimated cost (pixels x paths; the first one half as large, so the
    // device starts early).  The host flattens and uploads chunk k + 1 into
    // one slot while the device renders chunk k from the other; every chunk
    // is an ordinary submission, so the pixels are those of one submission.
    for (uint32_t i = 0; i < count; i++)
        if (!trees[i]) { set_error("invalid batch entry %u", i); return RGPU_ERR_INVALID_ARG; }
    std::vector<double> cum(count + 1, 0.0);
    for (uint32_t i = 0; i < count; i++) {
        const rgpu_tree *tr = trees[i];
        cum[i + 1] = cum[i] + (double)widths[i] * (double)heights[i] * (double)std::max<size_t>(1, tr->paths.size());
    }
    std::vector<uint32_t> cut(nch + 1, count);
    cut[0] = 0;
    {
        const double unit = cum[count] / (nch - 0.5);  // the first chunk takes half a unit
        uint32_t i = 0;
        for (uint32_t k = 1; k < nch; k++) {
            const double target = unit * (k - 0.5);
            while (i < count && cum[i + 1] <= target) i++;
            cut[k] = std::max(cut[k - 1] + 1, std::min(i + 1, count - (nch - k)));
            i = cut[k];
        }
    }
    CK(c.pipe_err.ensure(nch * sizeof(uint32_t)));
    uint32_t *herr = (uint32_t *)c.pipe_err.p;
    for (auto &sl : c.pipe)
        if (!sl.done) CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
    g_stats.raster_ms = 0.0f;
    float raster_ms = 0.0f;
    rgpu_stats acc{};
    for (uint32_t k = 0; k < nch; k++) {
        PipeSlot &sl = c.pipe[k & 1u];
        // the slot's previous chunk (k - 2) has finished with its buffers and staging
        CK(cudaEventSynchronize(sl.done));
        if (k >= 2 && sl.timer.used) {
            for (int t = 0; t < sl.timer.used; t++) {
                float ms = 0.0f;
                if (cudaEventElapsedTime(&ms, sl.timer.start[t], sl.timer.stop[t]) == cudaSuccess) raster_ms += ms;
            }
            sl.timer.used = 0;
        }
        Plan p;
        const uint32_t a = cut[k], n = cut[k + 1] - cut[k];
        std::memset(&g_stats, 0, sizeof(g_stats));
        if ((r = build_batch(p, trees + a, transforms + a, n, widths + a, heights + a, device_pixmaps + a, nullptr)))
            return r;
        if ((r = plan_scene(c, p))) return r;
        if ((r = upload_plan(c, sl.buf, p, s, &sl.staging))) return r;
        if ((r = enqueue_plan(c, sl.buf, p, s, &sl.timer))) return r;
        CK(cudaMemcpyAsync(herr + k, sl.buf.err.p, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(sl.done, s));
        acc.draws += g_stats.draws;
        acc.edges += g_stats.edges;
        acc.work_items += g_stats.work_items;
        acc.kernel_launches += g_stats.kernel_launches;
        acc.h2d_bytes += g_stats.h2d_bytes;
    }
    CK(cudaStreamSynchronize(s));
    for (auto &sl : c.pipe) {
        for (int t = 0; t < sl.timer.used; t++) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, sl.timer.start[t], sl.timer.stop[t]) == cudaSuccess) raster_ms += ms;
        }
        sl.timer.used = 0;
    }
    cudaGetLastError();
    g_stats = acc;
    g_stats.raster_ms = raster_ms;
    for (uint32_t k = 0; k < nch; k++)
        if (herr[k]) {
            set_error("raster kernel reported error flags 0x%x (chunk %u of %u)", herr[k], k, nch);
            return RGPU_ERR_DEVICE_FAULT;
        }
    return RGPU_OK;
}

int rgpu_scene_prepare(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                       const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps,
                       const uint32_t *strides, rgpu_scene **out) {
    g_last_error.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!out || !trees || !transforms || !widths || !heights || !device_pixmaps || count == 0) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    *out = nullptr;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    rgpu_scene *sc = new rgpu_scene();
    if ((r = build_batch(sc->plan, trees, transforms, count, widths, heights, device_pixmaps, strides)) ||
        (r = plan_scene(c, sc->plan)) || (r = upload_plan(c, sc->buf, sc->plan, c.stream))) {
        delete sc;
        return r;
    }
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) {
        set_error("rgpu_scene_prepare: %s", cudaGetErrorString(e));
        delete sc;
        return RGPU_ERR_CUDA;
    }
    *out = sc;
    return RGPU_OK;
}

int rgpu_scene_render(rgpu_scene *sc, void *stream) {
    g_last_error.clear();
    g_last_warning.clear();
    if (!sc) { set_error("invalid arguments"); return RGPU_ERR_INVALID_ARG; }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    WritebackJoin writebacks;  // joined before the lock is released
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    sc->last_stream = s;
    int r;
    if (!sc->plan.sized || sc->timing) {
        // the first render sizes the edge and bin buffers (two synchronisations);
        // timing renders run un-captured with events around the raster kernel
        r = enqueue_plan(c, sc->buf, sc->plan, s, sc->timing ? &sc->timer : nullptr);
        sc->timed_valid = sc->timing && r == RGPU_OK;
        return r;
    }
    sc->timed_valid = false;
    if (!sc->graph || sc->graph_stream != s) {
        if (sc->graph) { cudaGraphExecDestroy(sc->graph); sc->graph = nullptr; }
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        r = enqueue_plan(c, sc->buf, sc->plan, s, nullptr);
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (r) return r;
        CK(e);
        e = cudaGraphInstantiate(&sc->graph, g, 0);
        cudaGraphDestroy(g);
        CK(e);
        sc->graph_stream = s;
    }
    CK(cudaGraphLaunch(sc->graph, s));
    return RGPU_OK;
}

int rgpu_scene_set_timing(rgpu_scene *sc, int enabled) {
    if (!sc) return RGPU_ERR_INVALID_ARG;
    sc->timing = enabled != 0;
    return RGPU_OK;
}

int rgpu_scene_check(rgpu_scene *sc, float *raster_ms) {
    if (!sc) return RGPU_ERR_INVALID_ARG;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    cudaStream_t s = sc->last_stream ? sc->last_stream : c.stream;
    int r = check_err(sc->buf, s, sc->timed_valid ? &sc->timer : nullptr);
    if (raster_ms) *raster_ms = sc->timed_valid ? g_stats.raster_ms : -1.0f;
    return r;
}

int rgpu_scene_info(const rgpu_scene *sc, rgpu_scene_stats *st) {
    if (!sc || !st) return RGPU_ERR_INVALID_ARG;
    const Plan &p = sc->plan;
    st->streams = p.sb.streams.size();
    st->draws = p.sb.draws.size();
    st->commands = p.sb.cmds.size();
    st->segments = p.nsegs;
    st->edges = p.nedges;
    st->binned_edges = p.nbinned;
    st->work_items = p.items.size();
    st->grid = p.grid;
    st->pixels_per_thread = p.px;
    st->kernel_launches = 13;
    uint64_t px = 0;
    for (auto &s : p.sb.streams) px += (uint64_t)s.out_w * s.out_h;
    st->output_pixels = px;
    uint64_t layer_px = 0;
    for (auto &l : p.sb.layers) layer_px += (uint64_t)l.w * l.h;
    st->layer_pixels = layer_px;
    st->record_bytes = p.sb.verbs.size() + p.sb.pts.size() * 4 + p.sb.draws.size() * sizeof(DrawRec) +
                       p.sb.paints.size() * sizeof(PaintRec) + p.sb.grads.size() * sizeof(GradRec) +
                       p.sb.layers.size() * sizeof(LayerRec) + p.sb.cmds.size() * sizeof(Cmd);
    return RGPU_OK;
}

void rgpu_scene_free(rgpu_scene *sc) {
    if (!sc) return;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    if (c.stream) cudaStreamSynchronize(c.stream);
    delete sc;
}

int rgpu_set_tuning(const rgpu_tuning *t) {
    if (!t) return RGPU_ERR_INVALID_ARG;
    if (t->band_rows && t->band_rows != 1 && t->band_rows != 2 && t->band_rows != 4 && t->band_rows != 8)
        return RGPU_ERR_INVALID_ARG;
    if (t->pixels_per_thread && t->pixels_per_thread != 4 && t->pixels_per_thread != 8 && t->pixels_per_thread != 16)
        return RGPU_ERR_INVALID_ARG;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    c.tuning.band_rows = t->band_rows;
    c.tuning.px = t->pixels_per_thread;
    return RGPU_OK;
}

int rgpu_set_tuning_table(const rgpu_tuning_entry *entries, uint32_t count) {
    if (count && !entries) return RGPU_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < count; i++) {
        const uint32_t b = entries[i].band_rows;
        if (b && b != 1 && b != 2 && b != 4 && b != 8) return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    c.tuning.table.assign(entries, entries + count);
    return RGPU_OK;
}

int rgpu_get_tuning_table(rgpu_tuning_entry *entries, uint32_t capacity, uint32_t *count) {
    if (!count || (capacity && !entries)) return RGPU_ERR_INVALID_ARG;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    *count = (uint32_t)c.tuning.table.size();
    for (uint32_t i = 0; i < capacity && i < *count; i++) entries[i] = c.tuning.table[i];
    return RGPU_OK;
}

int rgpu_get_tuning(rgpu_tuning *t) {
    if (!t) return RGPU_ERR_INVALID_ARG;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    t->band_rows = c.tuning.band_rows;
    t->pixels_per_thread = c.tuning.px;
    t->reserved = 0;
    return RGPU_OK;
}

int rgpu_autotune(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                  const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps,
                  const uint32_t *strides, const rgpu_tuning *candidates, uint32_t ncand, uint32_t reps,
                  rgpu_tuning *best, float *best_ms) {
    g_last_error.clear();
    if (!candidates || !ncand || !best || !reps) { set_error("invalid arguments"); return RGPU_ERR_INVALID_ARG; }
    rgpu_tuning saved;
    rgpu_get_tuning(&saved);
    cudaStream_t s;
    {
        Context &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        int r = ensure_device(c);
        if (r) return r;
        s = c.stream;
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); set_error("event"); return RGPU_ERR_CUDA; }
    float best_t = 0.0f;
    int best_i = -1, last_err = RGPU_OK;
    for (uint32_t i = 0; i < ncand; i++) {
        if (rgpu_set_tuning(&candidates[i]) != RGPU_OK) continue;
        rgpu_scene *sc = nullptr;
        int r = rgpu_scene_prepare(trees, transforms, count, widths, heights, device_pixmaps, strides, &sc);
        // first render sizes the buffers, the second captures the graph
        if (r == RGPU_OK) r = rgpu_scene_render(sc, s);
        if (r == RGPU_OK) r = rgpu_scene_render(sc, s);
        if (r == RGPU_OK) r = rgpu_scene_check(sc, nullptr);
        float ms = 0.0f;
        if (r == RGPU_OK) {
            cudaEventRecord(e0, s);
            for (uint32_t k = 0; k < reps && r == RGPU_OK; k++) r = rgpu_scene_render(sc, s);
            cudaEventRecord(e1, s);
            if (r == RGPU_OK) r = rgpu_scene_check(sc, nullptr);
            if (r == RGPU_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) r = RGPU_ERR_CUDA;
            ms /= (float)reps;
        }
        if (sc) rgpu_scene_free(sc);
        if (r != RGPU_OK) { last_err = r; continue; }
        if (best_i < 0 || ms < best_t) { best_t = ms; best_i = (int)i; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_i < 0) {
        rgpu_set_tuning(&saved);
        if (g_last_error.empty()) set_error("no candidate tuning rendered");
        return last_err != RGPU_OK ? last_err : RGPU_ERR_INVALID_ARG;
    }
    rgpu_set_tuning(&candidates[best_i]);
    *best = candidates[best_i];
    if (best_ms) *best_ms = best_t;
    g_last_error.clear();
    return RGPU_OK;
}

int rgpu_set_wait_limit(uint32_t rounds) {
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    raster_set_wait_limit(rounds);
    return RGPU_OK;
}

int rgpu_test_withhold_window(int enabled) {
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    raster_set_withhold(enabled != 0);
    return RGPU_OK;
}

int rgpu_test_fail_allocations(uint32_t count) {
    g_fail_allocs.store(count);
    return RGPU_OK;
}

int rgpu_set_batch_chunks(uint32_t chunks) {
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    c.batch_chunks = chunks;
    return RGPU_OK;
}

int rgpu_trim(void) {
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    if (c.device < 0) return RGPU_OK;
    cudaDeviceSynchronize();  // pipelined batches may still run on a caller's stream
    cudaGetLastError();
    c.buf.release();
    c.surface.release();
    c.staging.release();
    for (auto &sl : c.pipe) {
        sl.buf.release();
        sl.staging.release();
    }
    c.pipe_err.release();
    return RGPU_OK;
}

int rgpu_set_stroke_mode(int on_device) {
    set_device_stroke(on_device != 0);
    return RGPU_OK;
}

int rgpu_stroke_paths(const rgpu_stroke_desc *descs, uint32_t count, const uint8_t *verbs, uint32_t verb_count,
                      const float *pts, uint32_t pt_count, const float *dashes, uint32_t dash_count, int on_device,
                      uint8_t *out_verbs, uint32_t verb_cap, float *out_pts, uint32_t pt_cap, uint32_t *out_counts) {
    g_last_error.clear();
    if ((count && (!descs || !verbs || !pts || !out_counts)) || (verb_cap && !out_verbs) || (pt_cap && !out_pts)) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    for (uint32_t i = 0; i < count; i++) {
        const rgpu_stroke_desc &d = descs[i];
        if ((uint64_t)d.verb_off + d.verb_cnt > verb_count || (uint64_t)d.pt_off + d.pt_cnt > pt_count ||
            (d.dash_cnt && (!dashes || (uint64_t)d.dash_off + d.dash_cnt > dash_count))) {
            set_error("path %u lies outside the verb / point / dash arrays", i);
            return RGPU_ERR_INVALID_ARG;
        }
    }
    uint64_t vo = 0, po = 0;
    auto put = [&](uint32_t i, const uint8_t *v, uint32_t nv, const float *q, uint32_t np) -> int {
        if (vo + nv > verb_cap || po + np > pt_cap) {
            set_error("the outlines exceed the output arrays");
            return RGPU_ERR_CAPACITY;
        }
        std::memcpy(out_verbs + vo, v, nv);
        std::memcpy(out_pts + 2 * po, q, (size_t)np * 8);
        vo += nv;
        po += np;
        out_counts[2 * i] = nv;
        out_counts[2 * i + 1] = np;
        return RGPU_OK;
    };
    if (!on_device) {
        for (uint32_t i = 0; i < count; i++) {
            const rgpu_stroke_desc &d = descs[i];
            StrokeStyle st;
            st.width = d.width;
            st.miter_limit = d.miter_limit;
            st.cap = d.cap;
            st.join = d.join;
            PathData o, dashed;
            const uint8_t *sv = verbs + d.verb_off;
            const float *sp = pts + 2 * (size_t)d.pt_off;
            size_t nv = d.verb_cnt, np = d.pt_cnt;
            bool draw = true;
            if (d.dash_cnt && dash_path(sv, nv, sp, np, dashes + d.dash_off, d.dash_cnt, d.dash_phase, d.res_scale, dashed)) {
                draw = !dashed.empty();
                sv = dashed.verbs.data();
                sp = dashed.pts.data();
                nv = dashed.verbs.size();
                np = dashed.pts.size() / 2;
            }
            if (!draw || !stroke_path(sv, nv, sp, np, st, d.res_scale, o)) o = PathData();
            int r = put(i, o.verbs.data(), (uint32_t)o.verbs.size(), o.pts.data(), (uint32_t)(o.pts.size() / 2));
            if (r) return r;
        }
        return RGPU_OK;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    if (!count) return RGPU_OK;
    cudaStream_t s = c.stream;
    // one job per path over a standalone plan: every job has its own DrawRec
    static Buffers b;
    Plan p;
    p.sb.verbs.assign(verbs, verbs + verb_count);
    p.sb.pts.assign(pts, pts + 2 * (size_t)pt_count);
    p.sb.draws.resize(count);
    std::memset(p.sb.draws.data(), 0, count * sizeof(DrawRec));
    p.sb.stroke_jobs.resize(count);
    for (uint32_t i = 0; i < count; i++) {
        const rgpu_stroke_desc &d = descs[i];
        StrokeJob &j = p.sb.stroke_jobs[i];
        std::memset(&j, 0, sizeof(j));
        j.src_verb_off = d.verb_off; j.src_verb_cnt = d.verb_cnt;
        j.src_pt_off = d.pt_off; j.src_pt_cnt = d.pt_cnt;
        j.width = d.width; j.miter_limit = d.miter_limit; j.res_scale = d.res_scale;
        j.cap_join = (d.cap & 0xFFu) | (d.join & 0xFFu) << 8;
        j.draw = i;
        if (d.dash_cnt) {
            j.dash_off = (uint32_t)p.sb.dashes.size();
            j.dash_cnt = d.dash_cnt;
            j.dash_phase = d.dash_phase;
            p.sb.dashes.insert(p.sb.dashes.end(), dashes + d.dash_off, dashes + d.dash_off + d.dash_cnt);
        }
    }
    if ((r = plan_scene(c, p))) return r;
    CK(b.verbs.ensure(std::max<size_t>(p.sb.verbs.size(), 1)));
    CK(b.pts.ensure(std::max<size_t>(p.sb.pts.size(), 1) * 4));
    CK(b.draws.ensure(count * sizeof(DrawRec)));
    CK(b.sjobs.ensure(count * sizeof(StrokeJob)));
    CK(b.totals.ensure(64));
    CK(b.scan_scratch.ensure(scan_scratch_words((uint64_t)count + 1) * 4));
    if ((r = ensure_stroke_buffers(b, p))) return r;
    CK(cudaMemcpyAsync(b.verbs.p, p.sb.verbs.data(), p.sb.verbs.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.pts.p, p.sb.pts.data(), p.sb.pts.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.draws.p, p.sb.draws.data(), count * sizeof(DrawRec), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.sjobs.p, p.sb.stroke_jobs.data(), count * sizeof(StrokeJob), cudaMemcpyHostToDevice, s));
    if (!p.sb.dashes.empty())
        CK(cudaMemcpyAsync(b.sdash.p, p.sb.dashes.data(), p.sb.dashes.size() * 4, cudaMemcpyHostToDevice, s));
    if ((r = run_strokes(b, p, s))) return r;
    std::vector<uint8_t> hv(p.sverbs);
    std::vector<float> hp(2 * p.spts);
    if (p.sverbs) CK(cudaMemcpyAsync(hv.data(), b.sverbs.p, p.sverbs, cudaMemcpyDeviceToHost, s));
    if (p.spts) CK(cudaMemcpyAsync(hp.data(), b.spts.p, p.spts * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // the plan orders jobs by shape; job.draw is the path's index
    std::vector<uint32_t> job_of(count);
    for (uint32_t k = 0; k < count; k++) job_of[p.sb.stroke_jobs[k].draw] = k;
    for (uint32_t i = 0; i < count; i++) {
        const StrokeJob &j = p.sb.stroke_jobs[job_of[i]];
        // a job whose stroke produced nothing has an empty slice
        if ((r = put(i, hv.data() + j.verb_off, j.verb_cap, hp.data() + 2 * (size_t)j.pt_off, j.pt_cap))) return r;
    }
    return RGPU_OK;
}

int rgpu_get_stats(rgpu_stats *s) {
    if (!s) return RGPU_ERR_INVALID_ARG;
    *s = g_stats;
    return RGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- filter kernels on caller images
static DevBuf g_ftmp;
static DevBuf g_fplane;

extern "C" {

int rgpu_filter_box_blur(uint8_t *img, uint32_t w, uint32_t h, double sx, double sy, void *stream) {
    g_last_error.clear();
    if (!img || !w || !h) { set_error("invalid arguments"); return RGPU_ERR_INVALID_ARG; }
    if (!(sx >= 0.0 && sx <= kBoxSigmaMax) || !(sy >= 0.0 && sy <= kBoxSigmaMax)) {
        set_error("standard deviation must be finite, >= 0 and <= 1e8");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    CK(g_ftmp.ensure((size_t)w * h * 4));
    CK(filter_box_blur((uint32_t *)img, g_ftmp.as<uint32_t>(), (int)w, (int)h, sx, sy, s));
    if (!stream) CK(cudaStreamSynchronize(s));  // a caller stream: asynchronous
    return RGPU_OK;
}

int rgpu_filter_iir_blur(uint8_t *img, uint32_t w, uint32_t h, double sx, double sy, void *stream) {
    g_last_error.clear();
    if (!img || !w || !h) { set_error("invalid arguments"); return RGPU_ERR_INVALID_ARG; }
    if (!(sx >= 0.0 && sx < 1.0e8) || !(sy >= 0.0 && sy < 1.0e8)) {
        set_error("standard deviation must be finite, >= 0 and < 1e8");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    CK(g_fplane.ensure((size_t)w * h * 8 * 4));  // four f64 planes
    CK(filter_iir_blur((uint32_t *)img, g_fplane.as<double>(), (int)w, (int)h, sx, sy, s));
    if (!stream) CK(cudaStreamSynchronize(s));  // a caller stream: asynchronous
    return RGPU_OK;
}

int rgpu_set_iir_precision(uint32_t mode) {
    if (mode > 1) { set_error("IIR precision: 0 (f64, bit-exact) or 1 (f32 chunked scan)"); return RGPU_ERR_INVALID_ARG; }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    filter_set_iir_fast(mode == 1);
    return RGPU_OK;
}

int rgpu_filter_morphology(uint8_t *img, uint32_t w, uint32_t h, int dilate, float rx, float ry, void *stream) {
    g_last_error.clear();
    if (!img || !w || !h || !(rx > 0) || !(ry > 0)) { set_error("invalid arguments"); return RGPU_ERR_INVALID_ARG; }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    CK(g_ftmp.ensure((size_t)w * h * 4));
    CK(filter_morphology((uint32_t *)img, g_ftmp.as<uint32_t>(), (int)w, (int)h, dilate != 0, rx, ry, s));
    if (!stream) CK(cudaStreamSynchronize(s));  // a caller stream: asynchronous
    return RGPU_OK;
}

int rgpu_filter_color_space(uint8_t *img, uint32_t w, uint32_t h, int to_linear, void *stream) {
    g_last_error.clear();
    if (!img || !w || !h) { set_error("invalid arguments"); return RGPU_ERR_INVALID_ARG; }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    CK(filter_color_space((uint32_t *)img, (size_t)w * h, to_linear != 0, s));
    if (!stream) CK(cudaStreamSynchronize(s));  // a caller stream: asynchronous
    return RGPU_OK;
}

static Buffers g_fjob;
static DevBuf g_fresult;
int rgpu_filter_apply(const rgpu_filter *filter, const rgpu_primitive *prims, uint32_t prim_count,
                      const int32_t *merge_inputs, uint32_t merge_count, resvg_transform ts, uint8_t *img,
                      uint32_t w, uint32_t h, void *stream) {
    g_last_error.clear();
    if (!filter || (!prims && prim_count) || (!merge_inputs && merge_count) || !img || !w || !h ||
        (uint64_t)w * h > ((uint64_t)1 << 28)) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    for (uint32_t i = 0; i < prim_count; i++) {
        const rgpu_primitive &p = prims[i];
        if (p.kind == RGPU_FE_MERGE &&
            (p.i[0] < 0 || p.i[1] < 0 || (uint64_t)(uint32_t)p.i[0] + (uint32_t)p.i[1] > merge_count)) {
            set_error("merge inputs out of range");
            return RGPU_ERR_INVALID_ARG;
        }
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    rgpu_filter f = *filter;
    f.prim_offset = 0;
    f.prim_count = prim_count;
    const uint32_t ref = 0;
    rgpu_tree_view view;
    std::memset(&view, 0, sizeof(view));
    view.filters = &f; view.filter_count = 1;
    view.filter_refs = &ref; view.filter_ref_count = 1;
    view.prims = prims; view.prim_count = prim_count;
    view.merge_inputs = merge_inputs; view.merge_input_count = merge_count;
    FilterJob job;
    std::memset(&job, 0, sizeof(job));
    job.w = (int32_t)w; job.h = (int32_t)h;
    job.ts = Xf::row(ts.a, ts.b, ts.c, ts.d, ts.e, ts.f);
    job.tree = &view;
    job.filter_ref_offset = 0; job.filter_count = 1;
    CK(g_fresult.ensure((size_t)w * h * 4));
    BufScratch scratch(g_fjob);
    std::string ferr;
    g_last_warning.clear();
    r = run_filter_job(job, (uint32_t *)img, g_fresult.as<uint32_t>(), scratch, s, ferr);
    if (scratch.e != cudaSuccess) CK(scratch.e);
    if (r) { set_error("filter: %s", ferr.c_str()); return r; }
    if (!ferr.empty()) add_warning("filter: " + ferr + " (layer cleared)");
    CK(cudaMemcpyAsync(img, g_fresult.p, (size_t)w * h * 4, cudaMemcpyDeviceToDevice, s));
    if (!stream) CK(cudaStreamSynchronize(s));
    return RGPU_OK;
}

}  // extern "C"
