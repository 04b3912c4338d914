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
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "../kernels/kernels.h"
#include "flatten.h"
#include "resvg_gpu.h"
#include "tree.h"

struct rgpu_tree : rgpu::Tree {};

namespace rgpu {
namespace {

thread_local std::string g_last_error;
thread_local rgpu_stats g_stats{};

void set_error(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
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
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T> T *as() const { return (T *)p; }
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
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
};

struct Tuning {
    uint32_t band_rows = 0;  // 0: automatic
    uint32_t px = 0;         // pixels per thread: 0 automatic, else 4/8/16
};

struct Context {
    std::mutex mu;
    int device = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DevBuf verbs, pts, draws, paints, grads, layers, cmds, streams, items;
    DevBuf tpts, segs, seg_counts, seg_offsets, scan_scratch, totals;
    DevBuf edges, edge_draw, bin_counts, bin_offsets, bins;
    DevBuf stack, span_ovf, err, counter, surface;
    HostBuf staging;
    Tuning tuning;
};

Context &ctx() {
    static Context c;
    return c;
}

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
    CK(cudaEventCreate(&c.ev0));
    CK(cudaEventCreate(&c.ev1));
    c.device = dev;
    return RGPU_OK;
}

template <class T>
int upload(Context &c, DevBuf &d, const std::vector<T> &v, size_t &stage_off, cudaStream_t s) {
    size_t bytes = v.size() * sizeof(T);
    CK(d.ensure(bytes ? bytes : 16));
    if (!bytes) return RGPU_OK;
    std::memcpy((char *)c.staging.p + stage_off, v.data(), bytes);
    CK(cudaMemcpyAsync(d.p, (char *)c.staging.p + stage_off, bytes, cudaMemcpyHostToDevice, s));
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
uint32_t pick_bh(int32_t w, uint32_t px, const Tuning &tu) {
    if (tu.band_rows) return tu.band_rows;
    uint32_t bh = 1;
    while (bh < 8 && (256 / (bh * 2)) * px >= (uint32_t)w) bh *= 2;
    return bh;
}

// Runs the device pipeline for a flattened submission on `s`.
int run_scene(Context &c, SceneBuild &sb, cudaStream_t s) {
    uint32_t px = pick_px(sb, c.tuning);
    // work items and bin layout
    std::vector<WorkItem> items;
    uint64_t nbins = 0;
    uint32_t max_depth = 1;
    for (uint32_t si = 0; si < sb.streams.size(); si++) {
        StreamRec &st = sb.streams[si];
        uint32_t bh = pick_bh(st.out_w, px, c.tuning);
        st.band_rows = bh;
        st.nbands = (uint32_t)((st.out_h + (int32_t)bh - 1) / (int32_t)bh);
        st.bin_off = (uint32_t)nbins;
        nbins += (uint64_t)st.nbands * st.draw_cnt;
        max_depth = std::max(max_depth, st.max_depth + 1);
        int32_t cw = (int32_t)((256 / bh) * px);
        for (uint32_t b = 0; b < st.nbands; b++)
            for (int32_t x0 = 0; x0 < st.out_w; x0 += cw) items.push_back(WorkItem{si, b, x0, std::min(x0 + cw, st.out_w)});
    }
    if (nbins > 0xF0000000ull) { set_error("too many (band, draw) bins"); return RGPU_ERR_CAPACITY; }
    g_stats.draws += sb.draws.size();
    g_stats.work_items += items.size();
    // staging: all record arrays
    size_t stage = 0;
    auto rup = [](size_t b) { return (b + 255) & ~(size_t)255; };
    stage += rup(sb.verbs.size()) + rup(sb.pts.size() * 4) + rup(sb.draws.size() * sizeof(DrawRec)) +
             rup(sb.paints.size() * sizeof(PaintRec)) + rup(sb.grads.size() * sizeof(GradRec)) +
             rup(sb.layers.size() * sizeof(LayerRec)) + rup(sb.cmds.size() * sizeof(Cmd)) +
             rup(sb.streams.size() * sizeof(StreamRec)) + rup(items.size() * sizeof(WorkItem)) + 4096;
    CK(c.staging.ensure(stage));
    size_t off = 0;
    int r;
    if ((r = upload(c, c.verbs, sb.verbs, off, s))) return r;
    if ((r = upload(c, c.pts, sb.pts, off, s))) return r;
    if ((r = upload(c, c.draws, sb.draws, off, s))) return r;
    if ((r = upload(c, c.paints, sb.paints, off, s))) return r;
    if ((r = upload(c, c.grads, sb.grads, off, s))) return r;
    if ((r = upload(c, c.layers, sb.layers, off, s))) return r;
    if ((r = upload(c, c.cmds, sb.cmds, off, s))) return r;
    if ((r = upload(c, c.streams, sb.streams, off, s))) return r;
    if ((r = upload(c, c.items, items, off, s))) return r;
    uint32_t ndraws = (uint32_t)sb.draws.size();
    uint64_t nsegs = sb.nsegs;
    CK(c.tpts.ensure(std::max<uint64_t>(sb.ntpts, 1) * 8));
    CK(c.segs.ensure(std::max<uint64_t>(nsegs, 1) * sizeof(SegRec)));
    CK(c.seg_counts.ensure((nsegs + 1) * 4));
    CK(c.seg_offsets.ensure((nsegs + 1) * 4));
    CK(c.totals.ensure(64));
    CK(c.scan_scratch.ensure(scan_scratch_words(std::max<uint64_t>(nsegs + 1, nbins + 1)) * 4));
    uint32_t *totals = c.totals.as<uint32_t>();
    CK(launch_draw_setup(c.draws.as<DrawRec>(), ndraws, c.verbs.as<uint8_t>(), c.pts.as<float>(), c.tpts.p,
                         c.segs.as<SegRec>(), s));
    CK(cudaMemsetAsync(c.seg_counts.p, 0, (nsegs + 1) * 4, s));
    CK(launch_edges(false, c.segs.as<SegRec>(), (uint32_t)nsegs, c.draws.as<DrawRec>(), c.tpts.p,
                    c.seg_counts.as<uint32_t>(), nullptr, nullptr, nullptr, 0, s));
    CK(launch_exclusive_scan(c.seg_counts.as<uint32_t>(), c.seg_offsets.as<uint32_t>(), nsegs + 1,
                             c.scan_scratch.as<uint32_t>(), totals, s));
    uint32_t host_tot[2] = {0, 0};
    CK(cudaMemcpyAsync(host_tot, totals, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint32_t nedges = host_tot[0];
    g_stats.edges += nedges;
    CK(c.edges.ensure(std::max<uint32_t>(nedges, 1) * sizeof(EdgeRec)));
    CK(c.edge_draw.ensure(std::max<uint32_t>(nedges, 1) * 4));
    CK(launch_edges(true, c.segs.as<SegRec>(), (uint32_t)nsegs, c.draws.as<DrawRec>(), c.tpts.p,
                    c.seg_counts.as<uint32_t>(), c.seg_offsets.as<uint32_t>(), c.edges.as<EdgeRec>(),
                    c.edge_draw.as<uint32_t>(), nedges, s));
    CK(launch_draw_edges(c.draws.as<DrawRec>(), ndraws, c.seg_offsets.as<uint32_t>(), s));
    // bins
    CK(c.bin_counts.ensure((nbins + 1) * 4));
    CK(c.bin_offsets.ensure((nbins + 1) * 4));
    CK(cudaMemsetAsync(c.bin_counts.p, 0, (nbins + 1) * 4, s));
    CK(launch_bin(false, c.edges.as<EdgeRec>(), c.edge_draw.as<uint32_t>(), nedges, c.draws.as<DrawRec>(),
                  c.streams.as<StreamRec>(), c.bin_counts.as<uint32_t>(), nullptr, nullptr, s));
    CK(launch_exclusive_scan(c.bin_counts.as<uint32_t>(), c.bin_offsets.as<uint32_t>(), nbins + 1,
                             c.scan_scratch.as<uint32_t>(), totals + 1, s));
    CK(cudaMemcpyAsync(host_tot + 1, totals + 1, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint32_t nbinned = host_tot[1];
    CK(c.bins.ensure(std::max<uint32_t>(nbinned, 1) * sizeof(EdgeRec)));
    CK(cudaMemsetAsync(c.bin_counts.p, 0, (nbins + 1) * 4, s));
    CK(launch_bin(true, c.edges.as<EdgeRec>(), c.edge_draw.as<uint32_t>(), nedges, c.draws.as<DrawRec>(),
                  c.streams.as<StreamRec>(), c.bin_counts.as<uint32_t>(), c.bin_offsets.as<uint32_t>(),
                  c.bins.as<EdgeRec>(), s));
    // raster
    uint32_t per_sm = (uint32_t)raster_max_blocks_per_sm((int)px);
    uint32_t grid = std::min<uint32_t>((uint32_t)items.size(), (uint32_t)c.sms * per_sm);
    if (grid == 0) grid = 1;
    const uint32_t ovf_cap = 64;
    size_t stack_words = (size_t)max_depth * raster_threads() * px;
    CK(c.stack.ensure((size_t)grid * stack_words * 4));
    CK(c.span_ovf.ensure((size_t)grid * raster_threads() * ovf_cap * 8));
    CK(c.err.ensure(16));
    CK(c.counter.ensure(16));
    CK(cudaMemsetAsync(c.err.p, 0, 4, s));
    CK(cudaMemsetAsync(c.counter.p, 0, 4, s));
    CK(cudaEventRecord(c.ev0, s));
    CK(launch_raster((int)px, grid, max_depth, c.streams.as<StreamRec>(), c.items.as<WorkItem>(),
                     (uint32_t)items.size(), c.counter.as<uint32_t>(), c.cmds.as<Cmd>(), c.draws.as<DrawRec>(),
                     c.paints.as<PaintRec>(), c.grads.as<GradRec>(), c.layers.as<LayerRec>(), c.bins.as<EdgeRec>(),
                     c.bin_offsets.as<uint32_t>(), c.bin_counts.as<uint32_t>(), c.stack.as<uint32_t>(),
                     c.span_ovf.as<int2>(), ovf_cap, c.err.as<uint32_t>(), s));
    CK(cudaEventRecord(c.ev1, s));
    g_stats.kernel_launches += 12;
    return RGPU_OK;
}

int check_err(Context &c, cudaStream_t s) {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, c.err.p, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c.ev0, c.ev1) == cudaSuccess) g_stats.raster_ms = ms;
    if (e) {
        set_error("raster kernel reported error flags 0x%x", e);
        return RGPU_ERR_DEVICE_FAULT;
    }
    return RGPU_OK;
}

int render_host(const rgpu_tree *tree, const resvg_transform &ts, uint32_t w, uint32_t h, char *pixmap) {
    g_last_error.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!tree || !pixmap || w == 0 || h == 0 || w > 32767 || h > 32767) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = c.stream;
    size_t bytes = (size_t)w * h * 4;
    CK(c.surface.ensure(bytes));
    SceneBuild sb;
    rgpu_tree *tr = const_cast<rgpu_tree *>(tree);
    if (!tr->finalized) tr->finalize();
    if (sb.add_tree(*tr, Xf::row(ts.a, ts.b, ts.c, ts.d, ts.e, ts.f), (int32_t)w, (int32_t)h,
                    (uint64_t)(uintptr_t)c.surface.p, w * 4) < 0) {
        set_error("%s", sb.error.c_str());
        return RGPU_ERR_UNSUPPORTED;
    }
    CK(c.staging.ensure(bytes));
    std::memcpy(c.staging.p, pixmap, bytes);
    CK(cudaMemcpyAsync(c.surface.p, c.staging.p, bytes, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // staging is reused by run_scene
    g_stats.h2d_bytes += bytes;
    r = run_scene(c, sb, s);
    if (r) return r;
    r = check_err(c, s);
    if (r) return r;
    CK(c.staging.ensure(bytes));
    CK(cudaMemcpyAsync(c.staging.p, c.surface.p, bytes, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::memcpy(pixmap, c.staging.p, bytes);
    g_stats.d2h_bytes += bytes;
    return RGPU_OK;
}

}  // namespace
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

void resvg_render(const resvg_render_tree *tree, resvg_transform transform, uint32_t width, uint32_t height,
                  char *pixmap) {
    int r = render_host(tree, transform, width, height, pixmap);
    if (r != RGPU_OK) fprintf(stderr, "resvg_render: %s\n", g_last_error.c_str());
}

bool resvg_render_node(const resvg_render_tree *tree, const char *id, resvg_transform transform, uint32_t width,
                       uint32_t height, char *pixmap) {
    (void)tree; (void)id; (void)transform; (void)width; (void)height; (void)pixmap;
    set_error("resvg_render_node: not implemented");
    return false;
}

int rgpu_render_device(const resvg_render_tree *tree, resvg_transform ts, uint32_t w, uint32_t h,
                       uint8_t *device_pixmap, uint32_t stride, void *stream) {
    g_last_error.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!tree || !device_pixmap || w == 0 || h == 0 || stride < w * 4) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    SceneBuild sb;
    rgpu_tree *tr = const_cast<rgpu_tree *>(tree);
    if (!tr->finalized) tr->finalize();
    if (sb.add_tree(*tr, Xf::row(ts.a, ts.b, ts.c, ts.d, ts.e, ts.f), (int32_t)w, (int32_t)h,
                    (uint64_t)(uintptr_t)device_pixmap, stride) < 0) {
        set_error("%s", sb.error.c_str());
        return RGPU_ERR_UNSUPPORTED;
    }
    r = run_scene(c, sb, s);
    if (r) return r;
    return check_err(c, s);
}

int rgpu_render_batch(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                      const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps, void *stream) {
    g_last_error.clear();
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!trees || !transforms || !widths || !heights || !device_pixmaps) {
        set_error("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    int r = ensure_device(c);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    SceneBuild sb;
    for (uint32_t i = 0; i < count; i++) {
        rgpu_tree *tr = const_cast<rgpu_tree *>(trees[i]);
        if (!tr || !device_pixmaps[i] || !widths[i] || !heights[i]) {
            set_error("invalid batch entry %u", i);
            return RGPU_ERR_INVALID_ARG;
        }
        if (!tr->finalized) tr->finalize();
        const resvg_transform &ts = transforms[i];
        if (sb.add_tree(*tr, Xf::row(ts.a, ts.b, ts.c, ts.d, ts.e, ts.f), (int32_t)widths[i], (int32_t)heights[i],
                        (uint64_t)(uintptr_t)device_pixmaps[i], widths[i] * 4) < 0) {
            set_error("batch entry %u: %s", i, sb.error.c_str());
            return RGPU_ERR_UNSUPPORTED;
        }
    }
    r = run_scene(c, sb, s);
    if (r) return r;
    return check_err(c, s);
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

int rgpu_get_tuning(rgpu_tuning *t) {
    if (!t) return RGPU_ERR_INVALID_ARG;
    Context &c = ctx();
    std::lock_guard<std::mutex> lock(c.mu);
    t->band_rows = c.tuning.band_rows;
    t->pixels_per_thread = c.tuning.px;
    t->reserved = 0;
    return RGPU_OK;
}

int rgpu_get_stats(rgpu_stats *s) {
    if (!s) return RGPU_ERR_INVALID_ARG;
    *s = g_stats;
    return RGPU_OK;
}

}  // extern "C"
