// Device-side data layout shared by the host flattener and the CUDA kernels.
//
// The host walks the render tree the way resvg's render.rs does and emits,
// per scene:
//   * DrawRec   — one per filled path (strokes arrive as host-stroked outlines),
//                 holding the path's geometry range, its full transform into its
//                 target layer, the layer size (the tiny-skia clip rect) and paint;
//   * PaintRec  — the resolved paint in the form the raster pipeline consumes;
//   * LayerRec  — isolated-group layers / clip and mask pixmaps (integer rects);
//   * Cmd       — the command stream the band VM executes in order.
// Geometry (verbs, f32 points) is uploaded as-is; the device transforms points,
// builds fixed-point edges, bins them into row bands and rasterises.
#pragma once
#include <stdint.h>
#include <stddef.h>

namespace rgpu {

constexpr int kMaxGradStops = 12;   // intervals incl. the two constant ends (<= 10 stops after padding)

// Laid out so that a gradient of n intervals is the record's first
// 112 + 32 n bytes (the header, the stop positions, then per interval the
// factor and bias rows): shading touches only that prefix.
struct alignas(16) GradRec {
    float ts[6];         // device pixel -> unit gradient space (sx, ky, kx, sy, tx, ty)
    uint32_t flags;      // see GRAD_* below
    uint32_t spread;     // rgpu_spread
    uint32_t n;          // number of t_values / factors / biases
    float fr0, fr1, cdx, cdy;  // two-point conical parameters (unit space)
    uint32_t _pad[3];
    float t[kMaxGradStops];
    struct Row {
        float f[4];      // colour = t * f + b (16-byte rows: one vector load each)
        float b[4];
    } iv[kMaxGradStops];
};
static_assert(sizeof(GradRec) == 496 && offsetof(GradRec, t) == 64 && offsetof(GradRec, iv) == 112,
              "GradRec prefix layout");
enum : uint32_t {
    GRAD_TWO_STOP = 1, GRAD_PAD_CLAMP = 2, GRAD_PREMUL = 4, GRAD_RADIAL_SIMPLE = 8, GRAD_RADIAL_CONICAL = 16
};

// A precomputed source image (a pattern shader evaluated per pixel, highp
// premultiplied float4, bw x bh from layer pixel (bx, by)); stored in a
// GradRec slot, the device address filled in when the scene's buffers exist.
struct ImageRec {
    uint64_t ptr;
    int32_t bx, by, bw, bh;
};
static_assert(sizeof(ImageRec) <= sizeof(GradRec), "ImageRec fits a GradRec slot");

// A gradient paint carries copies of its record's transform, flags, spread and
// interval count in place of the uniform colours, so that the raster kernel
// reads them from the paint it already holds in shared memory and goes to the
// GradRec only for the stop positions and colour rows.
struct PaintRec {
    uint32_t kind;       // 0 solid, 1 gradient, 2 image (ImageRec in the GradRec slot)
    uint32_t blend;      // rgpu_blend after tiny-skia's strength reduction
    uint32_t flags;      // PAINT_* below
    uint32_t grad;       // index into GradRec when kind != 0
    union {
        struct {
            uint16_t rgba16[4];  // lowp uniform colour
            float colorf[4];     // highp uniform colour (premultiplied)
        };
        float gts[6];            // kind 1: GradRec::ts
    };
    uint8_t memset_rgba[4];
    uint32_t gmeta;      // kind 1: GradRec flags | spread << 8 | n << 16
};
static_assert(sizeof(PaintRec) == 48 && offsetof(PaintRec, gts) == 16 && offsetof(PaintRec, colorf) == 24,
              "PaintRec layout");
enum : uint32_t { PAINT_LOWP = 1, PAINT_MEMSET = 2, PAINT_SKIP = 4 };

struct DrawRec {
    // ---- set by the host
    uint32_t verb_off, verb_cnt, pt_off, pt_cnt;  // geometry ranges
    float ts[6];
    int32_t clip_w, clip_h;      // target pixmap size (tiny-skia clip rect)
    int32_t ox, oy;              // target pixmap origin in the stream's output space
    uint32_t flags;              // DRAW_* below
    uint32_t paint;
    uint32_t seg_base;           // segment slots: [seg_base, seg_base + verb_cnt + 1)
    uint32_t tpt_base;           // transformed points: [tpt_base, tpt_base + pt_cnt)
    uint32_t stream;             // stream the draw belongs to
    // ---- set by the setup kernel
    int32_t valid;
    int32_t shift;               // 2: anti-aliased (4x4 supersampling), 0: aliased
    int32_t contained;           // path inside the clip: edges are not clipped
    int32_t sect_l, sect_t, sect_r, sect_b;      // pixel rect coverage may land in
    int32_t start_y, stop_y, right_clip, super_left;  // scan range in (sub)scanline units
    uint32_t edge_base, edge_count;
};
enum : uint32_t {
    DRAW_EVENODD = 1,
    DRAW_AA = 2,
    DRAW_STROKED = 4,  // the geometry is a stroke outline built on the device (stroke arrays)
};

// One path stroked on the device (tiny-skia's Path::dash and Path::stroke,
// one thread per job): the source path in the scene's geometry arrays, the
// dash array (dash_cnt 0: not dashed) and the stroke, and the slices of the
// stroke arrays the job works in.  The thread writes the outline's verb and
// point counts into draws[draw]; a job that outgrows a slice sets its status
// word instead and draws nothing.
struct StrokeJob {
    uint32_t src_verb_off, src_verb_cnt, src_pt_off, src_pt_cnt;
    float width, miter_limit, res_scale;
    uint32_t cap_join;     // rgpu_cap | rgpu_join << 8
    uint32_t draw;         // the DrawRec that fills the outline
    uint32_t verb_off, verb_cap;  // outline slice: verbs
    uint32_t pt_off, pt_cap;      // outline slice: points (x, y pairs)
    uint32_t seg_off, seg_cap;    // segment scratch of the path being stroked
    uint32_t dash_off, dash_cnt;  // dash intervals in the dash array
    float dash_phase;
    uint32_t dverb_off, dverb_cap, dpt_off, dpt_cap;  // the dashed path (scratch)
    uint32_t mseg_off, mseg_cap, mpt_off, mpt_cap;    // one measured contour (scratch)
    uint32_t _pad[6];
};
static_assert(sizeof(StrokeJob) == 128, "StrokeJob layout");

// One outline moved from its sizing slice to its exact slice.
struct StrokeMove {
    uint32_t src_verb, dst_verb, verbs;
    uint32_t src_pt, dst_pt, pts;
    uint32_t draw;
};

struct SegRec {
    uint32_t draw;
    uint32_t kind;   // 0 empty, 1 line, 2 quad, 3 cubic
    uint32_t p0;     // index of the first point in tpts
    uint32_t p1;     // line end point index (close lines point back to the move point)
};

// A fixed-point line edge (SkEdge after curve forward differencing).
struct EdgeRec {
    int32_t x;        // 16.16 at first_y
    int32_t dx;       // 16.16 per (sub)scanline
    int32_t first_y;  // first (sub)scanline, target pixmap coordinates
    int32_t hw;       // (last_y - first_y) << 8 | (winding & 0xff)
};

struct LayerRec {
    int32_t x, y, w, h;   // in the stream's output space
    int32_t surf;         // internal surface holding the layer's initial content (filter result), or -1
    int32_t _pad;
    uint64_t buf;         // device address of that surface (patched when surfaces are allocated)
};

enum CmdOp : uint32_t {
    CMD_FILL = 0,         // a = draw
    CMD_PUSH = 1,         // a = layer, b = init (0 transparent, 1 opaque black, 2 the layer's surface)
    CMD_POP_COMPOSITE = 2,// a = popped layer, b = blend, f = opacity
    CMD_POP_CLIP = 3,     // a = popped layer: mask = 255 - alpha, applied to the new top
    CMD_POP_MASK = 4,     // a = popped layer, b = 0 luminance / 1 alpha
    CMD_APPLY_REGION = 5, // a = draw: top *= coverage(draw)
    CMD_CLEAR = 6,        // top = transparent
    CMD_END = 7,
    CMD_HAIR = 8          // a = hairline draw (HairRec): anti-aliased hairline stroke
};

struct Cmd {
    uint32_t op, a, b;
    float f;
};

// One unit of raster work: a band of output rows [band*band_rows, +band_rows)
// and the x range [x0, x1) of one stream.
struct WorkItem {
    uint32_t stream, band;
    int32_t x0, x1;
};

// One stream = one target surface rendered by the band VM.
struct StreamRec {
    uint32_t cmd_off, cmd_cnt;
    uint32_t draw_off, draw_cnt;   // draws referenced by this stream
    uint32_t layer_off;
    int32_t out_w, out_h;          // target surface size
    uint32_t out_stride;           // bytes per row
    uint64_t out_ptr;              // device pointer of the target surface
    uint32_t band_rows, nbands;    // band height and count
    uint32_t bin_off;              // dense (band, draw) counters for this stream
    uint32_t max_depth;            // layer-stack depth needed
    int32_t surface;               // internal surface rendered into (filter content), or -1
    uint32_t level;                // dependency level: content streams render before their parents
    uint32_t fill_off, fill_cnt;   // this stream's fill / region commands (indices into its commands)
};


// An anti-aliased hairline stroke (tiny-skia scan/hairline_aa.rs): its line
// spans after do_anti_hairline's setup, drawn with `paint` into the current
// layer (layer origin ox, oy in the stream's output space); [x0, x1) x
// [y0, y1) bounds the layer pixels of all its spans.
struct HairRec {
    uint32_t span_off, span_cnt, paint;
    int32_t ox, oy, x0, y0, x1, y1;
    uint32_t _pad[3];
};

// One set-up do_anti_hairline line: n steps along the major axis from
// `istart`; the minor coordinate of step k is (FDot16, clamped at 0 as the
// blitters clamp it) c_k = max(f0 + k*slope, 0) for slope < 0, else
// max(f0, 0) + k*slope, with f0 = fstart + 1/2.  Only pixels inside the rect
// [x0, x1) x [y0, y1) (the clip, the layer and the line's own bounds
// intersected) are touched.  `pack` holds the blitter kind (bits 0-1: 0 hline,
// 1 horish, 2 vline, 3 vertish), the end-cap scales of the first (bits 2-8)
// and last (bits 9-15, 0 = none) step, n (bits 16-25, at most 512) and
// HAIR_SECOND: a vline whose two blit columns coincide is emitted twice, the
// first span drawing only the first blit, the second only the second.
struct HairSpan {
    int32_t istart, f0, slope;
    uint32_t pack;
    int32_t x0, y0, x1, y1;
};
enum : uint32_t { HAIR_SECOND = 1u << 26 };

}  // namespace rgpu
