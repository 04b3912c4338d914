// Host-side geometry of anti-aliased hairline strokes.
//
// tiny-skia draws a stroke whose device width is at most one pixel on both
// axes as an anti-aliased hairline instead of filling its outline
// (Pixmap::stroke_path -> treat_as_hairline -> scan::hairline_aa, the port of
// Skia's SkScan_Antihair).  resvg reaches it through path.rs:113.  The steps
// before any pixel is touched live here: the coverage that modulates the
// paint's opacity, the device-space path with round/square cap extension,
// subdivision of quads and cubics into polylines (scan/hairline.rs), and the
// per-line clipping to fixed-point range and to the target (anti_hair_line_rgn).
// What comes out is an ordered list of fixed-point line calls, and for each
// call do_anti_hairline's split and setup as spans; the blits run on the
// device (kernels/raster.cu), each pixel evaluating the spans that cover it.
#pragma once
#include <cstdint>
#include <vector>
#include "../device_types.h"
#include "geom.h"
#include "xform.h"

namespace rgpu {

// One do_anti_hairline call: endpoints in FDot6 (26.6 fixed point) and the
// clip rectangle it runs under (has_clip = 0: unclipped).
struct HairCall {
    int32_t x0, y0, x1, y1;
    int32_t clip_l, clip_t, clip_r, clip_b;
    uint32_t has_clip;
};

// treat_as_hairline: true when a stroke of `width` under `ts` is drawn as an
// anti-aliased hairline; *coverage is the factor that scales the paint.
bool treat_as_hairline(bool anti_alias, float width, const Xf &ts, float *coverage);

// The paint opacity factor tiny-skia applies for a hairline coverage < 1
// (source-over-like blend modes only): (255 * floor(coverage * 256)) >> 8, / 255.
float hairline_opacity(float coverage);

// The line calls of a hairline stroke of `path` (user space) under `ts` onto a
// target of clip_w x clip_h pixels with the given cap (rgpu_cap).
void hairline_calls(const PathData &path, const Xf &ts, uint32_t cap, int32_t clip_w, int32_t clip_h,
                    std::vector<HairCall> &out);

// do_anti_hairline's arithmetic before any pixel: the split of long lines
// (more than 511 px along an axis) into halves, the choice of blitter, the
// fixed-point start, slope, end-cap scales and the clip adjustments, as
// spans whose rect is the clip intersected with the pixels the line touches.
void hairline_spans(const HairCall &call, std::vector<HairSpan> &out);

}  // namespace rgpu
