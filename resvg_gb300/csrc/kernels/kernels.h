// Host-side launchers of the CUDA kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "../device_types.h"
#include "rgpu_tree.h"

namespace rgpu {

// stroke.cu: device-side stroking (one thread per stroked path) and the
// per-draw segment / point bases that follow from the outlines' sizes
size_t stroke_seg_bytes();
cudaError_t stroke_warmup(cudaStream_t s);
// the arrays a stroking pass reads and writes (slices per job in StrokeJob)
struct StrokeBuffers {
    const uint8_t *src_verbs;
    const float *src_pts;
    const float *dashes;
    uint8_t *out_verbs;
    float *out_pts;
    uint8_t *scr_verbs;
    float *scr_pts;
    void *segs;
    uint8_t *dash_verbs;
    float *dash_pts;
    void *msegs;
    float *mpts;
    DrawRec *draws;
    uint32_t *status;
};
size_t stroke_mseg_bytes();
cudaError_t launch_stroke(const StrokeJob *jobs, uint32_t njobs, const StrokeBuffers &b, cudaStream_t s);
cudaError_t launch_stroke_gather(const StrokeMove *moves, uint32_t n, const uint8_t *src_verbs, const float *src_pts,
                                 uint8_t *dst_verbs, float *dst_pts, DrawRec *draws, cudaStream_t s);
cudaError_t launch_draw_sizes(const DrawRec *draws, uint32_t ndraws, uint32_t *seg_sizes, uint32_t *tpt_sizes,
                              cudaStream_t s);
cudaError_t launch_draw_bases(DrawRec *draws, uint32_t ndraws, const uint32_t *seg_base, const uint32_t *tpt_base,
                              cudaStream_t s);

// edges.cu
cudaError_t launch_draw_setup(DrawRec *draws, uint32_t ndraws, const uint8_t *verbs, const float *pts,
                              const uint8_t *stroke_verbs, const float *stroke_pts, void *tpts, SegRec *segs,
                              cudaStream_t s);
cudaError_t launch_edges(bool emit, const SegRec *segs, uint32_t nsegs, const DrawRec *draws, const void *tpts,
                         uint32_t *counts, const uint32_t *offsets, EdgeRec *edges, uint32_t *edge_draw,
                         uint32_t edge_cap, cudaStream_t s);
cudaError_t launch_draw_edges(DrawRec *draws, uint32_t ndraws, const uint32_t *seg_offsets, cudaStream_t s);
cudaError_t launch_bin(bool scatter, const EdgeRec *edges, const uint32_t *edge_draw, uint32_t nedges,
                       const DrawRec *draws, const StreamRec *streams, uint32_t *bin_counts,
                       const uint32_t *bin_offsets, uint32_t bin_cap, uint32_t *err, EdgeRec *bins, cudaStream_t s);
size_t scan_scratch_words(uint64_t n);
cudaError_t launch_exclusive_scan(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *scratch, uint32_t *total,
                                  cudaStream_t s);

// raster.cu
cudaError_t raster_init();
size_t raster_smem_bytes();
size_t raster_stack_words_per_cta(int px);
int raster_threads();
cudaError_t launch_raster(int px, uint32_t grid, uint32_t stack_depth, const StreamRec *streams, const WorkItem *items, uint32_t nitems,
                          uint32_t *item_counter, const Cmd *cmds, const uint32_t *fill_cmds, const DrawRec *draws, const PaintRec *paints,
                          const GradRec *grads, const LayerRec *layers, const EdgeRec *bins,
                          const uint32_t *bin_offsets, const uint32_t *bin_counts, uint32_t *stack, int2 *span_ovf,
                          uint32_t ovf_cap, int2 *run_ovf, uint32_t run_ovf_cap, const HairRec *hairs, const HairSpan *hair_spans, uint32_t *err,
                          cudaStream_t s);
int raster_max_blocks_per_sm(int px);
// Failure-detection controls of the raster kernel: the try_wait rounds after
// which a producer/consumer hand-off is declared stuck (0 = the default), and
// a test hook that withholds the first window of CTA 0 so that wait must run
// out.  Both apply to launches made afterwards.
void raster_set_wait_limit(uint32_t rounds);
uint32_t raster_wait_limit();
void raster_set_withhold(bool on);
int raster_max_pairs();  // (draw, row) pairs of one phase-A window
int raster_window_buffers();  // phase-A window buffers per CTA (each with its own run-overflow area)

// filters.cu
cudaError_t filter_color_space(uint32_t *img, size_t n, bool to_linear, cudaStream_t s);
// the conversion of `src` written to `dst` (one pass instead of a copy and a conversion)
cudaError_t filter_color_space_copy(const uint32_t *src, uint32_t *dst, size_t n, bool to_linear, cudaStream_t s);
void box_sizes(float sigma, int sizes[5]);
// Largest standard deviation the box blur computes with; larger ones give the
// same (fully transparent) result and are clamped to it.
constexpr double kBoxSigmaMax = 1.0e8;
cudaError_t filter_box_blur(uint32_t *img, uint32_t *tmp, int w, int h, double sx, double sy, cudaStream_t s);
// buf: scratch for four f64 planes of w * h values (32 bytes per pixel)
cudaError_t filter_iir_blur(uint32_t *img, double *buf, int w, int h, double sx, double sy, cudaStream_t s);
// IIR precision: false (default) the reference's f64 recursions in its order,
// bit-exact; true an FP32 chunked parallel scan (lines up to 4096 values, else
// f64), within 1 of the f64 result per channel.
void filter_set_iir_fast(bool on);
bool filter_iir_fast();
cudaError_t filter_color_matrix(uint32_t *img, size_t n, int kind, const float *values, cudaStream_t s);
// out of place: `src` (read only) to `dst`; the same pixels as the in-place form
cudaError_t filter_color_matrix_to(const uint32_t *src, uint32_t *dst, size_t n, int kind, const float *values,
                                   cudaStream_t s);
cudaError_t filter_morphology_to(const uint32_t *src, uint32_t *dst, uint32_t *tmp, int w, int h, bool dilate,
                                 float rx, float ry, cudaStream_t s);
cudaError_t filter_morphology(uint32_t *img, uint32_t *tmp, int w, int h, bool dilate, float rx, float ry,
                              cudaStream_t s);
cudaError_t filter_arithmetic(const uint32_t *a, const uint32_t *b, uint32_t *dst, size_t n, const float k[4],
                              cudaStream_t s);
cudaError_t filter_copy(const uint32_t *src, uint32_t *dst, size_t n, cudaStream_t s);
cudaError_t filter_crop(uint32_t *img, int w, int h, int l, int t, int r, int b, cudaStream_t s);
// draw_pixmap of the sw x sh image src at (dx, dy) onto the dw x dh image dst
cudaError_t filter_draw(const uint32_t *src, int sw, int sh, uint32_t *dst, int dw, int dh, int dx, int dy,
                        uint32_t blend, cudaStream_t s);
cudaError_t filter_fill(uint32_t *img, size_t n, uint32_t v, cudaStream_t s);
cudaError_t filter_alpha_only(uint32_t *img, size_t n, cudaStream_t s);
// feComponentTransfer on a premultiplied image: demultiply, lut[c] holds the
// four channels' results for value c (r in the low byte), multiply.
cudaError_t filter_component_transfer(uint32_t *img, size_t n, const uint32_t lut[256], cudaStream_t s);
// feTurbulence (turbulence.rs) into a w x h image, premultiplied.  seed0 is the
// generator state after the seed clamp, in [1, 2^31 - 2]; octaves are bounded by
// the caller.
struct TurbParams {
    double ox, oy, sx, sy, bfx, bfy;
    int octaves, stitch, fractal;
    uint32_t seed0;
};
cudaError_t filter_turbulence(uint32_t *out, int w, int h, const TurbParams &tp, cudaStream_t s);
// feTile: the tile (l, t, tw, th) of the sw x sh image src, inside it, repeated
// from (ox, oy) over the w x h image dst.
cudaError_t filter_tile(const uint32_t *src, int sw, int sh, uint32_t *dst, int w, int h, int ox, int oy, int l,
                        int t, int tw, int th, cudaStream_t s);
// feDisplacementMap with the scaled factors sx, sy and the primitive's scale.
cudaError_t filter_displacement_map(const uint32_t *src, const uint32_t *map, uint32_t *dst, int w, int h, float sx,
                                    float sy, float scale, int xch, int ych, cudaStream_t s);
// The Pattern shader of a fill (tiny-skia's pattern pipeline, highp): for each
// layer pixel of (bx, by, bw, bh), the pixel centre through `inv` (sx, ky, kx,
// sy, tx, ty) into the tw x th tile, repeat or pad tiling, nearest (0),
// bilinear (1) or bicubic (2, then clamped) sampling, opacity; premultiplied
// float4 per pixel into `out`.
cudaError_t filter_pattern_shade(const uint32_t *tile, int tw, int th, float *out, int bx, int by, int bw, int bh,
                                 const float inv[6], int quality, bool repeat, float opacity, cudaStream_t s);
// feDropShadow after the shadow copy is blurred; flood = r | g << 8 | b << 16 | opacity_u8 << 24.
cudaError_t filter_drop_shadow(const uint32_t *in, const uint32_t *shadow, uint32_t *out, int w, int h, int dx,
                               int dy, uint32_t flood, bool linear, cudaStream_t s);

// feConvolveMatrix (convolve_matrix.rs): kernel k[rows * cols] row-major as
// given, applied flipped; edge = rgpu_edge_mode.
struct ConvolveParams {
    int32_t cols, rows, tx, ty, edge, preserve_alpha;
    float divisor, bias;
    float k[62];
};
cudaError_t filter_convolve(const uint32_t *src, uint32_t *dst, int w, int h, const ConvolveParams &cp,
                            cudaStream_t s);

// feDiffuseLighting / feSpecularLighting (lighting.rs) with the light source
// already in the region's pixel space; the distant light vector, the spot
// direction and the cosine of the cone angle are prepared on the host.
struct LightingParams {
    int32_t specular, kind;          // kind: rgpu_light_kind
    float surface_scale, constant, exponent;
    uint32_t color[3];               // lighting colour, u8 per channel
    float lv[3];                     // distant: unit light vector
    float pos[3];                    // point / spot: position
    float dir[3];                    // spot: direction (normalised where possible)
    float spot_exponent;
    int32_t has_cone;
    float cone_cos;
};
cudaError_t filter_lighting(const uint32_t *src, uint32_t *dst, int w, int h, const LightingParams &lp,
                            cudaStream_t s);

}  // namespace rgpu
