/*
 * resvg_gpu.h — C ABI of the GB300 rendering backend (libresvg_gb300.so).
 *
 * Drop-in surface: `resvg_render` / `resvg_render_node` keep the signatures
 * of resvg's C API (crates/c-api/resvg.h:485-489 and :505-510, implemented at
 * crates/c-api/lib.rs:875-893 and :908-942): the caller owns a host pixmap of
 * width*height*4 bytes of premultiplied RGBA8, and rendering draws onto its
 * existing content.  Rendering runs on the GPU through hand-written sm_103a
 * kernels; there is no CPU fallback — when no device is usable the call logs
 * the error (resvg_gpu_last_error) and leaves the pixmap untouched, the way
 * the reference logs and skips on internal failures (crates/resvg/src/render.rs:108).
 *
 * `resvg_render_tree` here wraps the backend's resolved tree (rgpu_tree.h),
 * the counterpart of the usvg::Tree that resvg_render_tree wraps in the
 * reference (crates/c-api/lib.rs:839-844).  Parsing SVG text stays outside
 * this library, as usvg stays on the host in the reference.
 *
 * Every function other than the two drop-ins returns an rgpu_status and
 * never aborts.
 */
#ifndef RESVG_GPU_H
#define RESVG_GPU_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include "rgpu_tree.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rgpu_status {
    RGPU_OK = 0,
    RGPU_ERR_INVALID_ARG = 1,
    RGPU_ERR_NO_DEVICE = 2,
    RGPU_ERR_CUDA = 3,
    RGPU_ERR_OUT_OF_MEMORY = 4,
    RGPU_ERR_CAPACITY = 5,      /* a work buffer was too small; the host resizes and retries */
    RGPU_ERR_DEVICE_FAULT = 6,  /* a kernel reported an error word (bounds/timeout), output untouched */
    RGPU_ERR_UNSUPPORTED = 7
} rgpu_status;

/* resvg_transform (crates/c-api/resvg.h, lib.rs:67-81): {a,b,c,d,e,f}. */
typedef struct resvg_transform {
    float a, b, c, d, e, f;
} resvg_transform;

typedef struct rgpu_tree resvg_render_tree;

/* ---- tree building (the usvg::Tree stand-in) ---------------------------- */
resvg_render_tree *rgpu_tree_new(float width, float height);
void rgpu_tree_free(resvg_render_tree *tree);
/* Adds a group under `parent` (-1: detached, e.g. a clip/mask root). */
int32_t rgpu_tree_add_group(resvg_render_tree *tree, int32_t parent, const rgpu_group *group);
int32_t rgpu_tree_add_path(resvg_render_tree *tree, int32_t parent, const rgpu_path *path, const uint8_t *verbs,
                           uint32_t verb_count, const float *points, uint32_t point_count, const float *dashes,
                           uint32_t dash_count);
int32_t rgpu_tree_add_paint(resvg_render_tree *tree, const rgpu_paint *paint, const rgpu_stop *stops,
                            uint32_t stop_count);
int32_t rgpu_tree_add_clip(resvg_render_tree *tree, const rgpu_clip *clip);
int32_t rgpu_tree_add_mask(resvg_render_tree *tree, const rgpu_mask *mask);
int32_t rgpu_tree_add_filter(resvg_render_tree *tree, const rgpu_filter *filter, const rgpu_primitive *prims,
                             uint32_t prim_count, const int32_t *merge_inputs, uint32_t merge_count);
/* Adds a decoded raster image (premultiplied RGBA8, width * height * 4 bytes,
 * copied); returns its index for an RGPU_PAINT_IMAGE paint, or -1. */
int32_t rgpu_tree_add_image(resvg_render_tree *tree, uint32_t width, uint32_t height, const uint8_t *rgba);
/* Gives a group (node_kind RGPU_NODE_GROUP) or a path (RGPU_NODE_PATH) its SVG
 * id, the `id` that usvg keeps on every node (crates/usvg/src/tree/mod.rs,
 * Node::id) and resvg_render_node looks up.  The string is copied. */
int rgpu_tree_set_node_id(resvg_render_tree *tree, uint32_t node_kind, uint32_t index, const char *id);
/* usvg's Tree::node_by_id (crates/usvg/src/tree/mod.rs:1629-1635,1718-1732):
 * the first node with this id in depth-first pre-order below the root group.
 * RGPU_OK and (kind, index) when found; RGPU_ERR_INVALID_ARG otherwise (an
 * empty id never matches). */
int rgpu_tree_find_node(const resvg_render_tree *tree, const char *id, uint32_t *node_kind, uint32_t *index);
/* Attaches filters (indices from rgpu_tree_add_filter) to a group. */
int rgpu_tree_set_group_filters(resvg_render_tree *tree, int32_t group, const uint32_t *filters, uint32_t count);
/* Computes path and layer bounding boxes; call once after building. */
int rgpu_tree_finalize(resvg_render_tree *tree);
const rgpu_tree_view *rgpu_tree_get_view(resvg_render_tree *tree);
/* Seeded synthetic workloads (see resvg_gb300/csrc/host/gen.cpp):
 * config 0..3; `scale` multiplies path counts (1.0 = full workload). */
resvg_render_tree *rgpu_tree_generate(int config, uint64_t seed, uint64_t index, float scale);

/* ---- drop-in render (host pixmap) --------------------------------------- */
/* resvg_render: crates/c-api/resvg.h:485, lib.rs:875-893. */
void resvg_render(const resvg_render_tree *tree, resvg_transform transform, uint32_t width, uint32_t height,
                  char *pixmap);
/* resvg_render_node: crates/c-api/resvg.h:505, lib.rs:908-942 (resvg::render_node,
 * crates/resvg/src/lib.rs:55-70).  `id` is an SVG id given with
 * rgpu_tree_set_node_id, resolved as usvg's node_by_id does
 * (rgpu_tree_find_node).  The node's absolute layer bounding box is moved to
 * the pixmap origin; returns false for an empty or unknown id or an empty box. */
bool resvg_render_node(const resvg_render_tree *tree, const char *id, resvg_transform transform, uint32_t width,
                       uint32_t height, char *pixmap);

/* ---- GPU-native entry points --------------------------------------------- */
/* Selects the CUDA device (no counterpart in the reference: resvg is CPU-only). */
int rgpu_init(int device);
/* Last error message of the calling thread ("" when none). */
const char *rgpu_last_error(void);
/* Warnings of the calling thread's last render or filter call ("" when none):
 * what the reference skips or clears with a log message while rendering goes
 * on, e.g. a filter that fails clears its layer (crates/resvg/src/filter/
 * mod.rs:343-354).  A warning is not an error: the call returned RGPU_OK. */
const char *rgpu_last_warning(void);
/* Render into a DEVICE pixmap on `stream` (cudaStream_t; 0 = default).  The
 * pixmap is premultiplied RGBA8, `stride` bytes per row; rendering draws onto
 * its content.  Asynchronous: returns after enqueueing.  Counterpart of
 * resvg::render (crates/resvg/src/lib.rs:34) without host copies. */
int rgpu_render_device(const resvg_render_tree *tree, resvg_transform transform, uint32_t width, uint32_t height,
                       uint8_t *device_pixmap, uint32_t stride, void *stream);
/* Batched form: renders `count` independent trees.  pixmaps[i] are DEVICE
 * pointers of widths[i]*heights[i]*4 bytes, cleared to transparent by the
 * caller or not (rendering draws onto content).  One submission; the work is
 * spread over persistent work-queue kernels replayed from a captured CUDA
 * graph.  No counterpart in the reference (resvg renders one tree per call). */
int rgpu_render_batch(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                      const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps, void *stream);

/* Prepared scene ("display list"): one or many trees flattened once, with
 * records and geometry resident in device memory and their own work buffers.
 * The first render sizes the edge/bin buffers (two stream synchronisations);
 * later renders are asynchronous and replay a captured CUDA graph.  The
 * device pixmaps given at prepare time are the render targets.  The batched
 * form (many trees) uses one persistent raster kernel over all scenes' bands. */
typedef struct rgpu_scene rgpu_scene;
int rgpu_scene_prepare(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                       const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps,
                       const uint32_t *strides, rgpu_scene **out);
int rgpu_scene_render(rgpu_scene *scene, void *stream);
/* Timing mode: renders run un-captured with CUDA events around the raster
 * kernel so rgpu_scene_check can report its device time (-1 otherwise). */
int rgpu_scene_set_timing(rgpu_scene *scene, int enabled);
/* Synchronises the stream of the last render and reports kernel error flags;
 * raster_ms = raster kernel time of the last render in timing mode, else -1. */
int rgpu_scene_check(rgpu_scene *scene, float *raster_ms);
typedef struct rgpu_scene_stats {
    uint64_t streams, draws, commands, segments, edges, binned_edges, work_items;
    uint64_t grid, pixels_per_thread, kernel_launches, output_pixels, layer_pixels, record_bytes;
} rgpu_scene_stats;
int rgpu_scene_info(const rgpu_scene *scene, rgpu_scene_stats *stats);
void rgpu_scene_free(rgpu_scene *scene);

/* Tuning knobs of the raster kernels (chosen by the autotuner). */
typedef struct rgpu_tuning {
    uint32_t band_rows;          /* pixel rows per raster work item: 0 (auto), 1, 2, 4 or 8 */
    uint32_t pixels_per_thread;  /* consecutive pixels per raster thread: 0 (auto), 4, 8 or 16 */
    uint32_t reserved;
} rgpu_tuning;
int rgpu_set_tuning(const rgpu_tuning *t);
int rgpu_get_tuning(rgpu_tuning *t);
/* Tuning table: with band_rows 0 in the tuning, each stream (a scene or an
 * internal surface) takes the band rows of the first entry whose max_width
 * and max_draws are at least its width and draw count (band_rows 0 in the
 * entry: the built-in rule on the width).  The autotuner fills it per
 * (canvas-size bucket, path-count bucket) (resvg_gb300.batch.autotune_table). */
typedef struct rgpu_tuning_entry {
    uint32_t max_width, max_draws, band_rows, reserved;
} rgpu_tuning_entry;
int rgpu_set_tuning_table(const rgpu_tuning_entry *entries, uint32_t count);
/* Copies up to `capacity` entries and stores the table's length in *count. */
int rgpu_get_tuning_table(rgpu_tuning_entry *entries, uint32_t capacity, uint32_t *count);
/* Autotuner (no counterpart in the reference): prepares the given scenes once
 * per candidate tuning, times `reps` graph replays of each with CUDA events,
 * keeps the fastest as the current tuning and returns it (and its ms per
 * render).  Candidates that fail are skipped. */
int rgpu_autotune(const resvg_render_tree *const *trees, const resvg_transform *transforms, uint32_t count,
                  const uint32_t *widths, const uint32_t *heights, uint8_t *const *device_pixmaps,
                  const uint32_t *strides, const rgpu_tuning *candidates, uint32_t candidate_count, uint32_t reps,
                  rgpu_tuning *best, float *best_ms);

/* Failure detection (no counterpart in the reference, whose only limits are
 * defensive skips: crates/resvg/src/render.rs:108-109, filter/mod.rs:343-354).
 * The raster kernel's producer/consumer hand-offs wait at most `rounds`
 * try_wait rounds (0 = the default, 4,194,304, about a second); a wait that
 * runs out makes the render return RGPU_ERR_DEVICE_FAULT with the pixmap
 * partly rendered, and the next render starts clean.  Applies to launches made
 * afterwards (a prepared scene's captured graph keeps the value it was
 * captured with). */
int rgpu_set_wait_limit(uint32_t rounds);
/* Test hooks of the failure paths, for the library's own tests:
 * rgpu_test_withhold_window(1) makes the first raster CTA withhold its first
 * window, so that hand-off's bounded wait must run out (no GPU fault is made);
 * rgpu_test_fail_allocations(n) makes the library's next n device or pinned
 * host allocations fail as if memory were exhausted (RGPU_ERR_OUT_OF_MEMORY,
 * the pixmap untouched). */
int rgpu_test_withhold_window(int enabled);
int rgpu_test_fail_allocations(uint32_t count);
/* rgpu_render_batch cuts a batch into chunks of about equal estimated cost
 * (pixels x paths) and flattens and uploads chunk k + 1 on the host while the
 * device renders chunk k.  `chunks` = 0: automatic (8 chunks for batches of
 * 64 scenes or more, else one submission); 1: always one submission; n: n
 * chunks (at most one per scene).  The pixels do not depend on it. */
int rgpu_set_batch_chunks(uint32_t chunks);
/* Frees the library's cached device buffers and pinned staging (they grow to
 * the largest render seen and are otherwise kept for reuse). */
int rgpu_trim(void);

/* Where stroke outlines are built when a tree is rendered: 1 (the default) on
 * the device, one thread per stroked path; 0 on the host.  Both run the same
 * dasher and stroker (tiny-skia-path's Path::dash and Path::stroke, called
 * from resvg's crates/resvg/src/path.rs:106-113 through Pixmap::stroke_path)
 * and give identical outlines. */
int rgpu_set_stroke_mode(int on_device);

/* Strokes `count` paths and returns their outlines (the path to fill with the
 * non-zero rule), as resvg's stroke_path does through tiny-skia-path:
 * Path::dash(dash, res_scale) when the path is dashed (an invalid dash array
 * strokes the undashed path, a dashing that leaves nothing gives no outline),
 * then Path::stroke(stroke, res_scale).  Path i is verbs[verb_off, verb_off +
 * verb_cnt) with points pts[2 * pt_off, 2 * (pt_off + pt_cnt)), dashed by
 * dashes[dash_off, dash_off + dash_cnt) from dash_phase (dash_cnt 0: not
 * dashed).  The outlines are written one after
 * another to out_verbs / out_pts (x, y pairs), out_counts[2i] and
 * out_counts[2i + 1] receiving path i's verb and point counts (0 when the
 * stroke produces nothing).  on_device selects the device stroker (1) or the
 * host one (0).  RGPU_ERR_CAPACITY when the outlines exceed verb_cap verbs or
 * pt_cap points. */
typedef struct rgpu_stroke_desc {
    uint32_t verb_off, verb_cnt, pt_off, pt_cnt;
    float width, miter_limit, res_scale;
    uint32_t cap;   /* rgpu_cap */
    uint32_t join;  /* rgpu_join */
    uint32_t dash_off, dash_cnt;
    float dash_phase;
} rgpu_stroke_desc;
int rgpu_stroke_paths(const rgpu_stroke_desc *descs, uint32_t count, const uint8_t *verbs, uint32_t verb_count,
                      const float *pts, uint32_t pt_count, const float *dashes, uint32_t dash_count, int on_device,
                      uint8_t *out_verbs, uint32_t verb_cap, float *out_pts, uint32_t pt_cap, uint32_t *out_counts);

/* Per-call statistics of the last render on this thread (for benchmarking). */
typedef struct rgpu_stats {
    uint64_t draws, edges, crossings_capacity, work_items, kernel_launches;
    uint64_t h2d_bytes, d2h_bytes;
    float raster_ms;         /* device time of the raster kernel (CUDA events) */
    float stroke_ms;         /* device time of the stroke kernel's last pass when it ran (CUDA events) */
    uint64_t stroke_jobs;    /* paths stroked on the device */
} rgpu_stats;
int rgpu_get_stats(rgpu_stats *s);

/* ---- filter kernels on device images (filter module primitives) --------- */
/* With stream == NULL the call runs on the library's stream and returns when
 * the image is done; with a stream it is enqueued there and returns at once. */
/* Box blur, 5 passes of (vertical, horizontal) box sums: crates/resvg/src/filter/box_blur.rs:23.
 * Standard deviations must be finite, >= 0 and <= 1e8 (RGPU_ERR_INVALID_ARG otherwise). */
int rgpu_filter_box_blur(uint8_t *device_img, uint32_t width, uint32_t height, double sigma_x, double sigma_y,
                         void *stream);
/* IIR (recursive Gaussian) blur in f64: crates/resvg/src/filter/iir_blur.rs:47. */
int rgpu_filter_iir_blur(uint8_t *device_img, uint32_t width, uint32_t height, double sigma_x, double sigma_y,
                         void *stream);
/* Precision of the IIR blur (iir_blur.rs:79-140) everywhere it runs (filter
 * jobs of a render, rgpu_filter_iir_blur, rgpu_filter_apply): 0 (default) the
 * reference's f64 recursions in the reference's order, bit-exact; 1 an FP32
 * chunked parallel scan of the same recursions, within 1 per channel of mode 0
 * (the 1/255 the IIR blur may differ by), for lines up to 4096 pixels (longer
 * lines use mode 0).  Read when work is enqueued: a prepared scene's captured
 * graph keeps the mode it was captured with. */
int rgpu_set_iir_precision(uint32_t mode);
/* Morphology erode (0) / dilate (1): crates/resvg/src/filter/morphology.rs:15. */
int rgpu_filter_morphology(uint8_t *device_img, uint32_t width, uint32_t height, int dilate, float rx, float ry,
                           void *stream);
/* sRGB <-> linearRGB on premultiplied pixels: crates/resvg/src/filter/mod.rs:115-125. */
int rgpu_filter_color_space(uint8_t *device_img, uint32_t width, uint32_t height, int to_linear, void *stream);
/* A whole filter (region + primitive chain, as rgpu_tree_add_filter takes it)
 * applied in place to a device pixmap that is the filtered layer, under the
 * layer transform `ts`: crates/resvg/src/filter/mod.rs:335-354 (filter::apply).
 * SourceGraphic is the pixmap; primitives that make region-sized images
 * (flood, composite, merge, blend, tile, turbulence, lighting, displacement
 * map) make them at the pixmap origin, as the reference does.  A filter that
 * fails (an invalid region, sizes the reference cannot combine) clears the
 * pixmap and the call still returns RGPU_OK with a warning
 * (rgpu_last_warning), as filter::apply clears on error. */
int rgpu_filter_apply(const rgpu_filter *filter, const rgpu_primitive *prims, uint32_t prim_count,
                      const int32_t *merge_inputs, uint32_t merge_count, resvg_transform ts, uint8_t *device_pixmap,
                      uint32_t width, uint32_t height, void *stream);

/* Allocation-free box blur (no counterpart in the reference): the same result
 * as rgpu_filter_box_blur, with the intermediate image in a fixed device array
 * instead of a cudaMalloc'd buffer, for callers that may not allocate device
 * memory (embedders that own the memory budget through their own allocator or
 * a hard cap, and latency paths where cudaMalloc/cudaFree would synchronise
 * the device).  At most 1,048,576 pixels per image (4 MiB of scratch); larger
 * images return RGPU_ERR_INVALID_ARG.  The first call on a device does the
 * set-up (looks up the array's address) and should come before any stream
 * capture.  The scratch is shared by all calls on a device: overlapping calls
 * race.  With a NULL stream the blur runs on the default stream and the call
 * returns after it finished; with a stream it is enqueued there and the call
 * returns at once.  Standard deviations must be finite, >= 0 and <= 1e8. */
int rgpu_filter_box_blur_noalloc(uint8_t *device_img, uint32_t width, uint32_t height, double sigma_x,
                                 double sigma_y, void *stream);

/* ---- differentiable soft-coverage form ---------------------------------- */
/* A batch of scenes for the FP32 analytic-area soft rasteriser and its
 * hand-written adjoint (no counterpart in the reference: resvg's coverage is
 * not differentiable).  All pointers are DEVICE pointers; every scene has the
 * same canvas (width <= 1024) and `paths_per_scene` closed cubic paths drawn
 * in order.  Path j = scene * paths_per_scene + p owns n = seg_offset[j+1] -
 * seg_offset[j] cubics and the 3n points (x, y) starting at
 * points[2 * 3 * seg_offset[j]]: its start point, then (control 1, control 2,
 * end) per cubic except the last, which has (control 1, control 2) and ends
 * at the start point (closed by construction).  See
 * resvg_gb300/csrc/kernels/soft.cu for the coverage, paint, composite and blur
 * definitions.  Limits: width <= 1024 (4 pixels per thread of a 256-thread
 * row), blur radius 12 (sigma up to 4), at most 512 flattened lines of one path
 * crossing one pixel row (RGPU_ERR_CAPACITY beyond). */
typedef struct rgpu_soft_batch {
    uint32_t scenes, width, height, paths_per_scene;
    uint32_t total_segments;     /* seg_offset[scenes * paths_per_scene] */
    const uint32_t *seg_offset;  /* scenes * paths_per_scene + 1 */
    const float *points;         /* (x, y) pairs as above */
    const uint32_t *paint_kind;  /* per path: 0 solid colour, 1 linear gradient */
    const float *colors;         /* per path: straight RGBA (solid) */
    const float *stop_offsets;   /* per path: 4 ascending offsets (gradient) */
    const float *stop_colors;    /* per path: 4 straight RGBA stop colours */
    const float *grad_line;      /* per path: x1, y1, x2, y2 of the gradient (pad spread) */
    const float *sigma;          /* per scene: Gaussian blur sigma */
    const float *opacity;        /* per path: opacity multiplying the paint's alpha (NULL: 1), as
                                    resvg's fill opacity (crates/resvg/src/path.rs:49) */
} rgpu_soft_batch;
/* Gradients, same layouts as the parameters (device; overwritten).  opacity
 * may be NULL when the batch has no opacity parameter. */
typedef struct rgpu_soft_grads {
    float *points, *colors, *stop_offsets, *stop_colors, *sigma, *opacity;
} rgpu_soft_grads;
/* image = composite (premultiplied RGBA, scenes x height x width x 4 floats),
 * blurred = its Gaussian blur.  Synchronous. */
int rgpu_soft_forward(const rgpu_soft_batch *batch, float *image, float *blurred, void *stream);
/* Vector-Jacobian product: given dL/d(blurred) (same layout), writes dL/d of
 * every parameter.  `image` is the forward's composite.  Coverage is
 * recomputed row by row; scratch is bounded by the number of SMs. */
int rgpu_soft_backward(const rgpu_soft_batch *batch, const float *image, const float *grad_blurred,
                       rgpu_soft_grads *grads, void *stream);
/* Mean squared error over `count` floats: loss (1 float) and, if non-null,
 * dloss/d(blurred). */
int rgpu_soft_mse(const float *blurred, const float *target, size_t count, float *loss, float *grad_blurred,
                  void *stream);

#ifdef __cplusplus
}
#endif
#endif
