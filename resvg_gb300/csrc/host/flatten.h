// Host flattener: walks a render tree the way resvg's renderer does
// (crates/resvg/src/render.rs:10-142, path.rs:6-177, clip.rs:6-98,
// mask.rs:6-46) and emits device records (draws, paints, gradients, layers)
// and the band VM's command streams instead of rasterising.
//
// A group with filters (render.rs:113-117) splits the work: its content is
// flattened into a stream of its own that renders into an internal surface at
// an earlier dependency level, a FilterJob runs the filter chain on that
// surface (filter_exec.cpp), and the parent stream pushes a layer initialised
// from the job's result before applying clip, mask and the composite.
#pragma once
#include <string>
#include <vector>
#include "../device_types.h"
#include "tree.h"
#include "xform.h"

namespace rgpu {

struct SurfaceReq {
    int32_t w, h;
    const uint8_t *init = nullptr;  // host pixels copied in at upload (raster images)
};

struct FilterJob {
    uint32_t content;               // surface with the rendered group content (SourceGraphic)
    uint32_t result;                // surface receiving the filtered layer
    int32_t w, h;
    Xf ts;                          // the layer's transform (filter regions are mapped with it)
    const rgpu_tree_view *tree;
    uint32_t filter_ref_offset, filter_count;
    uint32_t level;                 // runs after the raster pass of this level
    uint32_t image_first, image_count;  // its feImage renders in SceneBuild::fe_images
};

// A pattern or raster-image fill: its tile is rendered by a stream into `tile`
// (tw x th), or holds the image's pixels; after that stream's raster pass, the shader (inverse transform `inv`, nearest or
// bicubic, opacity) is evaluated per layer pixel of (bx, by, bw, bh) into the
// float4 surface `shade`, which the draw's ImageRec (GradRec slot `grad`)
// points to.
struct PatternReq {
    uint32_t grad, tile;
    int32_t tw, th;
    uint32_t shade;
    int32_t bx, by, bw, bh;
    Xf inv;
    int32_t quality;   // 0 nearest, 1 bilinear, 2 bicubic
    int32_t repeat;    // 1 repeat (patterns), 0 pad (raster images)
    float opacity;
    uint32_t level;
};

// A feImage primitive's element, rendered into its own surface before the job.
struct FeImageReq {
    uint32_t prim;     // global primitive index
    uint32_t surface;
};

// A device stroke job's entry in its tree's outline cache: once the device
// has built the outline, later flattens of the tree reuse it.
struct StrokeKey {
    Tree *tree;
    uint32_t path;
    float res_scale;
};

struct StreamBuild {
    std::vector<DrawRec> draws;     // seg_base / tpt_base / stream assigned on append
    std::vector<StrokeJob> strokes; // draw = index within this stream; outline slices set by the plan
    std::vector<StrokeKey> stroke_keys;  // per stroke job: where its outline is cached
    std::vector<Cmd> cmds;          // FILL / APPLY_REGION: a = draw index within this stream
    std::vector<LayerRec> layers;
    int32_t out_w = 0, out_h = 0;
    uint32_t stride = 0;
    uint64_t out_ptr = 0;
    int32_t surface = -1;
    uint32_t max_depth = 0;
    uint32_t level = 0;
};

struct SceneBuild {
    std::vector<DrawRec> draws;
    std::vector<PaintRec> paints;
    std::vector<GradRec> grads;
    std::vector<LayerRec> layers;
    std::vector<Cmd> cmds;
    std::vector<StreamRec> streams;
    std::vector<SurfaceReq> surfaces;
    std::vector<FilterJob> jobs;
    std::vector<FeImageReq> fe_images;
    std::vector<PatternReq> patterns;
    std::vector<HairRec> hairs;       // anti-aliased hairline strokes
    std::vector<HairSpan> hair_spans;
    std::vector<uint32_t> fill_cmds;  // per stream: its fill / region command indices (plan_scene)
    std::vector<uint8_t> verbs;
    std::vector<float> pts;
    std::vector<StrokeJob> stroke_jobs;  // paths stroked on the device (their draws carry DRAW_STROKED)
    std::vector<StrokeKey> stroke_keys;  // per job: the tree outline cache entry it fills
    std::vector<float> dashes;           // dash intervals of the stroke jobs
    uint64_t nsegs = 0, ntpts = 0;
    uint32_t max_level = 0;
    std::string error;

    // Appends one tree rendered onto a device surface (`out_ptr`, `stride`,
    // size w x h); returns the index of its output stream or -1.
    int add_tree(Tree &tree, const Xf &ts, int32_t w, int32_t h, uint64_t out_ptr, uint32_t stride);
    // Appends one node of a tree (render::render_node, crates/resvg/src/render.rs:31-46:
    // a group through render_group, a path through path::render) with `ts` as
    // its parent transform; node_kind is RGPU_NODE_GROUP or RGPU_NODE_PATH.
    int add_node(Tree &tree, uint32_t node_kind, uint32_t node_index, const Xf &ts, int32_t w, int32_t h,
                 uint64_t out_ptr, uint32_t stride);
    // internal: concatenates a finished stream
    uint32_t append_stream(StreamBuild &sbd);
    // Appends other builds in order (their trees after this one's), moving
    // every index their records hold, on up to `threads` host threads; lets
    // trees be flattened on separate threads.
    void merge(std::vector<SceneBuild> &parts, unsigned threads);
};

// Where stroke outlines are built: on the device by kernels/stroke.cu (the
// default) or on the host by stroke.cpp (the same stroker source).
void set_device_stroke(bool on);
bool device_stroke_enabled();

}  // namespace rgpu
