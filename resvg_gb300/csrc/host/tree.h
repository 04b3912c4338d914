// Host-side render tree: the resolved-SVG input both renderers consume.
//
// Stands in for `usvg::Tree` (crates/usvg/src/tree/mod.rs): it owns the
// arrays behind `rgpu_tree_view` (include/rgpu_tree.h) and computes, at
// finalize time, what usvg precomputes while building its tree: path stroke
// bounding boxes (tree/mod.rs:1321-1338,1443-1456) and group layer bounding
// boxes (tree/mod.rs:1866-1929).  Stroke outlines are cached per resolution
// scale so repeated renders of one tree do not re-stroke.
#pragma once
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <vector>
#include "rgpu_tree.h"
#include "geom.h"

namespace rgpu {

struct Tree {
    float width = 0, height = 0;
    std::vector<rgpu_group> groups;
    std::vector<std::vector<rgpu_node>> group_children;
    std::vector<rgpu_node> children;
    std::vector<rgpu_path> paths;
    std::vector<uint8_t> verbs;
    std::vector<float> points;
    std::vector<rgpu_paint> paints;
    std::vector<rgpu_stop> stops;
    std::vector<float> dashes;
    std::vector<rgpu_clip> clips;
    std::vector<rgpu_mask> masks;
    std::vector<uint32_t> filter_refs;
    std::vector<rgpu_filter> filters;
    std::vector<rgpu_primitive> prims;
    std::vector<int32_t> merge_inputs;
    std::vector<rgpu_image> images;
    std::vector<uint8_t> image_pixels;
    rgpu_tree_view view{};
    bool finalized = false;
    // SVG ids of groups and paths ("" = none), for resvg_render_node's lookup
    std::vector<std::string> group_ids, path_ids;

    // stroke outline cache: (path index, res_scale bits) -> outline
    std::mutex cache_mu;
    std::map<std::pair<uint32_t, uint32_t>, std::shared_ptr<PathData>> stroke_cache;

    int32_t add_group(int32_t parent, const rgpu_group &g);
    int32_t add_path(int32_t parent, const rgpu_path &p, const uint8_t *v, uint32_t nv, const float *pts,
                     uint32_t npts, const float *dash, uint32_t nd);
    int32_t add_paint(const rgpu_paint &p, const rgpu_stop *s, uint32_t ns);
    int32_t add_image(uint32_t w, uint32_t h, const uint8_t *rgba);
    int32_t add_filter(const rgpu_filter &f, const rgpu_primitive *pr, uint32_t n, const int32_t *merge, uint32_t nm);
    bool finalize();
    const rgpu_tree_view *get_view();
    // Gives node (kind, index) an SVG id; false for an unknown node.
    bool set_node_id(uint32_t kind, uint32_t index, const char *id);
    // usvg's Tree::node_by_id (crates/usvg/src/tree/mod.rs:1629-1635,1718-1732):
    // the first node, in depth-first pre-order over the root group's
    // descendants, whose id equals `id`; an empty id matches nothing.
    bool node_by_id(const char *id, uint32_t *kind, uint32_t *index) const;

    // Stroke outline of path `pi` (dashing applied) at resolution scale `rs`;
    // null when the stroke produces nothing.
    std::shared_ptr<PathData> stroke_outline(uint32_t pi, float rs);
    // The cached outline without computing one: *found tells a cached "no
    // outline" (nullptr) from a miss.  store_* fills the cache (outlines the
    // device built).
    std::shared_ptr<PathData> cached_stroke_outline(uint32_t pi, float rs, bool *found);
    void store_stroke_outline(uint32_t pi, float rs, std::shared_ptr<PathData> out);
};

// Stroke outline for a path of any tree view (used by the oracle too).
bool stroke_outline_view(const rgpu_tree_view &t, uint32_t pi, float res_scale, PathData &out);
// The path a hairline stroke draws: the dashed path when the stroke is dashed
// (false when dashing leaves nothing), else the path itself.
bool hairline_source_view(const rgpu_tree_view &t, uint32_t pi, float res_scale, PathData &out);

}  // namespace rgpu
