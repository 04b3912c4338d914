// C ABI: tree building and generators (see include/resvg_gpu.h).
#include <cstring>
#include "resvg_gpu.h"
#include "tree.h"

struct rgpu_tree : rgpu::Tree {};

namespace rgpu {
Tree *generate_scene(int config, uint64_t seed, uint64_t index, float scale);
}

extern "C" {

resvg_render_tree *rgpu_tree_new(float width, float height) {
    if (!(width > 0) || !(height > 0)) return nullptr;
    rgpu_tree *t = new rgpu_tree();
    t->width = width;
    t->height = height;
    return t;
}

void rgpu_tree_free(resvg_render_tree *tree) { delete tree; }

int32_t rgpu_tree_add_group(resvg_render_tree *t, int32_t parent, const rgpu_group *g) {
    if (!t || !g) return -1;
    return t->add_group(parent, *g);
}

int32_t rgpu_tree_add_path(resvg_render_tree *t, int32_t parent, const rgpu_path *p, const uint8_t *verbs,
                           uint32_t nv, const float *pts, uint32_t npts, const float *dashes, uint32_t nd) {
    if (!t || !p || (nv && !verbs) || (npts && !pts)) return -1;
    return t->add_path(parent, *p, verbs, nv, pts, npts, dashes, nd);
}

int32_t rgpu_tree_add_paint(resvg_render_tree *t, const rgpu_paint *p, const rgpu_stop *stops, uint32_t n) {
    if (!t || !p) return -1;
    return t->add_paint(*p, stops, n);
}

int32_t rgpu_tree_add_clip(resvg_render_tree *t, const rgpu_clip *c) {
    if (!t || !c) return -1;
    t->clips.push_back(*c);
    return (int32_t)t->clips.size() - 1;
}

int32_t rgpu_tree_add_mask(resvg_render_tree *t, const rgpu_mask *m) {
    if (!t || !m) return -1;
    t->masks.push_back(*m);
    return (int32_t)t->masks.size() - 1;
}

int32_t rgpu_tree_add_filter(resvg_render_tree *t, const rgpu_filter *f, const rgpu_primitive *prims, uint32_t n,
                             const int32_t *merge, uint32_t nm) {
    if (!t || !f || (n && !prims)) return -1;
    return t->add_filter(*f, prims, n, merge, nm);
}

int32_t rgpu_tree_add_image(resvg_render_tree *t, uint32_t w, uint32_t h, const uint8_t *rgba) {
    if (!t) return -1;
    return t->add_image(w, h, rgba);
}

int rgpu_tree_set_node_id(resvg_render_tree *t, uint32_t node_kind, uint32_t index, const char *id) {
    if (!t || !id) return RGPU_ERR_INVALID_ARG;
    return t->set_node_id(node_kind, index, id) ? RGPU_OK : RGPU_ERR_INVALID_ARG;
}

int rgpu_tree_find_node(const resvg_render_tree *t, const char *id, uint32_t *node_kind, uint32_t *index) {
    if (!t || !id || !node_kind || !index) return RGPU_ERR_INVALID_ARG;
    return t->node_by_id(id, node_kind, index) ? RGPU_OK : RGPU_ERR_INVALID_ARG;
}

int rgpu_tree_set_group_filters(resvg_render_tree *t, int32_t group, const uint32_t *filters, uint32_t count) {
    if (!t || group < 0 || group >= (int32_t)t->groups.size()) return RGPU_ERR_INVALID_ARG;
    t->groups[group].filter_offset = (uint32_t)t->filter_refs.size();
    t->groups[group].filter_count = count;
    for (uint32_t i = 0; i < count; i++) t->filter_refs.push_back(filters[i]);
    t->finalized = false;
    return RGPU_OK;
}

int rgpu_tree_finalize(resvg_render_tree *t) {
    if (!t) return RGPU_ERR_INVALID_ARG;
    return t->finalize() ? RGPU_OK : RGPU_ERR_INVALID_ARG;
}

const rgpu_tree_view *rgpu_tree_get_view(resvg_render_tree *t) {
    if (!t) return nullptr;
    if (!t->finalized) t->finalize();
    return t->get_view();
}

resvg_render_tree *rgpu_tree_generate(int config, uint64_t seed, uint64_t index, float scale) {
    rgpu::Tree *g = rgpu::generate_scene(config, seed, index, scale);
    if (!g) return nullptr;
    // rgpu_tree adds no members: move the generated tree into the ABI type.
    rgpu_tree *t = new rgpu_tree();
    t->width = g->width; t->height = g->height;
    t->groups = std::move(g->groups); t->group_children = std::move(g->group_children);
    t->children = std::move(g->children); t->paths = std::move(g->paths);
    t->verbs = std::move(g->verbs); t->points = std::move(g->points);
    t->paints = std::move(g->paints); t->stops = std::move(g->stops); t->dashes = std::move(g->dashes);
    t->clips = std::move(g->clips); t->masks = std::move(g->masks);
    t->filter_refs = std::move(g->filter_refs); t->filters = std::move(g->filters);
    t->prims = std::move(g->prims); t->merge_inputs = std::move(g->merge_inputs);
    t->images = std::move(g->images); t->image_pixels = std::move(g->image_pixels);
    t->group_ids = std::move(g->group_ids); t->path_ids = std::move(g->path_ids);
    t->finalized = g->finalized;
    delete g;
    t->get_view();
    return t;
}

}  // extern "C"
