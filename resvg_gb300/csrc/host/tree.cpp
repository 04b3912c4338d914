// Host-side render tree (see tree.h).
#include "tree.h"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace rgpu {

int32_t Tree::add_group(int32_t parent, const rgpu_group &g) {
    int32_t id = (int32_t)groups.size();
    groups.push_back(g);
    group_children.emplace_back();
    if (parent >= 0 && parent < id) group_children[parent].push_back(rgpu_node{RGPU_NODE_GROUP, (uint32_t)id});
    finalized = false;
    return id;
}

int32_t Tree::add_path(int32_t parent, const rgpu_path &p0, const uint8_t *v, uint32_t nv, const float *pts,
                       uint32_t npts, const float *dash, uint32_t nd) {
    rgpu_path p = p0;
    p.verb_offset = (uint32_t)verbs.size();
    p.verb_count = nv;
    p.point_offset = (uint32_t)(points.size() / 2);
    p.point_count = npts;
    verbs.insert(verbs.end(), v, v + nv);
    points.insert(points.end(), pts, pts + 2 * (size_t)npts);
    p.dash_offset = (uint32_t)dashes.size();
    p.dash_count = nd;
    if (nd) dashes.insert(dashes.end(), dash, dash + nd);
    int32_t id = (int32_t)paths.size();
    paths.push_back(p);
    if (parent >= 0 && parent < (int32_t)groups.size())
        group_children[parent].push_back(rgpu_node{RGPU_NODE_PATH, (uint32_t)id});
    finalized = false;
    return id;
}

int32_t Tree::add_paint(const rgpu_paint &p0, const rgpu_stop *s, uint32_t ns) {
    rgpu_paint p = p0;
    if (p.kind == RGPU_PAINT_PATTERN || p.kind == RGPU_PAINT_IMAGE) {  // stop_offset names the group / image
        p.stop_count = 0;
        paints.push_back(p);
        return (int32_t)paints.size() - 1;
    }
    p.stop_offset = (uint32_t)stops.size();
    p.stop_count = ns;
    if (ns) stops.insert(stops.end(), s, s + ns);
    paints.push_back(p);
    return (int32_t)paints.size() - 1;
}

int32_t Tree::add_image(uint32_t w, uint32_t h, const uint8_t *rgba) {
    if (!w || !h || !rgba || (uint64_t)w * h > ((uint64_t)1 << 28)) return -1;
    rgpu_image im{w, h, (uint64_t)image_pixels.size()};
    image_pixels.insert(image_pixels.end(), rgba, rgba + (size_t)w * h * 4);
    images.push_back(im);
    return (int32_t)images.size() - 1;
}

int32_t Tree::add_filter(const rgpu_filter &f0, const rgpu_primitive *pr, uint32_t n, const int32_t *merge,
                         uint32_t nm) {
    rgpu_filter f = f0;
    f.prim_offset = (uint32_t)prims.size();
    f.prim_count = n;
    uint32_t merge_base = (uint32_t)merge_inputs.size();
    for (uint32_t i = 0; i < n; i++) {
        rgpu_primitive q = pr[i];
        if (q.kind == RGPU_FE_MERGE) q.i[0] += (int32_t)merge_base;
        prims.push_back(q);
    }
    if (nm) merge_inputs.insert(merge_inputs.end(), merge, merge + nm);
    filters.push_back(f);
    return (int32_t)filters.size() - 1;
}

bool Tree::set_node_id(uint32_t kind, uint32_t index, const char *id) {
    std::vector<std::string> *ids = kind == RGPU_NODE_GROUP ? &group_ids : kind == RGPU_NODE_PATH ? &path_ids : nullptr;
    const size_t count = kind == RGPU_NODE_GROUP ? groups.size() : paths.size();
    if (!ids || index >= count || !id) return false;
    if (ids->size() < count) ids->resize(count);
    (*ids)[index] = id;
    return true;
}

bool Tree::node_by_id(const char *id, uint32_t *kind, uint32_t *index) const {
    if (!id || !*id || groups.empty()) return false;
    auto id_of = [&](const rgpu_node &n) -> const std::string * {
        const std::vector<std::string> &ids = n.kind == RGPU_NODE_GROUP ? group_ids : path_ids;
        return n.index < ids.size() ? &ids[n.index] : nullptr;
    };
    // explicit stack of (group, next child) for the pre-order walk
    std::vector<std::pair<uint32_t, size_t>> stack{{0u, (size_t)0}};
    while (!stack.empty()) {
        auto &top = stack.back();
        const std::vector<rgpu_node> &ch = group_children[top.first];
        if (top.second >= ch.size()) { stack.pop_back(); continue; }
        const rgpu_node n = ch[top.second++];
        const std::string *nid = id_of(n);
        if (nid && *nid == id) {
            *kind = n.kind;
            *index = n.index;
            return true;
        }
        if (n.kind == RGPU_NODE_GROUP && n.index < group_children.size()) stack.push_back({n.index, (size_t)0});
    }
    return false;
}

bool stroke_outline_view(const rgpu_tree_view &t, uint32_t pi, float res_scale, PathData &out) {
    const rgpu_path &p = t.paths[pi];
    if (p.stroke_paint < 0 || !(p.stroke_width > 0)) return false;
    const uint8_t *v = t.verbs + p.verb_offset;
    const float *pts = t.points + 2 * (size_t)p.point_offset;
    StrokeStyle st;
    st.width = p.stroke_width;
    st.miter_limit = p.miter_limit;
    st.cap = p.line_cap;
    st.join = p.line_join;
    if (p.dash_count) {
        PathData dashed;
        if (dash_path(v, p.verb_count, pts, p.point_count, t.dashes + p.dash_offset, p.dash_count, p.dash_phase,
                      res_scale, dashed)) {
            if (dashed.empty()) return false;
            return stroke_path(dashed.verbs.data(), dashed.verbs.size(), dashed.pts.data(), dashed.pts.size() / 2, st,
                               res_scale, out);
        }
    }
    return stroke_path(v, p.verb_count, pts, p.point_count, st, res_scale, out);
}

bool hairline_source_view(const rgpu_tree_view &t, uint32_t pi, float res_scale, PathData &out) {
    const rgpu_path &p = t.paths[pi];
    const uint8_t *v = t.verbs + p.verb_offset;
    const float *pts = t.points + 2 * (size_t)p.point_offset;
    if (p.dash_count) {
        PathData dashed;
        if (dash_path(v, p.verb_count, pts, p.point_count, t.dashes + p.dash_offset, p.dash_count, p.dash_phase,
                      res_scale, dashed)) {
            if (dashed.empty()) return false;
            out = std::move(dashed);
            return true;
        }
    }
    out.verbs.assign(v, v + p.verb_count);
    out.pts.assign(pts, pts + 2 * (size_t)p.point_count);
    return !out.verbs.empty();
}

std::shared_ptr<PathData> Tree::cached_stroke_outline(uint32_t pi, float rs, bool *found) {
    uint32_t bits;
    std::memcpy(&bits, &rs, 4);
    std::lock_guard<std::mutex> g(cache_mu);
    auto it = stroke_cache.find(std::make_pair(pi, bits));
    *found = it != stroke_cache.end();
    return *found ? it->second : nullptr;
}

void Tree::store_stroke_outline(uint32_t pi, float rs, std::shared_ptr<PathData> out) {
    uint32_t bits;
    std::memcpy(&bits, &rs, 4);
    std::lock_guard<std::mutex> g(cache_mu);
    stroke_cache[std::make_pair(pi, bits)] = std::move(out);
}

std::shared_ptr<PathData> Tree::stroke_outline(uint32_t pi, float rs) {
    uint32_t bits;
    std::memcpy(&bits, &rs, 4);
    auto key = std::make_pair(pi, bits);
    {
        std::lock_guard<std::mutex> g(cache_mu);
        auto it = stroke_cache.find(key);
        if (it != stroke_cache.end()) return it->second;
    }
    auto out = std::make_shared<PathData>();
    // a finalised tree's view is read-only: trees are flattened concurrently
    const rgpu_tree_view *tv = finalized ? &view : get_view();
    if (!stroke_outline_view(*tv, pi, rs, *out)) out.reset();
    std::lock_guard<std::mutex> g(cache_mu);
    stroke_cache[key] = out;
    return out;
}

static void bbox_expand(float b[4], bool &has, const float r[4]) {
    if (!has) { std::memcpy(b, r, 16); has = true; return; }
    float l = std::min(b[0], r[0]), t = std::min(b[1], r[1]);
    float rr = std::max(b[0] + b[2], r[0] + r[2]), bb = std::max(b[1] + b[3], r[1] + r[3]);
    b[0] = l; b[1] = t; b[2] = rr - l; b[3] = bb - t;
}

static bool bbox_transform(const float r[4], const rgpu_transform &ts, float out[4]) {
    float xs[4] = {r[0], r[0] + r[2], r[0] + r[2], r[0]}, ys[4] = {r[1], r[1], r[1] + r[3], r[1] + r[3]};
    float l = 1e30f, t = 1e30f, rr = -1e30f, b = -1e30f;
    for (int i = 0; i < 4; i++) {
        float x = xs[i] * ts.sx + ys[i] * ts.kx + ts.tx, y = xs[i] * ts.ky + ys[i] * ts.sy + ts.ty;
        l = std::min(l, x); rr = std::max(rr, x); t = std::min(t, y); b = std::max(b, y);
    }
    out[0] = l; out[1] = t; out[2] = rr - l; out[3] = b - t;
    return std::isfinite(l) && std::isfinite(t) && std::isfinite(rr) && std::isfinite(b);
}

bool Tree::finalize() {
    // flatten child lists
    children.clear();
    for (size_t g = 0; g < groups.size(); g++) {
        groups[g].child_offset = (uint32_t)children.size();
        groups[g].child_count = (uint32_t)group_children[g].size();
        children.insert(children.end(), group_children[g].begin(), group_children[g].end());
    }
    get_view();
    // path bboxes: stroke outline bounds, else fill bounds (usvg Path::new)
    for (size_t i = 0; i < paths.size(); i++) {
        rgpu_path &p = paths[i];
        float b[4] = {0, 0, 0, 0};
        bool ok = tight_bounds(verbs.data() + p.verb_offset, p.verb_count, points.data() + 2 * (size_t)p.point_offset,
                               p.point_count, b);
        if (p.stroke_paint >= 0 && p.stroke_width > 0) {
            PathData sp;
            StrokeStyle st;
            st.width = p.stroke_width; st.miter_limit = p.miter_limit; st.cap = p.line_cap; st.join = p.line_join;
            float sb[4];
            if (stroke_path(verbs.data() + p.verb_offset, p.verb_count, points.data() + 2 * (size_t)p.point_offset,
                            p.point_count, st, 1.0f, sp) &&
                tight_bounds(sp.verbs.data(), sp.verbs.size(), sp.pts.data(), sp.pts.size() / 2, sb)) {
                std::memcpy(b, sb, 16);
                ok = true;
            }
        }
        if (!ok) { b[0] = b[1] = b[2] = b[3] = 0; }
        p.bbox_x = b[0]; p.bbox_y = b[1]; p.bbox_w = b[2]; p.bbox_h = b[3];
    }
    // group layer bboxes, children before parents: groups are added parent
    // first, so a reverse sweep visits every child group before its parent.
    for (size_t gi = groups.size(); gi-- > 0;) {
        rgpu_group &g = groups[gi];
        float lb[4] = {0, 0, 0, 0};
        bool has = false;
        for (auto &c : group_children[gi]) {
            if (c.kind == RGPU_NODE_PATH) {
                const rgpu_path &p = paths[c.index];
                if (p.bbox_w > 0 || p.bbox_h > 0) {
                    float r[4] = {p.bbox_x, p.bbox_y, p.bbox_w, p.bbox_h};
                    bbox_expand(lb, has, r);
                }
            } else {
                const rgpu_group &cg = groups[c.index];
                if (!cg.has_layer_bbox) continue;
                float r[4] = {cg.layer_x, cg.layer_y, cg.layer_w, cg.layer_h}, tr[4];
                if (bbox_transform(r, cg.transform, tr)) bbox_expand(lb, has, tr);
            }
        }
        if (g.filter_count) {
            float fb[4];
            bool fh = false;
            for (uint32_t k = 0; k < g.filter_count; k++) {
                const rgpu_filter &f = filters[filter_refs[g.filter_offset + k]];
                float r[4] = {f.x, f.y, f.w, f.h};
                bbox_expand(fb, fh, r);
            }
            if (fh && fb[2] > 0 && fb[3] > 0) { std::memcpy(lb, fb, 16); has = true; }
        }
        g.has_layer_bbox = (has && lb[2] > 0 && lb[3] > 0) ? 1 : 0;
        g.layer_x = lb[0]; g.layer_y = lb[1]; g.layer_w = lb[2]; g.layer_h = lb[3];
    }
    finalized = true;
    get_view();
    return true;
}

const rgpu_tree_view *Tree::get_view() {
    view.width = width; view.height = height;
    view.groups = groups.data(); view.group_count = (uint32_t)groups.size();
    view.children = children.data(); view.child_count = (uint32_t)children.size();
    view.paths = paths.data(); view.path_count = (uint32_t)paths.size();
    view.verbs = verbs.data(); view.verb_count = (uint32_t)verbs.size();
    view.points = points.data(); view.point_count = (uint32_t)(points.size() / 2);
    view.paints = paints.data(); view.paint_count = (uint32_t)paints.size();
    view.stops = stops.data(); view.stop_count = (uint32_t)stops.size();
    view.dashes = dashes.data(); view.dash_count = (uint32_t)dashes.size();
    view.clips = clips.data(); view.clip_count = (uint32_t)clips.size();
    view.masks = masks.data(); view.mask_count = (uint32_t)masks.size();
    view.filter_refs = filter_refs.data(); view.filter_ref_count = (uint32_t)filter_refs.size();
    view.filters = filters.data(); view.filter_count = (uint32_t)filters.size();
    view.prims = prims.data(); view.prim_count = (uint32_t)prims.size();
    view.merge_inputs = merge_inputs.data(); view.merge_input_count = (uint32_t)merge_inputs.size();
    view.images = images.data(); view.image_count = (uint32_t)images.size();
    view.image_pixels = image_pixels.data(); view.image_pixel_bytes = (uint64_t)image_pixels.size();
    return &view;
}

}  // namespace rgpu
