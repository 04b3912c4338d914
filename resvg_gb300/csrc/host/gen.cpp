// Seeded synthetic scene generators for the benchmark workloads.
//
// resvg publishes no benchmark scenes; these generate trees with the shapes,
// sizes and value distributions of the workloads the backend is measured on:
//   0: 512x512, 200 closed cubic loops (4-16 segments), solid colours,
//      opacity U[0.3,1], fill rule alternating non-zero / even-odd.
//   1: 1024x1024, 2000 gradient fills (half linear, half radial; 2-8 stops;
//      pad/reflect/repeat; random affine gradientTransform) + 500 stroked
//      open cubics (width U[0.5,8], round|miter join, butt|round cap) + 20
//      nested clip groups (6-vertex polygons) + 10 luminance-masked groups.
//   2: 2048x2048, 500 loops inside a group with the filter chain
//      blur -> saturate -> morphology -> arithmetic composite, linearRGB.
//   3: one scene of the batch: side log-uniform 64..1024, path count
//      log-uniform 10..2000, config-1 paint mix with 20% strokes, 10% of
//      scenes with one clip + one Gaussian blur (sigma U[1,8]).
// The same generator feeds the GPU path, the oracle and the CPU baseline.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "tree.h"

namespace rgpu {
namespace {
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uf() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }  // [0,1)
    float uf(float a, float b) { return a + (b - a) * uf(); }
    int ui(int a, int b) { return a + (int)(next() % (uint64_t)(b - a + 1)); }  // inclusive
    uint8_t u8() { return (uint8_t)(next() >> 56); }
};

rgpu_transform ident() { return rgpu_transform{1, 0, 0, 1, 0, 0}; }

rgpu_group plain_group() {
    rgpu_group g{};
    g.transform = ident();
    g.opacity = 1.0f;
    g.blend = RGPU_BLEND_SOURCE_OVER;
    g.clip_path = -1;
    g.mask = -1;
    return g;
}

rgpu_path base_path() {
    rgpu_path p{};
    p.fill_paint = -1;
    p.stroke_paint = -1;
    p.fill_opacity = 1.0f;
    p.stroke_opacity = 1.0f;
    p.stroke_width = 1.0f;
    p.miter_limit = 4.0f;
    p.anti_alias = 1;
    p.visible = 1;
    return p;
}

void cubic_loop(Rng &r, float w, float h, std::vector<uint8_t> &v, std::vector<float> &pts) {
    int nseg = r.ui(4, 16);
    float x0 = r.uf(0, w), y0 = r.uf(0, h);
    v.push_back(RGPU_MOVE);
    pts.insert(pts.end(), {x0, y0});
    for (int s = 0; s < nseg; s++) {
        v.push_back(RGPU_CUBIC);
        float c1x = r.uf(0, w), c1y = r.uf(0, h), c2x = r.uf(0, w), c2y = r.uf(0, h);
        float ex = s + 1 == nseg ? x0 : r.uf(0, w), ey = s + 1 == nseg ? y0 : r.uf(0, h);
        pts.insert(pts.end(), {c1x, c1y, c2x, c2y, ex, ey});
    }
    v.push_back(RGPU_CLOSE);
}

void open_cubic(Rng &r, float w, float h, std::vector<uint8_t> &v, std::vector<float> &pts) {
    int nseg = r.ui(1, 3);
    v.push_back(RGPU_MOVE);
    pts.insert(pts.end(), {r.uf(0, w), r.uf(0, h)});
    for (int s = 0; s < nseg; s++) {
        v.push_back(RGPU_CUBIC);
        for (int k = 0; k < 3; k++) pts.insert(pts.end(), {r.uf(0, w), r.uf(0, h)});
    }
}

void polygon6(Rng &r, float w, float h, std::vector<uint8_t> &v, std::vector<float> &pts) {
    v.push_back(RGPU_MOVE);
    // a random 6-vertex polygon around a centre, so that nested clips keep
    // a usable area
    float cx = r.uf(0.3f * w, 0.7f * w), cy = r.uf(0.3f * h, 0.7f * h);
    for (int i = 0; i < 6; i++) {
        float a = (float)(i * 2.0 * M_PI / 6.0) + r.uf(-0.4f, 0.4f);
        float rad = r.uf(0.35f, 0.6f) * std::min(w, h);
        if (i) v.push_back(RGPU_LINE);
        pts.insert(pts.end(), {cx + rad * std::cos(a), cy + rad * std::sin(a)});
    }
    v.push_back(RGPU_CLOSE);
}

int32_t solid_paint(Tree &t, Rng &r) {
    rgpu_paint p{};
    p.kind = RGPU_PAINT_SOLID;
    p.r = r.u8(); p.g = r.u8(); p.b = r.u8();
    p.transform = ident();
    return t.add_paint(p, nullptr, 0);
}

int32_t gradient_paint(Tree &t, Rng &r, float w, float h, bool radial) {
    rgpu_paint p{};
    p.kind = radial ? RGPU_PAINT_RADIAL : RGPU_PAINT_LINEAR;
    p.spread = (uint32_t)r.ui(0, 2);
    if (radial) {
        p.cx = r.uf(0, w); p.cy = r.uf(0, h);
        p.r_ = r.uf(0.05f, 0.5f) * std::max(w, h);
        p.fx = p.cx; p.fy = p.cy; p.fr = 0;
    } else {
        p.x1 = r.uf(0, w); p.y1 = r.uf(0, h); p.x2 = r.uf(0, w); p.y2 = r.uf(0, h);
    }
    // random affine gradientTransform about the canvas centre
    float th = r.uf(0, 6.2831853f), sx = r.uf(0.5f, 1.5f), sy = r.uf(0.5f, 1.5f), k = r.uf(-0.3f, 0.3f);
    float c = std::cos(th), s = std::sin(th);
    // M = R * [[sx, k*sy],[0, sy]]
    float a = c * sx, b = s * sx, cc = c * k * sy - s * sy, d = s * k * sy + c * sy;
    float cx = 0.5f * w, cy = 0.5f * h;
    p.transform = rgpu_transform{a, b, cc, d, cx - (a * cx + cc * cy), cy - (b * cx + d * cy)};
    int n = r.ui(2, 8);
    std::vector<float> offs(n);
    for (int i = 0; i < n; i++) offs[i] = r.uf();
    std::sort(offs.begin(), offs.end());
    std::vector<rgpu_stop> st(n);
    for (int i = 0; i < n; i++) {
        st[i].offset = offs[i];
        st[i].r = r.u8(); st[i].g = r.u8(); st[i].b = r.u8();
        st[i].opacity = r.uf(0.3f, 1.0f);
    }
    // usvg stop normalisation: strictly increasing offsets
    for (int i = 1; i < n; i++)
        if (st[i - 1].offset >= st[i].offset) st[i - 1].offset = std::max(0.0f, st[i].offset - 1.1920929e-7f);
    return t.add_paint(p, st.data(), (uint32_t)n);
}

void add_fill(Tree &t, int32_t parent, Rng &r, float w, float h, int paint_kind, uint32_t rule) {
    std::vector<uint8_t> v;
    std::vector<float> pts;
    cubic_loop(r, w, h, v, pts);
    rgpu_path p = base_path();
    p.fill_rule = rule;
    p.fill_opacity = r.uf(0.3f, 1.0f);
    p.fill_paint = paint_kind == 0 ? solid_paint(t, r) : gradient_paint(t, r, w, h, paint_kind == 2);
    t.add_path(parent, p, v.data(), (uint32_t)v.size(), pts.data(), (uint32_t)pts.size() / 2, nullptr, 0);
}

void add_stroke(Tree &t, int32_t parent, Rng &r, float w, float h) {
    std::vector<uint8_t> v;
    std::vector<float> pts;
    open_cubic(r, w, h, v, pts);
    rgpu_path p = base_path();
    p.stroke_paint = solid_paint(t, r);
    p.stroke_opacity = r.uf(0.3f, 1.0f);
    p.stroke_width = r.uf(0.5f, 8.0f);
    p.line_join = r.ui(0, 1) ? RGPU_JOIN_ROUND : RGPU_JOIN_MITER;
    p.line_cap = r.ui(0, 1) ? RGPU_CAP_ROUND : RGPU_CAP_BUTT;
    t.add_path(parent, p, v.data(), (uint32_t)v.size(), pts.data(), (uint32_t)pts.size() / 2, nullptr, 0);
}

int32_t add_clip(Tree &t, Rng &r, float w, float h) {
    rgpu_group root = plain_group();
    int32_t rg = t.add_group(-1, root);
    std::vector<uint8_t> v;
    std::vector<float> pts;
    polygon6(r, w, h, v, pts);
    rgpu_path p = base_path();
    rgpu_paint black{};
    black.kind = RGPU_PAINT_SOLID;
    black.transform = ident();
    p.fill_paint = t.add_paint(black, nullptr, 0);
    t.add_path(rg, p, v.data(), (uint32_t)v.size(), pts.data(), (uint32_t)pts.size() / 2, nullptr, 0);
    rgpu_clip c{};
    c.transform = ident();
    c.clip_path = -1;
    c.root = (uint32_t)rg;
    t.clips.push_back(c);
    return (int32_t)t.clips.size() - 1;
}

// the config-1 paint mix: fills (solid / linear / radial) and strokes
void add_mixed(Tree &t, int32_t parent, Rng &r, float w, float h, float stroke_frac, bool allow_solid) {
    if (r.uf() < stroke_frac) { add_stroke(t, parent, r, w, h); return; }
    int kind = allow_solid ? r.ui(0, 2) : r.ui(1, 2);
    add_fill(t, parent, r, w, h, kind, (uint32_t)r.ui(0, 1));
}

void gen_config0(Tree &t, Rng &r, float side, int npaths) {
    t.width = t.height = side;
    int32_t root = t.add_group(-1, plain_group());
    (void)root;
    for (int i = 0; i < npaths; i++) add_fill(t, 0, r, side, side, 0, (uint32_t)(i & 1));
}

void gen_config1(Tree &t, Rng &r, float side, int nfill, int nstroke, int nclip, int nmask) {
    t.width = t.height = side;
    t.add_group(-1, plain_group());
    int total = nfill + nstroke;
    std::vector<uint8_t> is_stroke(total, 0);
    for (int i = 0; i < nstroke; i++) is_stroke[i] = 1;
    for (int i = total - 1; i > 0; i--) std::swap(is_stroke[i], is_stroke[r.ui(0, i)]);
    int chunks = 1 + nclip + nmask;
    int k = 0;
    auto emit = [&](int32_t parent, int count) {
        for (int i = 0; i < count && k < total; i++, k++) {
            if (is_stroke[k]) add_stroke(t, parent, r, side, side);
            else add_fill(t, parent, r, side, side, 1 + (k & 1), (uint32_t)r.ui(0, 1));
        }
    };
    int per = total / chunks;
    emit(0, per);
    int32_t parent = 0;
    for (int c = 0; c < nclip; c++) {
        rgpu_group g = plain_group();
        g.clip_path = add_clip(t, r, side, side);
        int32_t gi = t.add_group(parent, g);
        emit(gi, per);
        parent = gi;
    }
    for (int m = 0; m < nmask; m++) {
        int32_t mroot = t.add_group(-1, plain_group());
        for (int i = 0; i < 5; i++) add_fill(t, mroot, r, side, side, 1 + (i & 1), (uint32_t)(i & 1));
        rgpu_mask mk{};
        mk.x = 0; mk.y = 0; mk.w = side; mk.h = side;
        mk.kind = RGPU_MASK_LUMINANCE;
        mk.mask = -1;
        mk.root = (uint32_t)mroot;
        t.masks.push_back(mk);
        rgpu_group g = plain_group();
        g.mask = (int32_t)t.masks.size() - 1;
        int32_t gi = t.add_group(0, g);
        emit(gi, m + 1 == nmask ? total - k : per);
    }
    if (k < total) emit(0, total - k);
}

void add_filter_group(Tree &t, int32_t parent, Rng &r, float side, const std::vector<rgpu_primitive> &prims,
                      float rx, float ry, float rw, float rh, int32_t clip, std::vector<int32_t> *out_group) {
    rgpu_filter f{};
    f.x = rx; f.y = ry; f.w = rw; f.h = rh;
    int32_t fi = t.add_filter(f, prims.data(), (uint32_t)prims.size(), nullptr, 0);
    rgpu_group g = plain_group();
    g.filter_offset = (uint32_t)t.filter_refs.size();
    g.filter_count = 1;
    t.filter_refs.push_back((uint32_t)fi);
    g.clip_path = clip;
    int32_t gi = t.add_group(parent, g);
    if (out_group) out_group->push_back(gi);
    (void)r; (void)side;
}

void gen_config2(Tree &t, Rng &r, float side, int npaths) {
    t.width = t.height = side;
    t.add_group(-1, plain_group());
    // filter region: objectBoundingBox default -10%/120% of the content bbox;
    // the content spans the canvas, so the region is that of the canvas.
    float rx = -0.1f * side, ry = -0.1f * side, rw = 1.2f * side, rh = 1.2f * side;
    std::vector<rgpu_primitive> pr(4);
    for (auto &p : pr) { std::memset(&p, 0, sizeof(p)); p.x = rx; p.y = ry; p.w = rw; p.h = rh; p.linear_rgb = 1; }
    float sigma = r.uf(0.5f, 20.0f);
    pr[0].kind = RGPU_FE_BLUR; pr[0].in1 = RGPU_IN_SOURCE_GRAPHIC; pr[0].f[0] = sigma; pr[0].f[1] = sigma;
    pr[1].kind = RGPU_FE_COLOR_MATRIX; pr[1].in1 = 0; pr[1].i[0] = RGPU_CM_SATURATE; pr[1].f[0] = r.uf();
    pr[2].kind = RGPU_FE_MORPHOLOGY; pr[2].in1 = 1; pr[2].i[0] = r.ui(0, 1);
    float rad = (float)r.ui(1, 5);
    pr[2].f[0] = rad; pr[2].f[1] = rad;
    pr[3].kind = RGPU_FE_COMPOSITE; pr[3].in1 = 2; pr[3].in2 = RGPU_IN_SOURCE_GRAPHIC; pr[3].i[0] = RGPU_OP_ARITHMETIC;
    for (int i = 0; i < 4; i++) pr[3].f[i] = r.uf(-1.0f, 1.0f);
    std::vector<int32_t> grp;
    add_filter_group(t, 0, r, side, pr, rx, ry, rw, rh, -1, &grp);
    for (int i = 0; i < npaths; i++) add_fill(t, grp[0], r, side, side, 0, (uint32_t)(i & 1));
}

void gen_config3(Tree &t, Rng &r) {
    float side = std::round(std::exp(r.uf(std::log(64.0f), std::log(1024.0f))));
    int npaths = (int)std::lround(std::exp(r.uf(std::log(10.0f), std::log(2000.0f))));
    bool fx = r.uf() < 0.1f;
    t.width = t.height = side;
    t.add_group(-1, plain_group());
    int first = fx ? npaths / 2 : npaths;
    for (int i = 0; i < first; i++) add_mixed(t, 0, r, side, side, 0.2f, true);
    if (fx) {
        int32_t clip = add_clip(t, r, side, side);
        std::vector<rgpu_primitive> pr(1);
        std::memset(&pr[0], 0, sizeof(pr[0]));
        float rx = -0.1f * side, ry = -0.1f * side, rw = 1.2f * side, rh = 1.2f * side;
        pr[0].x = rx; pr[0].y = ry; pr[0].w = rw; pr[0].h = rh; pr[0].linear_rgb = 1;
        pr[0].kind = RGPU_FE_BLUR; pr[0].in1 = RGPU_IN_SOURCE_GRAPHIC;
        float sigma = r.uf(1.0f, 8.0f);
        pr[0].f[0] = sigma; pr[0].f[1] = sigma;
        std::vector<int32_t> grp;
        add_filter_group(t, 0, r, side, pr, rx, ry, rw, rh, clip, &grp);
        for (int i = first; i < npaths; i++) add_mixed(t, grp[0], r, side, side, 0.2f, true);
    }
}
}  // namespace

// config: 0..3; seed and index pick the scene.  `scale` multiplies counts
// (1.0 = the full workload; tests use smaller values).
Tree *generate_scene(int config, uint64_t seed, uint64_t index, float scale) {
    Tree *t = new Tree();
    Rng r(seed * 1000003ull + index * 7919ull + (uint64_t)config);
    auto sc = [&](int n) { return std::max(1, (int)std::lround(n * scale)); };
    switch (config) {
    case 0: gen_config0(*t, r, 512.0f, sc(200)); break;
    case 1: gen_config1(*t, r, 1024.0f, sc(2000), sc(500), std::min(20, sc(20)), std::min(10, sc(10))); break;
    case 2: gen_config2(*t, r, 2048.0f, sc(500)); break;
    case 3: gen_config3(*t, r); break;
    default: delete t; return nullptr;
    }
    t->finalize();
    return t;
}

}  // namespace rgpu
