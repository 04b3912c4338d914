// Host side of stroking and dashing.  The stroker itself (tiny-skia-path
// 0.12's stroker.rs) lives in stroke_core.h, shared with the device kernel
// (kernels/stroke.cu); here it runs over std::vector storage.  The dasher
// follows tiny-skia-path's dash.rs (StrokeDash + ContourMeasure).
#include <cmath>
#include <cstring>
#include <vector>
#include "geom.h"
#include "stroke_core.h"

namespace rgpu {
namespace {

using namespace sk;
struct HostTraits {
    template <class T> using Vec = std::vector<T>;
};
using Builder = BuilderT<HostTraits>;
using Stroker = StrokerT<HostTraits>;

// ---------------------------------------------------------------- dashing (dash.rs: StrokeDash + ContourMeasure)
constexpr uint32_t kMaxTValue = 0x3FFFFFFF;

inline float pt_length(Pt d) {
    float mag2 = d.x * d.x + d.y * d.y;
    if (std::isfinite(mag2)) return std::sqrt(mag2);
    double xx = d.x, yy = d.y;
    return (float)std::sqrt(xx * xx + yy * yy);
}
inline float interp(float a, float b, float t) { return a + (b - a) * t; }

void chop_quad_at(const Pt s[3], float t, Pt d[5]) {
    Pt p01 = P(s[0].x + (s[1].x - s[0].x) * t, s[0].y + (s[1].y - s[0].y) * t);
    Pt p12 = P(s[1].x + (s[2].x - s[1].x) * t, s[1].y + (s[2].y - s[1].y) * t);
    d[0] = s[0];
    d[1] = p01;
    d[2] = P(p01.x + (p12.x - p01.x) * t, p01.y + (p12.y - p01.y) * t);
    d[3] = p12;
    d[4] = s[2];
}

enum SegKind : uint8_t { SEG_LINE, SEG_QUAD, SEG_CUBIC };
struct MSeg {
    float distance;
    uint32_t point_index;
    uint32_t t_value;
    SegKind kind;
    float scalar_t() const { return (float)t_value * (1.0f / (float)kMaxTValue); }
};

struct Contour {
    std::vector<MSeg> segs;
    std::vector<Pt> pts;
    float length = 0;
    bool closed = false;
    float tolerance = 0.5f;

    float line_seg(Pt p0, Pt p1, float distance, uint32_t pi) {
        float d = pt_length(p1 - p0);
        float prev = distance;
        distance += d;
        if (distance > prev) segs.push_back(MSeg{distance, pi, kMaxTValue, SEG_LINE});
        return distance;
    }
    static bool quad_too_curvy(const Pt p[3], float tol) {
        float dx = p[1].x * 0.5f - (p[0].x + p[2].x) * 0.5f * 0.5f;
        float dy = p[1].y * 0.5f - (p[0].y + p[2].y) * 0.5f * 0.5f;
        return std::fmax(std::fabs(dx), std::fabs(dy)) > tol;
    }
    static bool cheap_dist_exceeds(Pt pt, float x, float y, float tol) {
        return std::fmax(std::fabs(x - pt.x), std::fabs(y - pt.y)) > tol;
    }
    static bool cubic_too_curvy(const Pt p[4], float tol) {
        const float third = 1.0f / 3.0f, two_third = 2.0f / 3.0f;
        return cheap_dist_exceeds(p[1], interp(p[0].x, p[3].x, third), interp(p[0].y, p[3].y, third), tol) ||
               cheap_dist_exceeds(p[2], interp(p[0].x, p[3].x, two_third), interp(p[0].y, p[3].y, two_third), tol);
    }
    float quad_segs(const Pt p[3], float distance, uint32_t mint, uint32_t maxt, uint32_t pi) {
        if (((maxt - mint) >> 10) != 0 && quad_too_curvy(p, tolerance)) {
            Pt tmp[5];
            uint32_t half = (mint + maxt) >> 1;
            chop_quad_at(p, 0.5f, tmp);
            distance = quad_segs(tmp, distance, mint, half, pi);
            distance = quad_segs(tmp + 2, distance, half, maxt, pi);
        } else {
            float d = pt_length(p[2] - p[0]);
            float prev = distance;
            distance += d;
            if (distance > prev) segs.push_back(MSeg{distance, pi, maxt, SEG_QUAD});
        }
        return distance;
    }
    float cubic_segs(const Pt p[4], float distance, uint32_t mint, uint32_t maxt, uint32_t pi) {
        if (((maxt - mint) >> 10) != 0 && cubic_too_curvy(p, tolerance)) {
            Pt tmp[7];
            uint32_t half = (mint + maxt) >> 1;
            chop_cubic_at2(p, 0.5f, tmp);
            distance = cubic_segs(tmp, distance, mint, half, pi);
            distance = cubic_segs(tmp + 3, distance, half, maxt, pi);
        } else {
            float d = pt_length(p[3] - p[0]);
            float prev = distance;
            distance += d;
            if (distance > prev) segs.push_back(MSeg{distance, pi, maxt, SEG_CUBIC});
        }
        return distance;
    }

    // distance -> (segment index, t); false when t is not a valid unit value
    bool distance_to_segment(float distance, size_t *idx, float *t) const {
        // lower bound over segment distances (SkTSearch, exact or insertion index)
        size_t lo = 0, hi = segs.size() - 1;
        while (lo < hi) {
            size_t mid = lo + ((hi - lo) >> 1);
            if (segs[mid].distance < distance) lo = mid + 1;
            else hi = mid;
        }
        if (segs[hi].distance < distance) hi += 1;
        if (hi >= segs.size()) return false;
        const MSeg &seg = segs[hi];
        float start_t = 0.0f, start_d = 0.0f;
        if (hi > 0) {
            start_d = segs[hi - 1].distance;
            if (segs[hi - 1].point_index == seg.point_index) start_t = segs[hi - 1].scalar_t();
        }
        float v = start_t + (seg.scalar_t() - start_t) * (distance - start_d) / (seg.distance - start_d);
        if (!(v >= 0.0f && v <= 1.0f)) return false;
        *idx = hi;
        *t = v;
        return true;
    }

    static Pt pos_at(const Pt *p, SegKind k, float t) {
        switch (k) {
        case SEG_LINE: return P(interp(p[0].x, p[1].x, t), interp(p[0].y, p[1].y, t));
        case SEG_QUAD: return eval_quad_at(p, t);
        default: return eval_cubic_pos_at(p, t);
        }
    }

    static void segment_to(const Pt *p, SegKind k, float start_t, float stop_t, Builder &pb) {
        if (start_t == stop_t) {
            Pt last;
            if (pb.last_point(&last)) pb.line_to(last.x, last.y);
            return;
        }
        Pt t0[7], t1[7];
        switch (k) {
        case SEG_LINE:
            if (stop_t == 1.0f) pb.line_to(p[1].x, p[1].y);
            else pb.line_to(interp(p[0].x, p[1].x, stop_t), interp(p[0].y, p[1].y, stop_t));
            break;
        case SEG_QUAD:
            if (start_t == 0.0f) {
                if (stop_t == 1.0f) {
                    pb.quad_to(p[1].x, p[1].y, p[2].x, p[2].y);
                } else {
                    chop_quad_at(p, stop_t, t0);
                    pb.quad_to(t0[1].x, t0[1].y, t0[2].x, t0[2].y);
                }
            } else {
                chop_quad_at(p, start_t, t0);
                if (stop_t == 1.0f) {
                    pb.quad_to(t0[3].x, t0[3].y, t0[4].x, t0[4].y);
                } else {
                    chop_quad_at(t0 + 2, (stop_t - start_t) / (1.0f - start_t), t1);
                    pb.quad_to(t1[1].x, t1[1].y, t1[2].x, t1[2].y);
                }
            }
            break;
        case SEG_CUBIC:
            if (start_t == 0.0f) {
                if (stop_t == 1.0f) {
                    pb.cubic_to(p[1].x, p[1].y, p[2].x, p[2].y, p[3].x, p[3].y);
                } else {
                    chop_cubic_at2(p, stop_t, t0);
                    pb.cubic_to(t0[1].x, t0[1].y, t0[2].x, t0[2].y, t0[3].x, t0[3].y);
                }
            } else {
                chop_cubic_at2(p, start_t, t0);
                if (stop_t == 1.0f) {
                    pb.cubic_to(t0[4].x, t0[4].y, t0[5].x, t0[5].y, t0[6].x, t0[6].y);
                } else {
                    chop_cubic_at2(t0 + 3, (stop_t - start_t) / (1.0f - start_t), t1);
                    pb.cubic_to(t1[1].x, t1[1].y, t1[2].x, t1[2].y, t1[3].x, t1[3].y);
                }
            }
            break;
        }
    }

    void push_segment(float start_d, float stop_d, bool move_to, Builder &pb) const {
        if (start_d < 0.0f) start_d = 0.0f;
        if (stop_d > length) stop_d = length;
        if (!(start_d <= stop_d)) return;
        if (segs.empty()) return;
        size_t si, ei;
        float start_t, stop_t;
        if (!distance_to_segment(start_d, &si, &start_t)) return;
        if (!distance_to_segment(stop_d, &ei, &stop_t)) return;
        MSeg seg = segs[si];
        const MSeg &stop_seg = segs[ei];
        if (move_to) {
            Pt p = pos_at(&pts[seg.point_index], seg.kind, start_t);
            pb.move_to(p.x, p.y);
        }
        if (seg.point_index == stop_seg.point_index) {
            segment_to(&pts[seg.point_index], seg.kind, start_t, stop_t, pb);
        } else {
            size_t k = si;
            for (;;) {
                segment_to(&pts[seg.point_index], seg.kind, start_t, 1.0f, pb);
                uint32_t old = seg.point_index;
                do { k++; } while (segs[k].point_index == old);
                seg = segs[k];
                start_t = 0.0f;
                if (seg.point_index >= stop_seg.point_index) break;
            }
            segment_to(&pts[seg.point_index], seg.kind, 0.0f, stop_t, pb);
        }
    }
};

// ContourMeasureIter over the path's contours (no forced close); contours
// with no measurable segment are skipped.
void measure_contours(const uint8_t *verbs, size_t nv, const float *pts, float res_scale, std::vector<Contour> &out) {
    float tol = 0.5f * (1.0f / res_scale);
    size_t vi = 0, pi = 0;
    Pt last_pt;
    while (vi < nv) {
        Contour c;
        c.tolerance = tol;
        int pt_index = -1;
        float distance = 0.0f;
        bool seen_close = false, seen_move = false;
        for (; vi < nv; vi++) {
            uint8_t v = verbs[vi];
            if (seen_move && v == V_MOVE) break;
            switch (v) {
            case V_MOVE:
                pt_index += 1;
                last_pt = P(pts[2 * pi], pts[2 * pi + 1]);
                pi += 1;
                c.pts.push_back(last_pt);
                seen_move = true;
                break;
            case V_LINE: {
                Pt p1 = P(pts[2 * pi], pts[2 * pi + 1]);
                pi += 1;
                float prev = distance;
                distance = c.line_seg(last_pt, p1, distance, (uint32_t)pt_index);
                if (distance > prev) {
                    c.pts.push_back(p1);
                    pt_index++;
                }
                last_pt = p1;
                break;
            }
            case V_QUAD: {
                Pt q[3] = {last_pt, P(pts[2 * pi], pts[2 * pi + 1]), P(pts[2 * pi + 2], pts[2 * pi + 3])};
                pi += 2;
                float prev = distance;
                distance = c.quad_segs(q, distance, 0, kMaxTValue, (uint32_t)pt_index);
                if (distance > prev) {
                    c.pts.push_back(q[1]);
                    c.pts.push_back(q[2]);
                    pt_index += 2;
                }
                last_pt = q[2];
                break;
            }
            case V_CUBIC: {
                Pt q[4] = {last_pt, P(pts[2 * pi], pts[2 * pi + 1]), P(pts[2 * pi + 2], pts[2 * pi + 3]),
                           P(pts[2 * pi + 4], pts[2 * pi + 5])};
                pi += 3;
                float prev = distance;
                distance = c.cubic_segs(q, distance, 0, kMaxTValue, (uint32_t)pt_index);
                if (distance > prev) {
                    c.pts.push_back(q[1]);
                    c.pts.push_back(q[2]);
                    c.pts.push_back(q[3]);
                    pt_index += 3;
                }
                last_pt = q[3];
                break;
            }
            case V_CLOSE:
                seen_close = true;
                if (!c.pts.empty()) last_pt = c.pts[0];
                break;
            default: break;
            }
        }
        if (!std::isfinite(distance)) return;
        if (c.segs.empty()) continue;
        if (seen_close) {
            float prev = distance;
            Pt first = c.pts[0];
            distance = c.line_seg(c.pts[(size_t)pt_index], first, distance, (uint32_t)pt_index);
            if (distance > prev) c.pts.push_back(first);
        }
        c.length = distance;
        c.closed = seen_close;
        out.push_back(std::move(c));
    }
}

void emit(const Builder &o, PathData &out) {
    size_t pi = 0;
    for (uint8_t v : o.verbs) {
        switch (v) {
        case V_MOVE: out.move_to(o.pts[pi].x, o.pts[pi].y); pi += 1; break;
        case V_LINE: out.line_to(o.pts[pi].x, o.pts[pi].y); pi += 1; break;
        case V_QUAD: out.quad_to(o.pts[pi].x, o.pts[pi].y, o.pts[pi + 1].x, o.pts[pi + 1].y); pi += 2; break;
        case V_CUBIC:
            out.cubic_to(o.pts[pi].x, o.pts[pi].y, o.pts[pi + 1].x, o.pts[pi + 1].y, o.pts[pi + 2].x, o.pts[pi + 2].y);
            pi += 3;
            break;
        case V_CLOSE: out.close(); break;
        }
    }
}

}  // namespace

bool stroke_path(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, const StrokeStyle &st,
                 float res_scale, PathData &out) {
    (void)npts;
    if (!(st.width > 0.0f) || !std::isfinite(st.width)) return false;
    std::vector<Seg> segs(2 * nv + 1);
    const long n = build_segments(verbs, nv, pts, segs.data());
    if (n < 0) return false;
    Stroker sk;
    StrokeParams sp;
    sp.width = st.width;
    sp.miter_limit = st.miter_limit;
    sp.cap = st.cap;
    sp.join = st.join;
    sp.res_scale = res_scale;
    if (!stroke_segments(sk, segs.data(), (size_t)n, sp)) return false;
    emit(sk.outer, out);
    return true;
}

// StrokeDash::new + Path::dash (dash.rs).  Returns false when the dash array
// is invalid (the caller strokes the undashed path); true otherwise, with
// `out` left empty when dashing produced no path (nothing is drawn).
bool dash_path(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, const float *dashes, size_t nd,
               float offset, float res_scale, PathData &out) {
    (void)npts;
    if (nd < 2 || nd % 2 != 0) return false;
    float interval = 0.0f;
    for (size_t i = 0; i < nd; i++) {
        if (dashes[i] < 0.0f) return false;
        interval += dashes[i];
    }
    if (!std::isnormal(interval) || interval <= 0.0f) return false;
    if (!std::isfinite(offset)) return false;
    // adjust_dash_offset
    if (offset < 0.0f) {
        offset = -offset;
        if (offset > interval) offset = std::fmod(offset, interval);
        offset = interval - offset;
        if (offset == interval) offset = 0.0f;
    } else if (offset >= interval) {
        offset = std::fmod(offset, interval);
    }
    // find_first_interval
    float first_len = dashes[0];
    size_t first_index = 0;
    {
        float o = offset;
        bool found = false;
        for (size_t i = 0; i < nd; i++) {
            float gap = dashes[i];
            if (o > gap || (o == gap && gap != 0.0f)) {
                o -= gap;
            } else {
                first_len = gap - o;
                first_index = i;
                found = true;
                break;
            }
        }
        if (!found) { first_len = dashes[0]; first_index = 0; }
    }
    std::vector<Contour> contours;
    measure_contours(verbs, nv, pts, res_scale, contours);
    Builder pb;
    float dash_count = 0.0f;
    for (const Contour &c : contours) {
        bool skip_first = c.closed;
        bool added = false;
        float length = c.length;
        size_t index = first_index;
        dash_count += length * (float)(nd >> 1) / interval;
        if (dash_count > 1000000.0f) return true;  // gives up: nothing drawn
        float distance = 0.0f;
        float d_len = first_len;
        while (distance < length) {
            added = false;
            if (index % 2 == 0 && !skip_first) {
                added = true;
                c.push_segment(distance, distance + d_len, true, pb);
            }
            distance += d_len;
            skip_first = false;
            index += 1;
            if (index == nd) index = 0;
            d_len = dashes[index];
        }
        if (c.closed && first_index % 2 == 0 && first_len >= 0.0f) c.push_segment(0.0f, first_len, !added, pb);
    }
    if (pb.verbs.size() <= 1) return true;
    emit(pb, out);
    return true;
}

}  // namespace rgpu
