// Dashing shared by the host and the device: tiny-skia-path 0.12's dash.rs
// (StrokeDash + ContourMeasure, a port of Skia's SkDashPath and
// SkContourMeasure).  Each contour is measured into line / quad / cubic
// pieces flat to `0.5 / res_scale`, then the dash intervals are cut from it
// by distance.  Like the stroker (stroke_core.h) it is one source compiled
// by both sides over a storage policy; the curve halving that dash.rs writes
// as recursion runs here over an explicit stack in the same order.
//
// Contours are measured and dashed one at a time (dash.rs measures them all
// first): the output is the same, since a contour's dashes depend only on that
// contour and the running dash count, and the scratch is one contour.
#pragma once
#include "stroke_core.h"

namespace rgpu {
namespace sk {

constexpr uint32_t kMaxTValue = 0x3FFFFFFF;

SK_HD inline float pt_length(Pt d) {
    float mag2 = d.x * d.x + d.y * d.y;
    if (sk_isfinite(mag2)) return sk_sqrt(mag2);
    double xx = d.x, yy = d.y;
    return (float)sk_sqrt(xx * xx + yy * yy);
}
SK_HD inline float interp(float a, float b, float t) { return a + (b - a) * t; }
SK_HD inline bool sk_isnormal(float v) { return sk_isfinite(v) && sk_fabs(v) >= 1.17549435e-38f; }
SK_HD inline float sk_fmod(float a, float b) {
#ifdef __CUDA_ARCH__
    return fmodf(a, b);
#else
    return std::fmod(a, b);
#endif
}

SK_HD inline void chop_quad_at(const Pt s[3], float t, Pt d[5]) {
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
    uint8_t kind;  // SegKind
    SK_HD float scalar_t() const { return (float)t_value * (1.0f / (float)kMaxTValue); }
};

template <class Tr> struct ContourT {
    typename Tr::template Vec<MSeg> segs;
    typename Tr::template Vec<Pt> pts;
    float length = 0;
    bool closed = false;
    float tolerance = 0.5f;

    SK_HD void reset() {
        segs.clear();
        pts.clear();
        length = 0;
        closed = false;
    }
    SK_HD float line_seg(Pt p0, Pt p1, float distance, uint32_t pi) {
        float d = pt_length(p1 - p0);
        float prev = distance;
        distance += d;
        if (distance > prev) segs.push_back(MSeg{distance, pi, kMaxTValue, SEG_LINE});
        return distance;
    }
    SK_HD static bool quad_too_curvy(const Pt p[3], float tol) {
        float dx = p[1].x * 0.5f - (p[0].x + p[2].x) * 0.5f * 0.5f;
        float dy = p[1].y * 0.5f - (p[0].y + p[2].y) * 0.5f * 0.5f;
        return sk_fmax(sk_fabs(dx), sk_fabs(dy)) > tol;
    }
    SK_HD static bool cheap_dist_exceeds(Pt pt, float x, float y, float tol) {
        return sk_fmax(sk_fabs(x - pt.x), sk_fabs(y - pt.y)) > tol;
    }
    SK_HD static bool cubic_too_curvy(const Pt p[4], float tol) {
        const float third = 1.0f / 3.0f, two_third = 2.0f / 3.0f;
        return cheap_dist_exceeds(p[1], interp(p[0].x, p[3].x, third), interp(p[0].y, p[3].y, third), tol) ||
               cheap_dist_exceeds(p[2], interp(p[0].x, p[3].x, two_third), interp(p[0].y, p[3].y, two_third), tol);
    }
    // Halving while the piece is too curvy and its t range spans at least 1024
    // steps (at most 20 levels): left half first, as the recursion does.
    SK_HD float quad_segs(const Pt p0[3], float distance, uint32_t mint0, uint32_t maxt0, uint32_t pi) {
        struct F { Pt p[3]; uint32_t mint, maxt; };
        F st[24];
        int sp = 0;
        st[sp++] = F{{p0[0], p0[1], p0[2]}, mint0, maxt0};
        while (sp > 0) {
            const F f = st[--sp];
            if (((f.maxt - f.mint) >> 10) != 0 && quad_too_curvy(f.p, tolerance) && sp + 2 <= 24) {
                Pt tmp[5];
                uint32_t half = (f.mint + f.maxt) >> 1;
                chop_quad_at(f.p, 0.5f, tmp);
                st[sp++] = F{{tmp[2], tmp[3], tmp[4]}, half, f.maxt};
                st[sp++] = F{{tmp[0], tmp[1], tmp[2]}, f.mint, half};
            } else {
                float d = pt_length(f.p[2] - f.p[0]);
                float prev = distance;
                distance += d;
                if (distance > prev) segs.push_back(MSeg{distance, pi, f.maxt, SEG_QUAD});
            }
        }
        return distance;
    }
    SK_HD float cubic_segs(const Pt p0[4], float distance, uint32_t mint0, uint32_t maxt0, uint32_t pi) {
        struct F { Pt p[4]; uint32_t mint, maxt; };
        F st[24];
        int sp = 0;
        st[sp++] = F{{p0[0], p0[1], p0[2], p0[3]}, mint0, maxt0};
        while (sp > 0) {
            const F f = st[--sp];
            if (((f.maxt - f.mint) >> 10) != 0 && cubic_too_curvy(f.p, tolerance) && sp + 2 <= 24) {
                Pt tmp[7];
                uint32_t half = (f.mint + f.maxt) >> 1;
                chop_cubic_at2(f.p, 0.5f, tmp);
                st[sp++] = F{{tmp[3], tmp[4], tmp[5], tmp[6]}, half, f.maxt};
                st[sp++] = F{{tmp[0], tmp[1], tmp[2], tmp[3]}, f.mint, half};
            } else {
                float d = pt_length(f.p[3] - f.p[0]);
                float prev = distance;
                distance += d;
                if (distance > prev) segs.push_back(MSeg{distance, pi, f.maxt, SEG_CUBIC});
            }
        }
        return distance;
    }

    // distance -> (segment index, t); false when t is not a valid unit value
    SK_HD bool distance_to_segment(float distance, size_t *idx, float *t) const {
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

    SK_HD static Pt pos_at(const Pt *p, uint8_t k, float t) {
        switch (k) {
        case SEG_LINE: return P(interp(p[0].x, p[1].x, t), interp(p[0].y, p[1].y, t));
        case SEG_QUAD: return eval_quad_at(p, t);
        default: return eval_cubic_pos_at(p, t);
        }
    }

    // the points of the piece of kind k starting at point i (copied: the
    // device storage clamps its reads)
    SK_HD void points_at(size_t i, uint8_t k, Pt *out) const {
        const int n = k == SEG_LINE ? 2 : (k == SEG_QUAD ? 3 : 4);
        for (int j = 0; j < n; j++) out[j] = pts[i + j];
    }

    template <class B> SK_HD static void segment_to(const Pt *p, uint8_t k, float start_t, float stop_t, B &pb) {
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

    template <class B> SK_HD void push_segment(float start_d, float stop_d, bool move_to, B &pb) const {
        if (start_d < 0.0f) start_d = 0.0f;
        if (stop_d > length) stop_d = length;
        if (!(start_d <= stop_d)) return;
        if (segs.empty()) return;
        size_t si, ei;
        float start_t, stop_t;
        if (!distance_to_segment(start_d, &si, &start_t)) return;
        if (!distance_to_segment(stop_d, &ei, &stop_t)) return;
        MSeg seg = segs[si];
        const MSeg stop_seg = segs[ei];
        Pt q[4];
        if (move_to) {
            points_at(seg.point_index, seg.kind, q);
            Pt p = pos_at(q, seg.kind, start_t);
            pb.move_to(p.x, p.y);
        }
        if (seg.point_index == stop_seg.point_index) {
            points_at(seg.point_index, seg.kind, q);
            segment_to(q, seg.kind, start_t, stop_t, pb);
        } else {
            size_t k = si;
            for (;;) {
                points_at(seg.point_index, seg.kind, q);
                segment_to(q, seg.kind, start_t, 1.0f, pb);
                uint32_t old = seg.point_index;
                // the next piece of another source segment (ei lies past si, so this ends)
                do { k++; } while (k < ei && segs[k].point_index == old);
                seg = segs[k];
                start_t = 0.0f;
                if (seg.point_index >= stop_seg.point_index) break;
            }
            points_at(seg.point_index, seg.kind, q);
            segment_to(q, seg.kind, 0.0f, stop_t, pb);
        }
    }
};

// ContourMeasureIter: measures the next contour of (verbs, pts) from verb
// *vi / point *pi into c (no forced close); false when the path is done.  A
// contour with no measurable piece comes back empty (c.segs.empty()).  A
// non-finite length ends the path (*stop), as the iterator does.
template <class Tr>
SK_HD inline bool measure_next_contour(const uint8_t *verbs, size_t nv, const float *pts, float tol, size_t *vi_io,
                                       size_t *pi_io, Pt *last_io, ContourT<Tr> &c, bool *stop) {
    size_t vi = *vi_io, pi = *pi_io;
    Pt last_pt = *last_io;
    if (vi >= nv) return false;
    c.reset();
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
    *vi_io = vi;
    *pi_io = pi;
    *last_io = last_pt;
    if (!sk_isfinite(distance)) {
        *stop = true;
        c.segs.clear();
        return true;
    }
    if (c.segs.empty()) return true;
    if (seen_close) {
        float prev = distance;
        Pt first = c.pts[0];
        distance = c.line_seg(c.pts[(size_t)pt_index], first, distance, (uint32_t)pt_index);
        if (distance > prev) c.pts.push_back(first);
    }
    c.length = distance;
    c.closed = seen_close;
    return true;
}

// StrokeDash::new + Path::dash into pb.  Returns -1 when the dash array is
// invalid (the caller strokes the undashed path), 0 when dashing gives up
// (more than a million dashes: nothing is drawn) or leaves nothing, 1 with
// the dashed path in pb.
template <class Tr>
SK_HD inline int dash_run(const uint8_t *verbs, size_t nv, const float *pts, const float *dashes, size_t nd,
                          float offset, float res_scale, ContourT<Tr> &c, BuilderT<Tr> &pb) {
    if (nd < 2 || nd % 2 != 0) return -1;
    float interval = 0.0f;
    for (size_t i = 0; i < nd; i++) {
        if (dashes[i] < 0.0f) return -1;
        interval += dashes[i];
    }
    if (!sk_isnormal(interval) || interval <= 0.0f) return -1;
    if (!sk_isfinite(offset)) return -1;
    // adjust_dash_offset
    if (offset < 0.0f) {
        offset = -offset;
        if (offset > interval) offset = sk_fmod(offset, interval);
        offset = interval - offset;
        if (offset == interval) offset = 0.0f;
    } else if (offset >= interval) {
        offset = sk_fmod(offset, interval);
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
        if (!found) {
            first_len = dashes[0];
            first_index = 0;
        }
    }
    const float tol = 0.5f * (1.0f / res_scale);
    size_t vi = 0, pi = 0;
    Pt last_pt;
    bool stop = false;
    float dash_count = 0.0f;
    while (!stop && measure_next_contour(verbs, nv, pts, tol, &vi, &pi, &last_pt, c, &stop)) {
        if (stop || c.segs.empty()) continue;
        bool skip_first = c.closed;
        bool added = false;
        float length = c.length;
        size_t index = first_index;
        dash_count += length * (float)(nd >> 1) / interval;
        if (dash_count > 1000000.0f) {
            pb.clear();
            return 0;  // gives up: nothing drawn
        }
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
    return pb.verbs.size() <= 1 ? 0 : 1;
}

}  // namespace sk
}  // namespace rgpu
