// Host side of stroking and dashing.  The stroker (tiny-skia-path 0.12's
// stroker.rs, stroke_core.h) and the dasher (dash.rs, dash_core.h) are shared
// with the device kernel (kernels/stroke.cu); here they run over std::vector
// storage.
#include <cmath>
#include <cstring>
#include <vector>
#include "geom.h"
#include "dash_core.h"

namespace rgpu {
namespace {

using namespace sk;
struct HostTraits {
    template <class T> using Vec = std::vector<T>;
};
using Builder = BuilderT<HostTraits>;
using Stroker = StrokerT<HostTraits>;

using Contour = ContourT<HostTraits>;

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

// StrokeDash::new + Path::dash (dash.rs, dash_core.h).  Returns false when
// the dash array is invalid (the caller strokes the undashed path); true
// otherwise, with `out` left empty when dashing produced no path (nothing is
// drawn).
bool dash_path(const uint8_t *verbs, size_t nv, const float *pts, size_t npts, const float *dashes, size_t nd,
               float offset, float res_scale, PathData &out) {
    (void)npts;
    Contour c;
    Builder pb;
    const int r = dash_run(verbs, nv, pts, dashes, nd, offset, res_scale, c, pb);
    if (r < 0) return false;
    if (r > 0) emit(pb, out);
    return true;
}

}  // namespace rgpu
