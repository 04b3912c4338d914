/*
 * rgpu_tree.h — flat, read-only view of a resolved SVG render tree.
 *
 * This is the input both renderers consume: the GPU backend (resvg_gb300) and
 * the CPU oracle.  It carries exactly what resvg's renderer reads from a
 * `usvg::Tree` after parsing (crates/usvg/src/tree/mod.rs): groups with
 * transform/opacity/blend/isolation/clip/mask/filters and a precomputed layer
 * bounding box (tree/mod.rs:1866-1929), paths with absolute M/L/Q/C/Z data,
 * fill/stroke (tree/mod.rs:582-698), resolved paint servers with normalised
 * stops (parser/paint_server.rs:277-405), clip paths (tree/mod.rs:793), masks
 * (tree/mod.rs:857) and filters (tree/filter.rs:82-100).
 *
 * All arrays are owned by whoever built the tree (see resvg_gpu.h for the
 * builder).  Indices are 0-based; -1 means "none".  The root is group 0.
 */
#ifndef RGPU_TREE_H
#define RGPU_TREE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Affine transform in resvg's row form {a,b,c,d,e,f} = {sx,ky,kx,sy,tx,ty}:
 *   x' = sx*x + kx*y + tx ;  y' = ky*x + sy*y + ty
 * Same layout as `resvg_transform` (crates/c-api/resvg.h). */
typedef struct rgpu_transform {
    float sx, ky, kx, sy, tx, ty;
} rgpu_transform;

enum rgpu_verb { RGPU_MOVE = 0, RGPU_LINE = 1, RGPU_QUAD = 2, RGPU_CUBIC = 3, RGPU_CLOSE = 4 };

enum rgpu_fill_rule { RGPU_NONZERO = 0, RGPU_EVENODD = 1 };

/* tiny-skia BlendMode order (the 16 SVG modes map through
 * crates/resvg/src/render.rs:145-164). */
enum rgpu_blend {
    RGPU_BLEND_CLEAR = 0, RGPU_BLEND_SOURCE, RGPU_BLEND_DESTINATION, RGPU_BLEND_SOURCE_OVER,
    RGPU_BLEND_DESTINATION_OVER, RGPU_BLEND_SOURCE_IN, RGPU_BLEND_DESTINATION_IN,
    RGPU_BLEND_SOURCE_OUT, RGPU_BLEND_DESTINATION_OUT, RGPU_BLEND_SOURCE_ATOP,
    RGPU_BLEND_DESTINATION_ATOP, RGPU_BLEND_XOR, RGPU_BLEND_PLUS, RGPU_BLEND_MODULATE,
    RGPU_BLEND_SCREEN, RGPU_BLEND_OVERLAY, RGPU_BLEND_DARKEN, RGPU_BLEND_LIGHTEN,
    RGPU_BLEND_COLOR_DODGE, RGPU_BLEND_COLOR_BURN, RGPU_BLEND_HARD_LIGHT,
    RGPU_BLEND_SOFT_LIGHT, RGPU_BLEND_DIFFERENCE, RGPU_BLEND_EXCLUSION,
    RGPU_BLEND_MULTIPLY, RGPU_BLEND_HUE, RGPU_BLEND_SATURATION, RGPU_BLEND_COLOR,
    RGPU_BLEND_LUMINOSITY
};

enum rgpu_paint_kind { RGPU_PAINT_SOLID = 0, RGPU_PAINT_LINEAR = 1, RGPU_PAINT_RADIAL = 2, RGPU_PAINT_PATTERN = 3,
                       RGPU_PAINT_IMAGE = 4 };
/* A raster image (resvg image.rs render_raster): stop_offset = an image of the
 * tree (rgpu_tree_add_image), spread = rgpu_image_quality; the pattern is
 * padded (not repeated) and sampled in the path's user space, where the image
 * spans (0, 0, width, height).  The path is that rect. */
enum rgpu_image_quality { RGPU_IMAGE_NEAREST = 0, RGPU_IMAGE_BILINEAR = 1, RGPU_IMAGE_BICUBIC = 2 };
typedef struct rgpu_image {
    uint32_t width, height;
    uint64_t pixel_offset;    /* into image_pixels: premultiplied RGBA8, row-major */
} rgpu_image;
/* A pattern (usvg::Pattern, resolved to user space): x1, y1, x2, y2 = the tile
 * rect x, y, width, height; transform = patternTransform; stop_offset = a
 * detached group whose children are the tile content (viewBox and content
 * units already applied); stop_count = 0. */
enum rgpu_spread { RGPU_SPREAD_PAD = 0, RGPU_SPREAD_REFLECT = 1, RGPU_SPREAD_REPEAT = 2 };
enum rgpu_cap { RGPU_CAP_BUTT = 0, RGPU_CAP_ROUND = 1, RGPU_CAP_SQUARE = 2 };
enum rgpu_join { RGPU_JOIN_MITER = 0, RGPU_JOIN_MITER_CLIP = 1, RGPU_JOIN_ROUND = 2, RGPU_JOIN_BEVEL = 3 };

/* One gradient stop after usvg's normalisation (offsets clamped and
 * monotonic).  Colour is sRGB 8-bit, opacity in [0,1]. */
typedef struct rgpu_stop {
    float offset;
    uint8_t r, g, b, _pad;
    float opacity;
} rgpu_stop;

/* A paint server in user space (objectBoundingBox already resolved). */
typedef struct rgpu_paint {
    uint32_t kind;            /* rgpu_paint_kind */
    uint8_t r, g, b, _pad;    /* solid colour */
    float x1, y1, x2, y2;     /* linear gradient vector */
    float cx, cy, r_, fx, fy, fr; /* radial: centre, radius, focal point, focal radius */
    uint32_t spread;          /* rgpu_spread */
    rgpu_transform transform; /* gradientTransform */
    uint32_t stop_offset, stop_count;
} rgpu_paint;

typedef struct rgpu_path {
    uint32_t verb_offset, verb_count;
    uint32_t point_offset, point_count; /* points are (x,y) float pairs */
    int32_t fill_paint;       /* -1: no fill */
    float fill_opacity;
    uint32_t fill_rule;
    int32_t stroke_paint;     /* -1: no stroke */
    float stroke_opacity;
    float stroke_width;
    float miter_limit;
    uint32_t line_cap, line_join;
    uint32_t dash_offset, dash_count; /* into dashes[] */
    float dash_phase;
    uint32_t stroke_first;    /* paint-order: 1 = stroke before fill */
    uint32_t anti_alias;      /* shape-rendering: 0 = crispEdges/optimizeSpeed */
    uint32_t visible;
    /* usvg's stroke bounding box (tight bounds of the stroked outline, or of
     * the fill when there is no stroke), in the path's user space. */
    float bbox_x, bbox_y, bbox_w, bbox_h;
} rgpu_path;

enum rgpu_node_kind { RGPU_NODE_GROUP = 0, RGPU_NODE_PATH = 1 };

typedef struct rgpu_node {
    uint32_t kind;   /* rgpu_node_kind */
    uint32_t index;  /* into groups[] or paths[] */
} rgpu_node;

typedef struct rgpu_group {
    rgpu_transform transform;
    float opacity;
    uint32_t blend;           /* rgpu_blend (SourceOver = normal) */
    uint32_t isolate;
    int32_t clip_path;        /* into clips[] */
    int32_t mask;             /* into masks[] */
    uint32_t filter_offset, filter_count; /* into filter_refs[] */
    uint32_t child_offset, child_count;   /* into children[] */
    uint32_t has_layer_bbox;
    /* layer bounding box in the group's own coordinates (before its transform) */
    float layer_x, layer_y, layer_w, layer_h;
} rgpu_group;

typedef struct rgpu_clip {
    rgpu_transform transform;
    int32_t clip_path;        /* nested clip on the clip path itself */
    uint32_t root;            /* group holding the clip children */
} rgpu_clip;

enum rgpu_mask_kind { RGPU_MASK_LUMINANCE = 0, RGPU_MASK_ALPHA = 1 };

typedef struct rgpu_mask {
    float x, y, w, h;         /* mask region in user space */
    uint32_t kind;
    int32_t mask;             /* nested mask */
    uint32_t root;            /* group holding the mask content */
} rgpu_mask;

enum rgpu_prim_kind {
    RGPU_FE_BLUR = 0, RGPU_FE_COLOR_MATRIX, RGPU_FE_MORPHOLOGY, RGPU_FE_COMPOSITE,
    RGPU_FE_CONVOLVE, RGPU_FE_DIFFUSE, RGPU_FE_SPECULAR, RGPU_FE_FLOOD, RGPU_FE_OFFSET,
    RGPU_FE_MERGE, RGPU_FE_BLEND, RGPU_FE_COMPONENT_TRANSFER, RGPU_FE_DROP_SHADOW,
    RGPU_FE_TURBULENCE, RGPU_FE_TILE, RGPU_FE_DISPLACEMENT_MAP, RGPU_FE_IMAGE
};

/* inputs */
#define RGPU_IN_SOURCE_GRAPHIC (-1)
#define RGPU_IN_SOURCE_ALPHA (-2)

enum rgpu_cm_kind { RGPU_CM_MATRIX = 0, RGPU_CM_SATURATE, RGPU_CM_HUE_ROTATE, RGPU_CM_LUM_TO_ALPHA };
enum rgpu_composite_op { RGPU_OP_OVER = 0, RGPU_OP_IN, RGPU_OP_OUT, RGPU_OP_ATOP, RGPU_OP_XOR, RGPU_OP_ARITHMETIC };
enum rgpu_edge_mode { RGPU_EDGE_NONE = 0, RGPU_EDGE_DUPLICATE, RGPU_EDGE_WRAP };
enum rgpu_light_kind { RGPU_LIGHT_DISTANT = 0, RGPU_LIGHT_POINT, RGPU_LIGHT_SPOT };
enum rgpu_transfer_kind { RGPU_TF_IDENTITY = 0, RGPU_TF_TABLE, RGPU_TF_DISCRETE, RGPU_TF_LINEAR, RGPU_TF_GAMMA };
#define RGPU_TF_MAX_VALUES 16

/* One filter primitive.  Which fields are meaningful depends on `kind`:
 *   BLUR:         f[0]=stdDeviationX f[1]=stdDeviationY
 *   COLOR_MATRIX: i[0]=rgpu_cm_kind; f[0..19]=matrix, or f[0]=saturate value / hue angle
 *   MORPHOLOGY:   i[0]=0 erode 1 dilate; f[0]=rx f[1]=ry
 *   COMPOSITE:    i[0]=rgpu_composite_op; f[0..3]=k1..k4
 *   CONVOLVE:     i[0]=columns i[1]=rows i[2]=target_x i[3]=target_y i[4]=edge mode
 *                 i[5]=preserve_alpha; f[0]=divisor f[1]=bias; kernel at f[2..]
 *   DIFFUSE:      f[0]=surface_scale f[1]=diffuse_constant; light below
 *   SPECULAR:     f[0]=surface_scale f[1]=specular_constant f[2]=specular_exponent
 *   lighting:     i[0]=rgpu_light_kind; i[1..3]=lighting colour rgb;
 *                 distant: f[4]=azimuth f[5]=elevation;
 *                 point:   f[4..6]=x,y,z;
 *                 spot:    f[4..6]=x,y,z f[7..9]=pointsAt f[10]=specularExponent
 *                          f[11]=limitingConeAngle (NaN: none)
 *   FLOOD:        i[0..2]=rgb f[0]=opacity
 *   OFFSET:       f[0]=dx f[1]=dy
 *   MERGE:        inputs in merge_inputs[i[0] .. i[0]+i[1])
 *   BLEND:        i[0]=rgpu_blend
 *   COMPONENT_TRANSFER: channel c = 0..3 (R, G, B, A): i[c]=rgpu_transfer_kind,
 *                 i[4+c]=number of table values (table, discrete; at most
 *                 RGPU_TF_MAX_VALUES); parameters at f[16*c ..]: the table values,
 *                 or slope, intercept (linear), or amplitude, exponent, offset (gamma)
 *   DROP_SHADOW:  i[0..2]=flood rgb; f[0]=stdDeviationX f[1]=stdDeviationY
 *                 f[2]=dx f[3]=dy f[4]=opacity (flood-opacity times the colour's alpha)
 *   TURBULENCE:   f[0]=baseFrequencyX f[1]=baseFrequencyY (both >= 0); i[0]=numOctaves
 *                 (at most RGPU_TURB_MAX_OCTAVES on the device) i[1]=seed
 *                 i[2]=stitchTiles i[3]=1 fractalNoise, 0 turbulence
 *   TILE:         in1 only
 *   DISPLACEMENT_MAP: i[0]=xChannelSelector i[1]=yChannelSelector (0..3 = R, G, B, A);
 *                 f[0]=scale; in1 = the image displaced, in2 = the map
 *   IMAGE:        i[0]=a detached group whose children are rendered (feImage of an
 *                 element), or -1 for nothing (transparent)
 */
#define RGPU_TURB_MAX_OCTAVES 1024
#define RGPU_PRIM_F 64
typedef struct rgpu_primitive {
    uint32_t kind;
    float x, y, w, h;         /* primitive subregion, user space */
    uint32_t linear_rgb;      /* color-interpolation-filters: 1 = linearRGB */
    int32_t in1, in2;         /* RGPU_IN_* or index of an earlier primitive */
    int32_t i[8];
    float f[RGPU_PRIM_F];
} rgpu_primitive;

typedef struct rgpu_filter {
    float x, y, w, h;         /* filter region, user space */
    uint32_t prim_offset, prim_count;
} rgpu_filter;

/* The whole tree. */
typedef struct rgpu_tree_view {
    float width, height;      /* canvas size in user units */
    const rgpu_group *groups; uint32_t group_count;
    const rgpu_node *children; uint32_t child_count;
    const rgpu_path *paths; uint32_t path_count;
    const uint8_t *verbs; uint32_t verb_count;
    const float *points; uint32_t point_count; /* number of (x,y) pairs */
    const rgpu_paint *paints; uint32_t paint_count;
    const rgpu_stop *stops; uint32_t stop_count;
    const float *dashes; uint32_t dash_count;
    const rgpu_clip *clips; uint32_t clip_count;
    const rgpu_mask *masks; uint32_t mask_count;
    const uint32_t *filter_refs; uint32_t filter_ref_count;
    const rgpu_filter *filters; uint32_t filter_count;
    const rgpu_primitive *prims; uint32_t prim_count;
    const int32_t *merge_inputs; uint32_t merge_input_count;
    const rgpu_image *images; uint32_t image_count;
    const uint8_t *image_pixels; uint64_t image_pixel_bytes;
} rgpu_tree_view;

#ifdef __cplusplus
}
#endif
#endif
