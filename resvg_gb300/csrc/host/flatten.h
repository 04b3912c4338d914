// Host flattener: walks a render tree the way resvg's renderer does
// (crates/resvg/src/render.rs:10-142, path.rs:6-177, clip.rs:6-98,
// mask.rs:6-46) and emits device records (draws, paints, gradients, layers)
// and the band VM's command stream instead of rasterising.
#pragma once
#include <string>
#include <vector>
#include "../device_types.h"
#include "tree.h"
#include "xform.h"

namespace rgpu {

struct FilterJob;  // filter groups rendered in a separate pass (filter_exec.cpp)

struct SceneBuild {
    std::vector<DrawRec> draws;
    std::vector<PaintRec> paints;
    std::vector<GradRec> grads;
    std::vector<LayerRec> layers;
    std::vector<Cmd> cmds;
    std::vector<StreamRec> streams;
    std::vector<uint8_t> verbs;
    std::vector<float> pts;
    uint64_t nsegs = 0, ntpts = 0;
    std::string error;

    // Appends one tree as one output stream; returns the stream index or -1.
    // `out_ptr`/`stride` describe the device surface; (w, h) its size.
    int add_tree(Tree &tree, const Xf &ts, int32_t w, int32_t h, uint64_t out_ptr, uint32_t stride);
};

}  // namespace rgpu
