// CPU oracle — TEST INFRASTRUCTURE ONLY: scene generation and scene-parallel
// rendering for the parity tests, the CPU baseline and the reference arm of
// the benchmark.
//
// oracle_tree_generate builds the seeded synthetic workloads from the same
// generator source the product ships (resvg_gb300/csrc/host/gen.cpp, compiled
// into this library), so the reference arm of the benchmark renders the same
// trees without loading the product library.
//
// oracle_render_many renders whole trees, one tree per worker thread at a time,
// each exactly as oracle_render does (resvg renders one tree per call,
// crates/resvg/src/lib.rs:34-43; a multi-scene CPU workload is parallelised
// over scenes).  Unlike oracle_render_parallel, which splits one canvas into
// translated strips for timing, every output here is bit-identical to a
// single-threaded oracle_render of the same tree.
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include "rgpu_tree.h"
#include "../resvg_gb300/csrc/host/tree.h"

namespace rgpu {
Tree *generate_scene(int config, uint64_t seed, uint64_t index, float scale);
}

extern "C" int oracle_render(const rgpu_tree_view *tree, const float ts6[6], uint32_t w, uint32_t h,
                             uint8_t *pixmap);

extern "C" {

void *oracle_tree_generate(int config, uint64_t seed, uint64_t index, float scale) {
    return rgpu::generate_scene(config, seed, index, scale);
}

const rgpu_tree_view *oracle_tree_view(void *tree) {
    if (!tree) return nullptr;
    rgpu::Tree *t = (rgpu::Tree *)tree;
    if (!t->finalized) t->finalize();
    return t->get_view();
}

void oracle_tree_free(void *tree) { delete (rgpu::Tree *)tree; }

// Renders trees[i] onto pixmaps[i] (widths[i] x heights[i] premultiplied
// RGBA8, drawn onto their content) under ts6[6*i .. 6*i+5], in the given
// order, on `threads` host threads that each take the next unrendered tree.
// Returns 0, or -1 when an argument or a render is invalid.
int oracle_render_many(const rgpu_tree_view *const *trees, const float *ts6, const uint32_t *widths,
                       const uint32_t *heights, uint8_t *const *pixmaps, uint32_t count, uint32_t threads) {
    if (!trees || !ts6 || !widths || !heights || !pixmaps) return -1;
    if (threads == 0) threads = 1;
    if (threads > count) threads = count ? count : 1;
    std::atomic<uint32_t> next{0};
    std::atomic<int> failed{0};
    auto work = [&]() {
        for (;;) {
            const uint32_t i = next.fetch_add(1);
            if (i >= count) return;
            if (oracle_render(trees[i], ts6 + 6 * (size_t)i, widths[i], heights[i], pixmaps[i]) != 0) failed = 1;
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t k = 1; k < threads; k++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    return failed ? -1 : 0;
}

}  // extern "C"
