// Host driver of a filter job: resvg's filter::apply / apply_inner
// (crates/resvg/src/filter/mod.rs:335-521) over device images.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "flatten.h"

namespace rgpu {

// Device scratch the driver draws images from; buffers stay valid (and at the
// same addresses) for the lifetime of the owner, so a captured graph can
// replay the launches.
struct FilterScratch {
    virtual ~FilterScratch() {}
    virtual uint32_t *image(uint32_t idx, size_t pixels) = 0;
    virtual double *plane(size_t n) = 0;
};

// Applies the job's filters to `content` (w x h, premultiplied sRGB) and
// writes the filtered layer to `result`.  Returns 0 or an rgpu_status (a CUDA
// error).  A filter that fails for reasons of its own (an invalid region, sizes
// the reference cannot combine, a primitive the device does not run) leaves a
// cleared layer, as resvg's filter::apply does, and rendering goes on: the job
// still returns 0 and the reasons are appended to `err` as warnings.
// `images` holds, for each feImage primitive (global index), the surface its
// element was rendered into; NULL when there are none.
struct FeImageSurface { uint32_t prim; const uint32_t *p; };
int run_filter_job(const FilterJob &job, uint32_t *content, uint32_t *result, FilterScratch &scratch, cudaStream_t s,
                   std::string &err, const std::vector<FeImageSurface> *images = nullptr);

}  // namespace rgpu
