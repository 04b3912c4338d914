// Allocation-free box blur: the filter module's box blur (the same kernels as
// rgpu_filter_box_blur) with its intermediate image in a fixed, file-scope
// device array instead of a cudaMalloc'd buffer.
//
// Who needs it: embedders that own the device memory budget and may not
// allocate behind their own allocator, for example a host that hands all
// device memory to a caching allocator (PyTorch's, an arena in a game engine)
// or runs with a hard per-process memory cap, and callers on a latency path
// where cudaMalloc/cudaFree would synchronise the device and stall the other
// streams.  This entry point calls no cudaMalloc, cudaFree or any allocating
// library routine.
//
// Limits and rules:
//  * the image may hold at most kNoAllocMaxPixels pixels (1,048,576 = 4 MiB of
//    scratch, e.g. 1024 x 1024); larger images are rejected with
//    RGPU_ERR_INVALID_ARG and a message, before any GPU work;
//  * the first call on a device does the set-up (it looks up the scratch
//    array's device address with cudaGetSymbolAddress while that device is
//    current); make that first call before any stream capture;
//  * the scratch array is shared by every call on a device, so calls that
//    overlap in time (from several host threads or on several streams without
//    ordering between them) race on it and corrupt each other's results;
//  * nothing in the scratch needs to start at zero: every blur pass writes the
//    whole intermediate image before the next pass reads it;
//  * with a NULL stream the blur runs on the default stream and the call
//    returns when it has finished; with a caller stream it is only enqueued
//    there and the call returns at once, like the other rgpu_filter_* calls
//    (the scratch is then in use until that stream reaches the end of it).
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "kernels.h"
#include "resvg_gpu.h"

namespace rgpu {
void set_last_error_message(const char *msg);  // render.cpp

namespace {

constexpr size_t kNoAllocMaxPixels = (size_t)1 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint32_t g_box_blur_scratch[kNoAllocMaxPixels];

std::mutex g_setup_mu;
uint32_t *g_scratch_ptr[kMaxDevices] = {};

// Resolves the scratch array's address on the current device once.
int scratch_for_current_device(uint32_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_last_error_message(cudaGetErrorString(e));
        return RGPU_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_error_message("device index beyond the allocation-free entry point's table");
        return RGPU_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        uint32_t *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_box_blur_scratch);
        if (e != cudaSuccess || !p) {
            set_last_error_message(e != cudaSuccess ? cudaGetErrorString(e) : "scratch symbol has no address");
            return RGPU_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return RGPU_OK;
}

}  // namespace
}  // namespace rgpu

extern "C" int rgpu_filter_box_blur_noalloc(uint8_t *device_img, uint32_t width, uint32_t height, double sigma_x,
                                            double sigma_y, void *stream) {
    using namespace rgpu;
    set_last_error_message("");
    if (!device_img || !width || !height) {
        set_last_error_message("invalid arguments");
        return RGPU_ERR_INVALID_ARG;
    }
    if (!(sigma_x >= 0.0 && sigma_x <= kBoxSigmaMax) || !(sigma_y >= 0.0 && sigma_y <= kBoxSigmaMax)) {
        set_last_error_message("standard deviation must be finite, >= 0 and <= 1e8");
        return RGPU_ERR_INVALID_ARG;
    }
    const size_t n = (size_t)width * height;
    if (n > kNoAllocMaxPixels) {
        set_last_error_message("image larger than the allocation-free box blur's scratch (1048576 pixels)");
        return RGPU_ERR_INVALID_ARG;
    }
    uint32_t *scratch = nullptr;
    int r = scratch_for_current_device(&scratch);
    if (r != RGPU_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = filter_box_blur((uint32_t *)device_img, scratch, (int)width, (int)height, sigma_x, sigma_y, s);
    if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error_message(cudaGetErrorString(e));
        return RGPU_ERR_CUDA;
    }
    return RGPU_OK;
}
