// Allocation-free entry point: the separable ambient-occlusion blur
// (FR_BLUR_SEPARABLE) on a caller-owned device buffer, with its intermediate
// plane in a fixed, file-scope device array instead of memory from cudaMalloc.
//
// It is meant for callers that must not allocate device memory while they
// run: a real-time frame loop that forbids allocation after start-up, a host
// that hands the library only buffers from its own pre-sized pool, or code that
// may not call the CUDA allocator from its thread. The scratch array is part of
// the library image: every GPU that loads the library holds it until the
// process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "fr_kernels.cuh"
#include "forkerrenderer.h"

namespace
{

// Scratch for the horizontal pass of the separable blur: one float per pixel.
static __device__ __align__(256) float g_blur_scratch[FR_NOALLOC_BLUR_MAX_PIXELS];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
float* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_blur_scratch on the current device. In host code the
// array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, once per device, with that device current.
int scratch_for_current_device(float** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FR_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev])
    {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_blur_scratch) != cudaSuccess || !p) return FR_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<float*>(p);
    }
    *out = g_scratch_ptr[dev];
    return FR_OK;
}

}  // namespace

extern "C" int fr_blur_separable_noalloc(float* ao, int32_t width, int32_t height, void* stream)
{
    if (!ao || width <= 0 || height <= 0) return FR_ERR_INVALID;
    if ((long long)width * height > (long long)FR_NOALLOC_BLUR_MAX_PIXELS) return FR_ERR_INVALID;
    // A launch error that earlier work left pending on this thread belongs to
    // that work: it is reported as FR_ERR_CUDA without launching anything, and
    // left pending for its owner to read.
    if (cudaPeekAtLastError() != cudaSuccess) return FR_ERR_CUDA;
    float* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != FR_OK) return rc;
    // Every scratch element the blur reads is written earlier in the same call
    // (the horizontal pass fills width * height values before the vertical pass
    // reads them), so nothing needs clearing between calls.
    int launches = 0;
    frk::launch_blur(FR_BLUR_SEPARABLE, width, height, ao, scratch, reinterpret_cast<cudaStream_t>(stream),
                     launches);
    // Nothing was pending before the launches, so an error now is theirs.
    return cudaGetLastError() == cudaSuccess ? FR_OK : FR_ERR_CUDA;
}
