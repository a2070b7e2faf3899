// Device buffers of a render context, for library code outside fr_context.cu
// (the learned-AO trainer).
#pragma once

#include <cuda_runtime.h>

struct fr_ctx;

float* frctx_ao(fr_ctx* ctx);           // AO plane of the last SSAO pass, W * H floats
const float* frctx_depth(fr_ctx* ctx);  // depth buffer, FLT_MAX where no triangle
cudaStream_t frctx_stream(fr_ctx* ctx);
void frctx_size(const fr_ctx* ctx, int* W, int* H);
