// Network description shared by the U-Net host code and the renderer.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

struct fr_aonet;

namespace fra
{

constexpr int kNumLayers = 10;
// Resolution step between pyramid levels (average pooling / bilinear upsampling factor).
constexpr int kScale = 4;
constexpr int kScaleLog2 = 2;
// H and W of a network call must be multiples of kScale^2 (the coarsest level).
constexpr int kLevelAlign = kScale * kScale;
constexpr int kNumParams = 118417;

// One 3x3 convolution: input channels c0 (+ c1 from a second, concatenated
// tensor), output channels, pyramid level (0 = full resolution), and the number
// of input channels that carry weights (the 4-channel input is padded to 8).
struct LayerSpec
{
    int c0, c1, cout, level, cinReal;
};

extern const LayerSpec kLayers[kNumLayers];

bool make_cp_map(CUtensorMap* m, const void* ptr, int C, int B, int H, int W, int bw, int bh);

}  // namespace fra

// Forward pass on a caller's stream (adds its kernel count to *launches).
int fra_forward(fr_aonet* n, const uint16_t* in, int B, int H, int W, float* ao, cudaStream_t st, int* launches);
int fra_device(const fr_aonet* n);
