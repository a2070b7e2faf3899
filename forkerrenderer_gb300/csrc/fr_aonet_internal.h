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
// Level 0 works on 2x2 pixel blocks: the 4-channel input is rearranged
// space-to-depth into 16 channels at H/2 x W/2, and the 1x1 head emits the
// four sub-pixel AO values of each block.
constexpr int kBlock = 2;
constexpr int kHeadOut = kBlock * kBlock;
constexpr int kHeadParams = kHeadOut * 16 + kHeadOut;
// H and W of a network call must be multiples of kBlock * kScale^2 (the coarsest level).
constexpr int kLevelAlign = kBlock * kScale * kScale;
constexpr int kNumParams = 120196;

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
// The same, for an input already in the 2x2-block layout [B][2][H/2][W/2][8]. With
// B = 1 and bgDepth / bg16 set, pixels whose depth is the cleared FLT_MAX get the
// plain SSAO's background value bg16[(y & 3) * 4 + (x & 3)] instead of the network's.
// allowFused: a single image (B = 1) may run as one cooperative launch of the
// whole network (fr_aonet_set_fused); callers whose streams run other kernels
// concurrently pass false.
int fra_forward_blocks(fr_aonet* n, const uint16_t* in_blocks, int B, int H, int W, float* ao, cudaStream_t st,
                       int* launches, const float* bgDepth = nullptr, const float* bg16 = nullptr,
                       bool allowFused = true);
// Allocates the forward buffers for B x H x W now (no allocation may happen
// while a stream is being captured).
int fra_reserve(fr_aonet* n, int B, int H, int W);
int fra_device(const fr_aonet* n);
// The network's status word (non-zero: a bounded device wait gave up), read and cleared.
int fra_take_status(fr_aonet* n);
