// tcgen05 BF16 convolution kernels of the learned ambient-occlusion U-Net.
//
// Activation layout ("chunk-planar", CP): bf16 [B][C/8][H][W][8]. Every pixel
// of an 8-channel chunk is one 16-byte vector, so a TMA box of
// (10 pixels x 8 channels, 18 rows, chunks) lands in shared memory as
// [chunk][y][x][8] -- exactly the no-swizzle core-matrix layout the tensor
// core reads, with zero fill outside the image supplying the convolution's
// zero padding.
//
// Output tiles are 8 x 16 pixels (M = 128 rows of the implicit GEMM: row
// r = 8 * y + x). For tap (dy, dx) the A operand is the halo tile shifted by
// (dy, dx): rows 16 B apart along x, 8-row groups one halo row (160 B) apart,
// K chunks one 8-channel plane (2880 B) apart.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace fra
{

constexpr int kTileW = 8;
constexpr int kTileH = 16;
constexpr int kHaloW = kTileW + 2;
constexpr int kHaloH = kTileH + 2;
constexpr int kRowBytes = kHaloW * 16;               // 160
constexpr int kPlaneBytes = kHaloW * kHaloH * 16;    // 2880
constexpr int kMaxStages = 4;

struct ConvArgs
{
    int B, H, W;
    int tilesX, tilesY, numTiles;
    int c0, c1;          // input channels from map0 / map1 (multiples of 8); cin = c0 + c1
    int cout;            // output channels: multiple of 16, at most 128
    int stages;          // shared-memory pipeline depth (2..kMaxStages)
    int mb;              // M-blocks per tile: the tile is 8 x (16 * mb) pixels
    const uint16_t* wpacked;  // bf16 weights in the shared-memory layout (see pack_conv_weights)
    uint32_t wbytes;
    const float* bias;   // [cout] (forward) or null
    int backward;        // 0: out = relu(acc + bias); 1: out = acc * (mask > 0) (mask optional)
    uint16_t* out0;      // CP tensor receiving channels [0, co0)
    int co0;
    uint16_t* out1;      // CP tensor receiving channels [co0, cout), or null when co0 == cout
    const uint16_t* mask;  // CP tensor with cout channels (backward), or null
    const float* head;   // fused 1x1 head (forward, cout == 16): w[4][16], b[4]; or null
    float* ao;           // [B][2H][2W] sigmoid outputs of the head: sub-pixel (sy, sx) of block (y, x)
                         // is output k = 2 sy + sx
    const float* bgDepth;  // (B = 1) full-resolution depth: where it is FLT_MAX the head writes
    const float* bg16;     // bg16[(y & 3) * 4 + (x & 3)] instead (plain SSAO's background), or null
    int* status;         // bit 1: a pipeline wait timed out
};

struct WgradArgs
{
    int B, H, W;
    int tilesX, tilesY, numTiles;
    int c0, c1;          // X channels from map0 / map1; cin = c0 + c1 <= 120
    int cout;            // dY channels: 16, 32 or 64
    int tapsPerGroup;    // taps handled by one blockIdx.y group
    float* partial;      // [gridDim.y][gridDim.x][tapsPerGroup][cin + 1][cout]
    int* status;
};

// ---- fused forward: the whole network in one cooperative launch ------------------
// Stages run in order with a grid-wide barrier after each: a convolution (its
// tiles spread over the persistent CTAs, weights re-loaded per layer, ring and
// TMEM buffers carried over), or an elementwise pooling / upsampling.
constexpr int kUnetMaxConvs = 10;
constexpr int kUnetMaxStages = 16;
enum UnetStageKind : int
{
    kStageConv = 0,
    kStagePool = 1,  // n output vectors of pool_vec(in, out, i, H, W)
    kStageUp = 2     // n output vectors of up_vec(in, out, i, H = h, W = w)
};

struct UnetConv
{
    CUtensorMap map0, map1;
    ConvArgs a;
};

struct UnetStage
{
    int kind, conv;  // conv: index into UnetArgs::conv
    const uint4* in;
    uint4* out;
    int n, H, W;
};

struct UnetArgs
{
    UnetConv conv[kUnetMaxConvs];
    UnetStage stage[kUnetMaxStages];
    int nStages;
    int ringStages;        // halo ring slots (every layer's tile fits one slot)
    uint32_t wRegion;      // shared bytes before the ring: the largest layer's weights
    uint32_t stageBytes;   // bytes of one ring slot
    uint32_t tmemCols;     // TMEM columns (power of two): the largest layer's two buffers
    unsigned* sync;        // [3] grid barrier count, generation, failure flag (zeroed before the launch)
    int* status;           // bit 4: a grid barrier timed out
    uint64_t waitNs;       // longest wait of a CTA at a grid barrier before it gives up
    int absentCta;         // tests of the bounded barrier: this CTA never arrives at the
                           // first barrier (it leaves the stage loop instead); -1 = none
};

// Launches the fused forward on `grid` co-resident CTAs (cooperative launch).
cudaError_t launch_unet_fwd(const UnetArgs& u, int grid, uint32_t smem, cudaStream_t st);
// CTAs of k_unet_fwd that fit on one SM with `smem` dynamic shared bytes.
int unet_fwd_ctas_per_sm(uint32_t smem);

// Shared-memory bytes of one launch.
uint32_t conv_smem_bytes(int cin, int cout, int stages, bool paired, int mb);
uint32_t wgrad_smem_bytes(int cout);
constexpr int kWgradStages = 2;
constexpr int kWgradXPlanes = 16;  // M = 128 rows = 16 planes of 8 channels

// programmatic: launch as a programmatic dependent of the stream's previous
// kernel (the prologue overlaps its tail; outputs are read after griddepcontrol.wait).
void launch_conv3x3(const CUtensorMap& map0, const CUtensorMap& map1, const ConvArgs& a, int grid,
                    uint32_t smem, cudaStream_t st, bool programmatic);
void launch_wgrad(const CUtensorMap& mapX0, const CUtensorMap& mapX1, const CUtensorMap& mapDY, const WgradArgs& a,
                  int gridX, int gridY, uint32_t smem, cudaStream_t st);

}  // namespace fra
