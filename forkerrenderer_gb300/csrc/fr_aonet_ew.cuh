// Elementwise stages of the learned-AO U-Net on chunk-planar BF16 tensors
// ([B][C/8][H][W][8], one 16-byte vector of 8 channels per pixel), shared by the
// per-layer kernels (fr_aonet.cu) and the fused forward (fr_aonet_conv.cu) so
// both compute bit-identical values. Levels are kScale x kScale apart: average
// pooling over kScale x kScale blocks, bilinear upsampling by kScale with
// half-pixel centres and clamped edges.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

#include "fr_aonet_internal.h"

namespace fra
{

constexpr float kPoolNorm = 1.f / (kScale * kScale);

__device__ __forceinline__ void unpack8(uint4 v, float* f)
{
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

__device__ __forceinline__ uint4 pack8(const float* f)
{
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
        w[i] = *reinterpret_cast<const uint32_t*>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// Inputs and weights of output coordinate o of a kScale-times upsampling of n
// samples. kScale = 4: phases 0..3 sit at i - 0.375, i - 0.125, i + 0.125,
// i + 0.375, so the nearer input weighs 0.625, 0.875, 0.875, 0.625.
__device__ __forceinline__ void up_taps(int o, int n, int& i0, int& i1, float& w0, float& w1)
{
    const int i = o / kScale, ph = o % kScale;
    const float nearW = (ph == 0 || ph == kScale - 1) ? 0.625f : 0.875f;
    if (ph < kScale / 2)
    {
        i0 = max(i - 1, 0), i1 = i;
        w1 = nearW, w0 = 1.f - w1;
    }
    else
    {
        i0 = i, i1 = min(i + 1, n - 1);
        w0 = nearW, w1 = 1.f - w0;
    }
}

// Output vector i of the average pooling of in ([BC8][H][W] vectors) into
// out ([BC8][H / kScale][W / kScale]): the block summed row by row, left to right.
__device__ __forceinline__ void pool_vec(const uint4* __restrict__ in, uint4* __restrict__ out, int i, int H, int W)
{
    const int h = H / kScale, w = W / kScale;
    const int x = i % w;
    const int r = i / w;
    const int y = r % h;
    const int bc = r / h;
    const uint4* src = in + (static_cast<size_t>(bc) * H + kScale * y) * W + kScale * x;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
    for (int dy = 0; dy < kScale; ++dy)
        for (int dx = 0; dx < kScale; ++dx)
        {
            unpack8(src[dy * W + dx], v);
#pragma unroll
            for (int e = 0; e < 8; ++e) acc[e] += v[e];
        }
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] *= kPoolNorm;
    out[i] = pack8(acc);
}

// Output vector i of the bilinear upsampling of in ([BC8][h][w]) into
// out ([BC8][kScale h][kScale w]).
__device__ __forceinline__ void up_vec(const uint4* __restrict__ in, uint4* __restrict__ out, int i, int h, int w)
{
    const int H = kScale * h, W = kScale * w;
    const int X = i % W;
    const int r = i / W;
    const int Y = r % H;
    const int bc = r / H;
    int x0, x1, y0, y1;
    float wx0, wx1, wy0, wy1;
    up_taps(X, w, x0, x1, wx0, wx1);
    up_taps(Y, h, y0, y1, wy0, wy1);
    const uint4* src = in + static_cast<size_t>(bc) * h * w;
    float A[8], B[8], C[8], D[8], o[8];
    unpack8(src[y0 * w + x0], A);
    unpack8(src[y0 * w + x1], B);
    unpack8(src[y1 * w + x0], C);
    unpack8(src[y1 * w + x1], D);
#pragma unroll
    for (int e = 0; e < 8; ++e) o[e] = wy0 * (wx0 * A[e] + wx1 * B[e]) + wy1 * (wx0 * C[e] + wx1 * D[e]);
    out[i] = pack8(o);
}

// Output vectors kScale q .. kScale q + kScale - 1 of one output row: the kScale
// phases of input column q, from the three input columns they share (q - 1, q,
// q + 1, clamped), each with up_vec's taps, weights and arithmetic.
// j indexes (bc, output row Y, input column q), q fastest.
__device__ __forceinline__ void up_row(const uint4* __restrict__ in, uint4* __restrict__ out, int j, int h, int w)
{
    static_assert(kScale == 4, "two phases on each side of the input column");
    const int H = kScale * h, W = kScale * w;
    const int q = j % w;
    const int r = j / w;
    const int Y = r % H;
    const int bc = r / H;
    int y0, y1;
    float wy0, wy1;
    up_taps(Y, h, y0, y1, wy0, wy1);
    const uint4* src = in + static_cast<size_t>(bc) * h * w;
    const int xs[3] = {max(q - 1, 0), q, min(q + 1, w - 1)};
    float R0[3][8], R1[3][8];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        unpack8(src[y0 * w + xs[c]], R0[c]);
        unpack8(src[y1 * w + xs[c]], R1[c]);
    }
    uint4* dst = out + (static_cast<size_t>(bc) * H + Y) * W + kScale * q;
#pragma unroll
    for (int ph = 0; ph < kScale; ++ph)
    {
        int x0, x1;
        float wx0, wx1;
        up_taps(kScale * q + ph, w, x0, x1, wx0, wx1);  // x0 = xs[c], x1 = xs[c + 1]
        const int c = ph < kScale / 2 ? 0 : 1;
        const float *A = R0[c], *B = R0[c + 1], *C = R1[c], *D = R1[c + 1];
        float o[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) o[e] = wy0 * (wx0 * A[e] + wx1 * B[e]) + wy1 * (wx0 * C[e] + wx1 * D[e]);
        dst[ph] = pack8(o);
    }
}

}  // namespace fra
