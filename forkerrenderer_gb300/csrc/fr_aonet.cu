// Learned ambient occlusion: the U-Net of fr_aonet.h -- parameters, Adam,
// forward and backward orchestration, and the CUDA-core kernels around the
// tensor-core convolutions (pooling, bilinear upsampling, head + loss,
// weight-gradient reduction, weight packing).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fr_aonet.h"
#include "fr_aonet_conv.cuh"
#include "fr_aonet_ew.cuh"
#include "fr_aonet_internal.h"

namespace fra
{

const LayerSpec kLayers[kNumLayers] = {
    {16, 0, 16, 0, 16},   // e0a: input, 2x2 pixel blocks (space-to-depth, 16 channels)
    {16, 0, 16, 0, 16},   // e0b -> skip s0
    {16, 0, 32, 1, 16},   // e1a: pooled s0
    {32, 0, 32, 1, 32},   // e1b -> skip s1
    {32, 0, 64, 2, 32},   // b0: pooled s1
    {64, 0, 64, 2, 64},   // b1
    {64, 32, 32, 1, 96},  // d1a: [upsampled b1 | s1]
    {32, 0, 32, 1, 32},   // d1b
    {32, 16, 16, 0, 48},  // d0a: [upsampled d1b | s0]
    {16, 0, 16, 0, 16},   // d0b -> 1x1 head
};

namespace
{

int blocks_for(long long n, int t) { return static_cast<int>((n + t - 1) / t); }

// ---- pooling / upsampling (chunk-planar, one thread per 8-channel vector; the
// per-vector arithmetic is in fr_aonet_ew.cuh) -------------------------------------

__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch as a programmatic dependent of the stream's previous kernel (the kernel
// waits in griddep_wait before it reads that kernel's outputs).
template <typename... KArgs, typename... Args>
void launch_pdl(void (*k)(KArgs...), int grid, int block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

__global__ void k_pool_fwd(const uint4* __restrict__ in, uint4* __restrict__ out, int BC8, int H, int W)
{
    griddep_wait();
    const int n = BC8 * (H / kScale) * (W / kScale);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pool_vec(in, out, i, H, W);
}

// g(y,x) = (gc(y,x) + gp(y/kScale, x/kScale) / kScale^2) * (mask(y,x) > 0)
__global__ void k_pool_bwd_add_mask(const uint4* __restrict__ gc, const uint4* __restrict__ gp,
                                    const uint4* __restrict__ mask, uint4* __restrict__ out, int BC8, int H, int W)
{
    const int n = BC8 * H * W;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = i % W;
    const int r = i / W;
    const int y = r % H;
    const int bc = r / H;
    float a[8], p[8], m[8], o[8];
    unpack8(gc[i], a);
    unpack8(gp[(static_cast<size_t>(bc) * (H / kScale) + y / kScale) * (W / kScale) + x / kScale], p);
    unpack8(mask[i], m);
#pragma unroll
    for (int e = 0; e < 8; ++e) o[e] = m[e] > 0.f ? a[e] + kPoolNorm * p[e] : 0.f;
    out[i] = pack8(o);
}

// out(Y,X) = wy0 * (wx0 * A + wx1 * B) + wy1 * (wx0 * C + wx1 * D),
// A = in(y0,x0), B = in(y0,x1), C = in(y1,x0), D = in(y1,x1).
// One thread per kScale output vectors of a row (up_row).
__global__ void k_up_fwd(const uint4* __restrict__ in, uint4* __restrict__ out, int BC8, int h, int w)
{
    griddep_wait();
    const int n = BC8 * (kScale * h) * w;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) up_row(in, out, j, h, w);
}

// Weight of input index j in output o (both taps may clamp onto j).
__device__ __forceinline__ float up_weight(int o, int j, int n)
{
    int i0, i1;
    float w0, w1;
    up_taps(o, n, i0, i1, w0, w1);
    return (i0 == j ? w0 : 0.f) + (i1 == j ? w1 : 0.f);
}

// Transpose of k_up_fwd, then the ReLU mask of the low-resolution activation:
// g(j,i) = (sum_oy w(oy) * sum_ox w(ox) * G(oy,ox)) * (mask(j,i) > 0), outputs in ascending order.
__global__ void k_up_bwd_mask(const uint4* __restrict__ G, const uint4* __restrict__ mask, uint4* __restrict__ out,
                              int BC8, int h, int w)
{
    const int H = kScale * h, W = kScale * w;
    const int n = BC8 * h * w;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int i = idx % w;
    const int r = idx / w;
    const int j = r % h;
    const int bc = r / h;
    const uint4* src = G + static_cast<size_t>(bc) * H * W;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int oy = kScale * j - kScale / 2; oy < kScale * j + kScale + kScale / 2; ++oy)
    {
        if (oy < 0 || oy >= H) continue;
        const float wy = up_weight(oy, j, h);
        if (wy == 0.f) continue;
        float row[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int ox = kScale * i - kScale / 2; ox < kScale * i + kScale + kScale / 2; ++ox)
        {
            if (ox < 0 || ox >= W) continue;
            const float wx = up_weight(ox, i, w);
            if (wx == 0.f) continue;
            float g[8];
            unpack8(src[oy * W + ox], g);
#pragma unroll
            for (int e = 0; e < 8; ++e) row[e] += wx * g[e];
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) acc[e] += wy * row[e];
    }
    float m[8];
    unpack8(mask[idx], m);
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = m[e] > 0.f ? acc[e] : 0.f;
    out[idx] = pack8(acc);
}

// ---- input rearrangement, head backward + loss ---------------------------------

// Space-to-depth of the 4-channel input: level-0 pixel (Y, X) holds the 2x2 block
// of full-resolution pixels, chunk c8 = row 2Y + c8 as [pixel 2X ch0..3 | pixel 2X+1 ch0..3].
__global__ void k_s2d(const uint4* __restrict__ in, uint4* __restrict__ out, int B, int h, int w)
{
    const int n = B * 2 * h * w;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int X = i % w;
    const int r = i / w;
    const int Y = r % h;
    const int bc = r / h;
    const int b = bc >> 1, c8 = bc & 1;
    const uint4* src = in + (static_cast<size_t>(b) * 2 * h + 2 * Y + c8) * (2 * w) + 2 * X;
    const uint4 p0 = src[0], p1 = src[1];
    out[i] = make_uint4(p0.x, p0.y, p1.x, p1.y);
}

constexpr int kHeadSums = 1 + kHeadParams;  // loss, d head w[4][16], d head b[4]
constexpr int kHeadThreads = 256;

// Per level-0 pixel and sub-pixel k: diff = ao - label (0 where label < 0);
// loss += diff^2; dz_k = 2 diff / N * ao (1 - ao); g7[c] = (sum_k dz_k hw[k][c]) * (a7[c] > 0);
// d hw[k][c] += dz_k a7[c]; d hb[k] += dz_k. Per-block sums go to part[block][kHeadSums].
__global__ void __launch_bounds__(kHeadThreads) k_head_bwd(const float* __restrict__ ao, const float* __restrict__ label,
                                                           const uint4* __restrict__ a7, const float* __restrict__ hw,
                                                           uint4* __restrict__ g7, float* __restrict__ part, int B,
                                                           int h, int w, float invN)
{
    __shared__ float red[kHeadSums][kHeadThreads / 32];
    const int HW = h * w;
    const int n = B * HW;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float s[kHeadSums];
#pragma unroll
    for (int k = 0; k < kHeadSums; ++k) s[k] = 0.f;
    if (p < n)
    {
        const int b = p / HW, pix = p - b * HW;
        const int Y = pix / w, X = pix - Y * w;
        float dz[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const size_t fi = (static_cast<size_t>(b) * 2 * h + 2 * Y + (k >> 1)) * (2 * w) + 2 * X + (k & 1);
            const float a = ao[fi];
            const float lab = label[fi];
            const float diff = lab >= 0.f ? a - lab : 0.f;  // a negative label marks a pixel outside the loss
            dz[k] = 2.f * diff * invN * a * (1.f - a);
            s[0] += diff * diff;
            s[1 + kHeadOut * 16 + k] = dz[k];
        }
        for (int c8 = 0; c8 < 2; ++c8)
        {
            const size_t vi = (static_cast<size_t>(b) * 2 + c8) * HW + pix;
            float hv[8], g[8];
            unpack8(a7[vi], hv);
#pragma unroll
            for (int e = 0; e < 8; ++e)
            {
                const int c = c8 * 8 + e;
                const float gs = ((dz[0] * hw[c] + dz[1] * hw[16 + c]) + dz[2] * hw[32 + c]) + dz[3] * hw[48 + c];
                g[e] = hv[e] > 0.f ? gs : 0.f;
#pragma unroll
                for (int k = 0; k < 4; ++k) s[1 + k * 16 + c] = dz[k] * hv[e];
            }
            g7[vi] = pack8(g);
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kHeadSums; ++k)
    {
        float v = s[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][wid] = v;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kHeadSums; k += blockDim.x)
    {
        float v = 0.f;
        for (int q = 0; q < kHeadThreads / 32; ++q) v += red[k][q];
        part[static_cast<size_t>(blockIdx.x) * kHeadSums + k] = v;
    }
}

// Sums the per-block head partials in a fixed order, one CTA per sum: loss ->
// out_loss, head grads -> grads. Each thread adds the blocks b = t mod 256, then a
// pairwise tree combines the 256 threads' sums (FP64 adds are slow on this GPU:
// a chain as long as the block count would dominate the training step).
constexpr int kHeadReduceThreads = 256;
__global__ void __launch_bounds__(kHeadReduceThreads) k_head_reduce(const float* __restrict__ part, int nblocks,
                                                                    float* __restrict__ grads_head,
                                                                    float* __restrict__ out_loss, float invN)
{
    const int k = blockIdx.x;  // gridDim.x == kHeadSums
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kHeadReduceThreads) acc += part[static_cast<size_t>(b) * kHeadSums + k];
    __shared__ double sum[kHeadReduceThreads];
    sum[threadIdx.x] = acc;
    __syncthreads();
    for (int h = kHeadReduceThreads / 2; h > 0; h >>= 1)
    {
        if (threadIdx.x < h) sum[threadIdx.x] += sum[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    if (k == 0)
        *out_loss = static_cast<float>(sum[0] * invN);
    else
        grads_head[k - 1] = static_cast<float>(sum[0]);  // w[4][16], then b[4]
}

// dW[co][ci][t] = sum over CTAs of partial[gy][cta][tt][ci][co] (t = gy * tpg + tt); db from row cin.
__global__ void k_wgrad_reduce(const float* __restrict__ partial, int gridX, int tpg, int cin, int cinReal, int cout,
                               float* __restrict__ dW, float* __restrict__ db)
{
    const int nW = cout * cinReal * 9;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nW + cout) return;
    int co, ci, t;
    if (i < nW)
    {
        co = i / (cinReal * 9);
        const int r = i - co * cinReal * 9;
        ci = r / 9;
        t = r - ci * 9;
    }
    else
    {
        co = i - nW;
        ci = cin;  // bias row
        t = 0;
    }
    const int gy = t / tpg, tt = t - gy * tpg;
    // 8 interleaved FP64 sums (CTA bx into sum bx mod 8), then combined pairwise:
    // a dependent chain of gridX / 8 + 3 adds instead of gridX
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const size_t stride = static_cast<size_t>(tpg) * (cin + 1) * cout;
    const float* src = partial + ((static_cast<size_t>(gy) * gridX * tpg + tt) * (cin + 1) + ci) * cout + co;
    int bx = 0;
    for (; bx + 8 <= gridX; bx += 8)
    {
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] += src[(bx + j) * stride];
    }
    for (int j = 0; bx + j < gridX; ++j) acc[j] += src[(bx + j) * stride];
    const double total = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
    if (i < nW)
        dW[i] = static_cast<float>(total);
    else
        db[co] = static_cast<float>(total);
}

// PyTorch's Adam: m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
// p -= step * m / (sqrt(v) / bc2sqrt + eps), step = lr / (1 - b1^t), bc2sqrt = sqrt(1 - b2^t).
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float b1, float b2, float eps, float step, float bc2sqrt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * (gi * gi);
    m[i] = mi;
    v[i] = vi;
    p[i] -= step * (mi / (sqrtf(vi) / bc2sqrt + eps));
}

__constant__ int c_pairA[5] = {0, 2, 4, 6, 7};
__constant__ int c_pairB[5] = {1, 3, 5, 7, 8};

// Packs FP32 W[cout][cinReal][9] into the BF16 shared-memory layouts of k_conv3x3:
// forward  [tap][cin/8][cout][8]           (paired input layer: [pair][2][cout][8])
// backward [tap'][cout/8][cin][8] with W'[ci][co][t'] = W[co][ci][8 - t'] (a 3x3
//          convolution of the output gradient gives the input gradient).
__global__ void k_pack(const float* __restrict__ W, int cin, int cinReal, int cout, int paired,
                       __nv_bfloat16* __restrict__ fwd, __nv_bfloat16* __restrict__ bwd)
{
    const int nf = paired ? 5 * 2 * cout * 8 : 9 * cin * cout;
    const int nb = bwd ? 9 * cin * cout : 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nf)
    {
        const int e = i & 7;
        const int r = i >> 3;
        const int co = r % cout;
        const int q = r / cout;  // tap * (cin/8) + chunk, or pair * 2 + which
        float val = 0.f;
        if (paired)
        {
            const int pr = q >> 1, which = q & 1;
            const int t = which ? c_pairB[pr] : c_pairA[pr];
            if (e < cinReal && !(pr == 4 && which == 0)) val = W[(co * cinReal + e) * 9 + t];
        }
        else
        {
            const int t = q / (cin / 8), cc = q % (cin / 8);
            const int ci = cc * 8 + e;
            if (ci < cinReal) val = W[(co * cinReal + ci) * 9 + t];
        }
        fwd[i] = __float2bfloat16_rn(val);
    }
    else if (i < nf + nb)
    {
        const int k = i - nf;
        const int e = k & 7;
        const int r = k >> 3;
        const int ci = r % cin;  // output channel of the backward convolution
        const int q = r / cin;   // tap' * (cout/8) + chunk
        const int tp = q / (cout / 8), cc = q % (cout / 8);
        const int co = cc * 8 + e;
        bwd[k] = __float2bfloat16_rn(W[(co * cinReal + ci) * 9 + (8 - tp)]);
    }
}

// ---- tensor maps ------------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

}  // namespace

// 3-D map over a chunk-planar tensor: (W * 8 elements, H, B * C/8), box
// (bw * 8, bh, C/8). A box row is bw whole pixels (bw * 16 contiguous bytes);
// x coordinates are 8 * pixel, so every start is 16-byte aligned.
bool make_cp_map(CUtensorMap* m, const void* ptr, int C, int B, int H, int W, int bw, int bh)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    std::memset(m, 0, sizeof *m);
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(W) * 8, static_cast<cuuint64_t>(H),
                          static_cast<cuuint64_t>(B) * (C / 8)};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(W) * 16, static_cast<cuuint64_t>(W) * H * 16};
    cuuint32_t box[3] = {static_cast<cuuint32_t>(bw) * 8, static_cast<cuuint32_t>(bh), static_cast<cuuint32_t>(C / 8)};
    cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(ptr), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace fra

using namespace fra;

// ------------------------------------------------------------------------------------
// Network object
// ------------------------------------------------------------------------------------

namespace
{

struct DevBuf
{
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct fr_aonet
{
    int device = 0;
    int numSMs = 0;
    // background of the head's full-resolution AO (fra_forward_blocks with B = 1):
    // where depth is the cleared FLT_MAX the AO is bg16[noise cell]
    const float* bgDepth = nullptr;
    const float* bg16 = nullptr;
    // fused forward (k_unet_fwd) for single images: its grid barrier words
    unsigned* unetSync = nullptr;
    bool fused = false;
    uint64_t barrierWaitNs = 2000000000ull;  // 2 s: far above any legitimate wait
    int absentCta = -1;
    std::string err;
    int paramOff[kNumLayers + 1] = {};  // W offsets; bias follows W; [kNumLayers] = head
    float* params = nullptr;
    float* grads = nullptr;
    float* adamM = nullptr;
    float* adamV = nullptr;
    long long adamT = 0;
    __nv_bfloat16* packFwd[kNumLayers] = {};
    __nv_bfloat16* packBwd[kNumLayers] = {};
    uint32_t packFwdBytes[kNumLayers] = {};
    int* status = nullptr;
    float* lossDev = nullptr;
    float* headPart = nullptr;
    int headPartCap = 0;
    float* partial = nullptr;
    size_t partialCap = 0;
    // activations (forward) and gradients (backward), sized for capPix pixels at level 0
    long long capFwd = 0, capBwd = 0;
    std::vector<DevBuf> fwdBufs, bwdBufs;
    uint16_t *xs, *a0, *s0, *p0, *a1, *s1, *p1, *a2, *a3, *u1, *a4, *a5, *u0, *a6, *a7;
    uint16_t *g7, *g6, *gu0, *gs0c, *g5, *g4, *gu1, *gs1c, *g3, *g2, *gp1, *gS1, *g1, *gp0, *gS0, *g0;
    float* aoTmp = nullptr;
    int launches = 0;
};

namespace
{

int net_fail(fr_aonet* n, int code, const std::string& msg)
{
    if (n) n->err = msg;
    return code;
}

#define NET_CUDA(n, x)                                                                                          \
    do                                                                                                          \
    {                                                                                                           \
        cudaError_t e_ = (x);                                                                                   \
        if (e_ != cudaSuccess) return net_fail((n), FR_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

int w_count(int L) { return kLayers[L].cout * kLayers[L].cinReal * 9; }

struct DeviceGuard
{
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01(uint64_t& s) { return (static_cast<double>(splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

double gaussian(uint64_t& s)
{
    const double u = uniform01(s), v = uniform01(s);
    return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
}

int alloc_set(fr_aonet* n, std::vector<DevBuf>& set, const std::vector<std::pair<uint16_t**, size_t>>& want)
{
    for (auto& b : set) cudaFree(b.p);
    set.clear();
    for (auto& w : want)
    {
        DevBuf b;
        b.bytes = w.second;
        NET_CUDA(n, cudaMalloc(&b.p, b.bytes));
        *w.first = static_cast<uint16_t*>(b.p);
        set.push_back(b);
    }
    return FR_OK;
}

// Bytes of a chunk-planar tensor with C channels at level `lv` for `pix` level-0 pixels.
size_t cp_bytes(long long pix, int C, int lv) { return static_cast<size_t>(pix >> (2 * kScaleLog2 * lv)) * C * 2 + 256; }

int ensure_fwd(fr_aonet* n, long long pix)
{
    if (pix <= n->capFwd) return FR_OK;
    std::vector<std::pair<uint16_t**, size_t>> w = {
        {&n->xs, cp_bytes(pix, 16, 0)},
        {&n->a0, cp_bytes(pix, 16, 0)}, {&n->s0, cp_bytes(pix, 16, 0)}, {&n->p0, cp_bytes(pix, 16, 1)},
        {&n->a1, cp_bytes(pix, 32, 1)}, {&n->s1, cp_bytes(pix, 32, 1)}, {&n->p1, cp_bytes(pix, 32, 2)},
        {&n->a2, cp_bytes(pix, 64, 2)}, {&n->a3, cp_bytes(pix, 64, 2)}, {&n->u1, cp_bytes(pix, 64, 1)},
        {&n->a4, cp_bytes(pix, 32, 1)}, {&n->a5, cp_bytes(pix, 32, 1)}, {&n->u0, cp_bytes(pix, 32, 0)},
        {&n->a6, cp_bytes(pix, 16, 0)}, {&n->a7, cp_bytes(pix, 16, 0)},
        {reinterpret_cast<uint16_t**>(&n->aoTmp), static_cast<size_t>(pix) * kHeadOut * 4 + 256}};
    int rc = alloc_set(n, n->fwdBufs, w);
    if (rc != FR_OK)
    {
        n->capFwd = 0;
        return rc;
    }
    n->capFwd = pix;
    return FR_OK;
}

int ensure_bwd(fr_aonet* n, long long pix)
{
    if (pix <= n->capBwd) return FR_OK;
    std::vector<std::pair<uint16_t**, size_t>> w = {
        {&n->g7, cp_bytes(pix, 16, 0)},  {&n->g6, cp_bytes(pix, 16, 0)},  {&n->gu0, cp_bytes(pix, 32, 0)},
        {&n->gs0c, cp_bytes(pix, 16, 0)}, {&n->g5, cp_bytes(pix, 32, 1)},  {&n->g4, cp_bytes(pix, 32, 1)},
        {&n->gu1, cp_bytes(pix, 64, 1)}, {&n->gs1c, cp_bytes(pix, 32, 1)}, {&n->g3, cp_bytes(pix, 64, 2)},
        {&n->g2, cp_bytes(pix, 64, 2)},  {&n->gp1, cp_bytes(pix, 32, 2)}, {&n->gS1, cp_bytes(pix, 32, 1)},
        {&n->g1, cp_bytes(pix, 32, 1)},  {&n->gp0, cp_bytes(pix, 16, 1)}, {&n->gS0, cp_bytes(pix, 16, 0)},
        {&n->g0, cp_bytes(pix, 16, 0)}};
    int rc = alloc_set(n, n->bwdBufs, w);
    if (rc != FR_OK)
    {
        n->capBwd = 0;
        return rc;
    }
    const int hb = blocks_for(pix, kHeadThreads);
    if (hb > n->headPartCap)
    {
        cudaFree(n->headPart);
        NET_CUDA(n, cudaMalloc(&n->headPart, sizeof(float) * kHeadSums * hb));
        n->headPartCap = hb;
    }
    n->capBwd = pix;
    return FR_OK;
}

int pack_all(fr_aonet* n, cudaStream_t st)
{
    for (int L = 0; L < kNumLayers; ++L)
    {
        const LayerSpec& s = kLayers[L];
        const int cin = s.c0 + s.c1;
        const int paired = cin == 8;
        const int nf = paired ? 5 * 2 * s.cout * 8 : 9 * cin * s.cout;
        const int nb = L > 0 ? 9 * cin * s.cout : 0;
        k_pack<<<blocks_for(nf + nb, 256), 256, 0, st>>>(n->params + n->paramOff[L], cin, s.cinReal, s.cout, paired,
                                                          n->packFwd[L], L > 0 ? n->packBwd[L] : nullptr);
    }
    NET_CUDA(n, cudaGetLastError());
    return FR_OK;
}

struct Shape
{
    int B, H, W;  // level 0: the 2x2 pixel blocks (half the input resolution)
    int h(int lv) const { return H >> (kScaleLog2 * lv); }
    int w(int lv) const { return W >> (kScaleLog2 * lv); }
};

// One 3x3 convolution (forward or backward-data) on the tensor cores.
// Large maps use 8 x 64 tiles (4 M-blocks per stage); small ones 8 x 16 tiles
// for more CTAs. programmatic: launched as a programmatic dependent of the
// previous kernel on the stream.
// One convolution's launch: tensor maps, arguments, shared memory and grid.
struct ConvPlan
{
    CUtensorMap m0, m1;
    ConvArgs a;
    uint32_t smem;       // dynamic shared bytes of a standalone launch
    int grid;            // CTAs of a standalone launch
    uint32_t wAligned;   // weight region (1 KB aligned)
    uint32_t stageBytes; // one halo ring slot (1 KB aligned)
    uint32_t tmemCols;   // two accumulator buffers
};

int plan_conv(fr_aonet* n, const Shape& S, int lv, const uint16_t* in0, int c0, const uint16_t* in1, int c1, int cout,
              const __nv_bfloat16* wpacked, uint32_t wbytes, const float* bias, bool backward, uint16_t* out0, int co0,
              uint16_t* out1, const uint16_t* mask, const float* head, float* ao, ConvPlan& P)
{
    const int H = S.h(lv), W = S.w(lv);
    const int cin = c0 + c1;
    const bool paired = cin == 8;
    const long long tiles1 = static_cast<long long>(S.B) * ((W + kTileW - 1) / kTileW) * ((H + kTileH - 1) / kTileH);
    int mb = (tiles1 >= 16LL * n->numSMs && 2 * 4 * cout <= 512) ? 4 : 1;
    while (mb > 1 && conv_smem_bytes(cin, cout, 2, paired, mb) > 200u * 1024u) mb >>= 1;
    const int tileH = kTileH * mb;
    if (!make_cp_map(&P.m0, in0, c0, S.B, H, W, kHaloW, tileH + 2)) return net_fail(n, FR_ERR_CUDA, "tensor map encode");
    if (c1 > 0)
    {
        if (!make_cp_map(&P.m1, in1, c1, S.B, H, W, kHaloW, tileH + 2))
            return net_fail(n, FR_ERR_CUDA, "tensor map encode");
    }
    else
        P.m1 = P.m0;
    ConvArgs& a = P.a;
    a = ConvArgs{};
    a.B = S.B, a.H = H, a.W = W;
    a.mb = mb;
    a.tilesX = (W + kTileW - 1) / kTileW;
    a.tilesY = (H + tileH - 1) / tileH;
    a.numTiles = S.B * a.tilesX * a.tilesY;
    a.c0 = c0, a.c1 = c1, a.cout = cout;
    a.wpacked = reinterpret_cast<const uint16_t*>(wpacked);
    a.wbytes = wbytes;
    a.bias = bias;
    a.backward = backward ? 1 : 0;
    a.out0 = out0, a.co0 = co0, a.out1 = out1;
    a.mask = mask;
    a.head = head;
    a.ao = ao;
    a.bgDepth = head ? n->bgDepth : nullptr;
    a.bg16 = head ? n->bg16 : nullptr;
    a.status = n->status;
    // Pipeline depth: as many halo stages as fit next to the weights (2..4), fewer
    // where that keeps 4 CTAs on an SM (their epilogues overlap: the 48-channel
    // level-0 layer runs 4 CTAs of 2 stages per SM faster than 2 CTAs of 4 stages).
    int stages = kMaxStages;
    while (stages > 2 && conv_smem_bytes(cin, cout, stages, paired, mb) > 200u * 1024u) --stages;
    while (stages > 2 && (228u * 1024u) / (conv_smem_bytes(cin, cout, stages, paired, mb) + 2048u) < 4u) --stages;
    a.stages = stages;
    P.smem = conv_smem_bytes(cin, cout, stages, paired, mb);
    const int cols = 2 * mb * cout;
    const int tmemCols = cols <= 32 ? 32 : cols <= 64 ? 64 : cols <= 128 ? 128 : cols <= 256 ? 256 : 512;
    int perSM = static_cast<int>((228u * 1024u) / (P.smem + 2048u));
    // at most 5 CTAs of 192 threads at 60 registers share an SM's 64 K registers
    perSM = std::max(1, std::min(perSM, std::min(512 / tmemCols, 5)));
    P.grid = std::min(a.numTiles, n->numSMs * perSM);
    const int tileRows = tileH + 2;
    P.wAligned = (wbytes + 1023u) & ~1023u;
    P.stageBytes = ((static_cast<uint32_t>(cin / 8) * kHaloW * tileRows * 16u) + 1023u) & ~1023u;
    P.tmemCols = static_cast<uint32_t>(tmemCols);
    return FR_OK;
}

int conv(fr_aonet* n, const Shape& S, int lv, const uint16_t* in0, int c0, const uint16_t* in1, int c1, int cout,
         const __nv_bfloat16* wpacked, uint32_t wbytes, const float* bias, bool backward, uint16_t* out0, int co0,
         uint16_t* out1, const uint16_t* mask, const float* head, float* ao, cudaStream_t st,
         bool programmatic = false)
{
    ConvPlan P;
    int rc = plan_conv(n, S, lv, in0, c0, in1, c1, cout, wpacked, wbytes, bias, backward, out0, co0, out1, mask, head,
                       ao, P);
    if (rc != FR_OK) return rc;
    launch_conv3x3(P.m0, P.m1, P.a, P.grid, P.smem, st, programmatic);
    n->launches++;
    return FR_OK;
}

// Weight gradient of layer L from its input X (one or two tensors) and its output gradient dY.
int wgrad(fr_aonet* n, const Shape& S, int L, const uint16_t* x0, const uint16_t* x1, const uint16_t* dY,
          cudaStream_t st)
{
    const LayerSpec& s = kLayers[L];
    const int lv = s.level;
    const int H = S.h(lv), W = S.w(lv);
    CUtensorMap mx0, mx1, mdy;
    if (!make_cp_map(&mx0, x0, s.c0, S.B, H, W, kHaloW, kHaloH) ||
        (s.c1 > 0 && !make_cp_map(&mx1, x1, s.c1, S.B, H, W, kHaloW, kHaloH)) ||
        !make_cp_map(&mdy, dY, s.cout, S.B, H, W, kTileW, kTileH))
        return net_fail(n, FR_ERR_CUDA, "tensor map encode");
    if (s.c1 == 0) mx1 = mx0;
    WgradArgs a{};
    a.B = S.B, a.H = H, a.W = W;
    a.tilesX = (W + kTileW - 1) / kTileW;
    a.tilesY = (H + kTileH - 1) / kTileH;
    a.numTiles = S.B * a.tilesX * a.tilesY;
    a.c0 = s.c0, a.c1 = s.c1, a.cout = s.cout;
    a.tapsPerGroup = s.cout == 64 ? 5 : 9;
    const int gridY = (9 + a.tapsPerGroup - 1) / a.tapsPerGroup;
    const int gridX = std::min(a.numTiles, n->numSMs);
    const int cin = s.c0 + s.c1;
    const size_t need = static_cast<size_t>(gridY) * gridX * a.tapsPerGroup * (cin + 1) * s.cout;
    if (need > n->partialCap) return net_fail(n, FR_ERR_INVALID, "wgrad partial buffer too small");
    a.partial = n->partial;
    a.status = n->status;
    launch_wgrad(mx0, mx1, mdy, a, gridX, gridY, wgrad_smem_bytes(s.cout), st);
    const int nOut = w_count(L) + s.cout;
    k_wgrad_reduce<<<blocks_for(nOut, 256), 256, 0, st>>>(n->partial, gridX, a.tapsPerGroup, cin, s.cinReal, s.cout,
                                                          n->grads + n->paramOff[L],
                                                          n->grads + n->paramOff[L] + w_count(L));
    n->launches += 2;
    return FR_OK;
}

int check_shape(fr_aonet* n, int B, int H, int W)
{
    if (B <= 0 || H <= 0 || W <= 0 || H % kLevelAlign || W % kLevelAlign)
        return net_fail(n, FR_ERR_INVALID, "B, H, W must be positive and H, W multiples of 32");
    if (static_cast<long long>(B) * H * W > FR_AONET_MAX_PIXELS)
        return net_fail(n, FR_ERR_INVALID, "B * H * W exceeds FR_AONET_MAX_PIXELS");
    return FR_OK;
}

#define NET_TRY(x)                \
    do                            \
    {                             \
        int rc_ = (x);            \
        if (rc_ != FR_OK) return rc_; \
    } while (0)

// in: [B][1][2H][2W][8] (full-resolution input), or the 2x2-block layout
// [B][2][H][W][8] when inBlocks (then the space-to-depth pass is skipped).
int forward_impl(fr_aonet* n, const uint16_t* in, const Shape& S, float* ao, cudaStream_t st, bool inBlocks = false)
{
    const long long pix = static_cast<long long>(S.B) * S.H * S.W;
    NET_TRY(ensure_fwd(n, pix));
    auto P = [&](int L) { return n->params + n->paramOff[L] + w_count(L); };  // bias
    const float* head = n->params + n->paramOff[kNumLayers];
    auto CV = [&](int L, const uint16_t* i0, const uint16_t* i1, uint16_t* out, const float* hd, float* aoOut) {
        const LayerSpec& s = kLayers[L];
        return conv(n, S, s.level, i0, s.c0, i1, s.c1, s.cout, n->packFwd[L], n->packFwdBytes[L], P(L), false, out,
                    s.cout, nullptr, nullptr, hd, aoOut, st, true);
    };
    const uint16_t* x0 = in;
    if (!inBlocks)
    {
        k_s2d<<<blocks_for((long long)S.B * 2 * S.H * S.W, 256), 256, 0, st>>>(
            reinterpret_cast<const uint4*>(in), reinterpret_cast<uint4*>(n->xs), S.B, S.H, S.W);
        x0 = n->xs;
        n->launches++;
    }
    NET_TRY(CV(0, x0, nullptr, n->a0, nullptr, nullptr));
    NET_TRY(CV(1, n->a0, nullptr, n->s0, nullptr, nullptr));
    launch_pdl(k_pool_fwd, blocks_for((long long)S.B * 2 * S.h(1) * S.w(1), 256), 256, st,
               reinterpret_cast<const uint4*>(n->s0), reinterpret_cast<uint4*>(n->p0), S.B * 2, S.H, S.W);
    NET_TRY(CV(2, n->p0, nullptr, n->a1, nullptr, nullptr));
    NET_TRY(CV(3, n->a1, nullptr, n->s1, nullptr, nullptr));
    launch_pdl(k_pool_fwd, blocks_for((long long)S.B * 4 * S.h(2) * S.w(2), 256), 256, st,
               reinterpret_cast<const uint4*>(n->s1), reinterpret_cast<uint4*>(n->p1), S.B * 4, S.h(1), S.w(1));
    NET_TRY(CV(4, n->p1, nullptr, n->a2, nullptr, nullptr));
    NET_TRY(CV(5, n->a2, nullptr, n->a3, nullptr, nullptr));
    launch_pdl(k_up_fwd, blocks_for((long long)S.B * 8 * S.h(1) * S.w(2), 256), 256, st,
               reinterpret_cast<const uint4*>(n->a3), reinterpret_cast<uint4*>(n->u1), S.B * 8, S.h(2), S.w(2));
    NET_TRY(CV(6, n->u1, n->s1, n->a4, nullptr, nullptr));
    NET_TRY(CV(7, n->a4, nullptr, n->a5, nullptr, nullptr));
    launch_pdl(k_up_fwd, blocks_for((long long)S.B * 4 * S.H * S.w(1), 256), 256, st,
               reinterpret_cast<const uint4*>(n->a5), reinterpret_cast<uint4*>(n->u0), S.B * 4, S.h(1), S.w(1));
    NET_TRY(CV(8, n->u0, n->s0, n->a6, nullptr, nullptr));
    NET_TRY(CV(9, n->a6, nullptr, n->a7, head, ao));
    n->launches += 4;
    NET_CUDA(n, cudaGetLastError());
    return FR_OK;
}

// The same forward as forward_impl (2x2-block input), in one cooperative launch
// of k_unet_fwd. Returns FR_ERR_UNSUPPORTED when the layers' buffers do not fit
// one CTA per SM (the caller then launches layer by layer).
int forward_fused(fr_aonet* n, const uint16_t* in_blocks, const Shape& S, float* ao, cudaStream_t st)
{
    const long long pix = static_cast<long long>(S.B) * S.H * S.W;
    NET_TRY(ensure_fwd(n, pix));
    UnetArgs U{};
    uint32_t wRegion = 0, stageBytes = 0, tmemCols = 32;
    auto P = [&](int L) { return n->params + n->paramOff[L] + w_count(L); };  // bias
    const float* head = n->params + n->paramOff[kNumLayers];
    auto CV = [&](int L, const uint16_t* i0, const uint16_t* i1, uint16_t* out, const float* hd, float* aoOut) {
        const LayerSpec& sp = kLayers[L];
        ConvPlan cp;
        const int rc = plan_conv(n, S, sp.level, i0, sp.c0, i1, sp.c1, sp.cout, n->packFwd[L], n->packFwdBytes[L], P(L),
                                 false, out, sp.cout, nullptr, nullptr, hd, aoOut, cp);
        if (rc != FR_OK) return rc;
        U.conv[L] = UnetConv{cp.m0, cp.m1, cp.a};
        U.stage[U.nStages++] = UnetStage{kStageConv, L, nullptr, nullptr, 0, 0, 0};
        wRegion = std::max(wRegion, cp.wAligned);
        stageBytes = std::max(stageBytes, cp.stageBytes);
        tmemCols = std::max(tmemCols, cp.tmemCols);
        return FR_OK;
    };
    auto EW = [&](int kind, const uint16_t* in, uint16_t* out, int nvec, int H, int W) {
        U.stage[U.nStages++] = UnetStage{kind, -1, reinterpret_cast<const uint4*>(in), reinterpret_cast<uint4*>(out),
                                         nvec, H, W};
    };
    NET_TRY(CV(0, in_blocks, nullptr, n->a0, nullptr, nullptr));
    NET_TRY(CV(1, n->a0, nullptr, n->s0, nullptr, nullptr));
    EW(kStagePool, n->s0, n->p0, S.B * 2 * S.h(1) * S.w(1), S.H, S.W);
    NET_TRY(CV(2, n->p0, nullptr, n->a1, nullptr, nullptr));
    NET_TRY(CV(3, n->a1, nullptr, n->s1, nullptr, nullptr));
    EW(kStagePool, n->s1, n->p1, S.B * 4 * S.h(2) * S.w(2), S.h(1), S.w(1));
    NET_TRY(CV(4, n->p1, nullptr, n->a2, nullptr, nullptr));
    NET_TRY(CV(5, n->a2, nullptr, n->a3, nullptr, nullptr));
    EW(kStageUp, n->a3, n->u1, S.B * 8 * S.h(1) * S.w(1), S.h(2), S.w(2));
    NET_TRY(CV(6, n->u1, n->s1, n->a4, nullptr, nullptr));
    NET_TRY(CV(7, n->a4, nullptr, n->a5, nullptr, nullptr));
    EW(kStageUp, n->a5, n->u0, S.B * 4 * S.H * S.W, S.h(1), S.w(1));
    NET_TRY(CV(8, n->u0, n->s0, n->a6, nullptr, nullptr));
    NET_TRY(CV(9, n->a6, nullptr, n->a7, head, ao));
    const uint32_t budget = 200u * 1024u;
    if (wRegion + 2u * stageBytes > budget) return FR_ERR_UNSUPPORTED;
    U.ringStages = static_cast<int>(std::min<uint32_t>(kMaxStages, (budget - wRegion) / stageBytes));
    U.wRegion = wRegion, U.stageBytes = stageBytes, U.tmemCols = tmemCols;
    U.sync = n->unetSync;
    U.status = n->status;
    U.waitNs = n->barrierWaitNs;
    U.absentCta = n->absentCta;
    const uint32_t smem = wRegion + static_cast<uint32_t>(U.ringStages) * stageBytes;
    if (unet_fwd_ctas_per_sm(smem) < 1) return FR_ERR_UNSUPPORTED;
    NET_CUDA(n, cudaMemsetAsync(n->unetSync, 0, 4 * sizeof(unsigned), st));
    NET_CUDA(n, launch_unet_fwd(U, n->numSMs, smem, st));
    n->launches += 1;
    return FR_OK;
}

int backward_impl(fr_aonet* n, const uint16_t* in, const float* label, const Shape& S, cudaStream_t st)
{
    const long long pix = static_cast<long long>(S.B) * S.H * S.W;
    NET_TRY(ensure_bwd(n, pix));
    auto DG = [&](int L, const uint16_t* dy, uint16_t* out0, int co0, uint16_t* out1, const uint16_t* mask) {
        const LayerSpec& s = kLayers[L];
        // backward data: input channels = the layer's cout, output channels = its cin
        return conv(n, S, s.level, dy, s.cout, nullptr, 0, s.c0 + s.c1, n->packBwd[L],
                    9u * (s.c0 + s.c1) * s.cout * 2u, nullptr, true, out0, co0, out1, mask, nullptr, nullptr, st);
    };
    const float invN = 1.f / static_cast<float>(pix * kHeadOut);  // full-resolution pixels
    const int hb = blocks_for(pix, kHeadThreads);
    k_head_bwd<<<hb, kHeadThreads, 0, st>>>(n->aoTmp, label, reinterpret_cast<const uint4*>(n->a7),
                                            n->params + n->paramOff[kNumLayers], reinterpret_cast<uint4*>(n->g7),
                                            n->headPart, S.B, S.H, S.W, invN);
    k_head_reduce<<<kHeadSums, kHeadReduceThreads, 0, st>>>(n->headPart, hb, n->grads + n->paramOff[kNumLayers],
                                                           n->lossDev, invN);
    n->launches += 2;
    // level 0 decoder
    NET_TRY(wgrad(n, S, 9, n->a6, nullptr, n->g7, st));
    NET_TRY(DG(9, n->g7, n->g6, 16, nullptr, n->a6));
    NET_TRY(wgrad(n, S, 8, n->u0, n->s0, n->g6, st));
    NET_TRY(DG(8, n->g6, n->gu0, 32, n->gs0c, nullptr));
    k_up_bwd_mask<<<blocks_for((long long)S.B * 4 * S.h(1) * S.w(1), 256), 256, 0, st>>>(
        reinterpret_cast<const uint4*>(n->gu0), reinterpret_cast<const uint4*>(n->a5), reinterpret_cast<uint4*>(n->g5),
        S.B * 4, S.h(1), S.w(1));
    // level 1 decoder
    NET_TRY(wgrad(n, S, 7, n->a4, nullptr, n->g5, st));
    NET_TRY(DG(7, n->g5, n->g4, 32, nullptr, n->a4));
    NET_TRY(wgrad(n, S, 6, n->u1, n->s1, n->g4, st));
    NET_TRY(DG(6, n->g4, n->gu1, 64, n->gs1c, nullptr));
    k_up_bwd_mask<<<blocks_for((long long)S.B * 8 * S.h(2) * S.w(2), 256), 256, 0, st>>>(
        reinterpret_cast<const uint4*>(n->gu1), reinterpret_cast<const uint4*>(n->a3), reinterpret_cast<uint4*>(n->g3),
        S.B * 8, S.h(2), S.w(2));
    // bottleneck
    NET_TRY(wgrad(n, S, 5, n->a2, nullptr, n->g3, st));
    NET_TRY(DG(5, n->g3, n->g2, 64, nullptr, n->a2));
    NET_TRY(wgrad(n, S, 4, n->p1, nullptr, n->g2, st));
    NET_TRY(DG(4, n->g2, n->gp1, 32, nullptr, nullptr));
    k_pool_bwd_add_mask<<<blocks_for((long long)S.B * 4 * S.h(1) * S.w(1), 256), 256, 0, st>>>(
        reinterpret_cast<const uint4*>(n->gs1c), reinterpret_cast<const uint4*>(n->gp1),
        reinterpret_cast<const uint4*>(n->s1), reinterpret_cast<uint4*>(n->gS1), S.B * 4, S.h(1), S.w(1));
    // level 1 encoder
    NET_TRY(wgrad(n, S, 3, n->a1, nullptr, n->gS1, st));
    NET_TRY(DG(3, n->gS1, n->g1, 32, nullptr, n->a1));
    NET_TRY(wgrad(n, S, 2, n->p0, nullptr, n->g1, st));
    NET_TRY(DG(2, n->g1, n->gp0, 16, nullptr, nullptr));
    k_pool_bwd_add_mask<<<blocks_for((long long)S.B * 2 * S.H * S.W, 256), 256, 0, st>>>(
        reinterpret_cast<const uint4*>(n->gs0c), reinterpret_cast<const uint4*>(n->gp0),
        reinterpret_cast<const uint4*>(n->s0), reinterpret_cast<uint4*>(n->gS0), S.B * 2, S.H, S.W);
    // level 0 encoder
    NET_TRY(wgrad(n, S, 1, n->a0, nullptr, n->gS0, st));
    NET_TRY(DG(1, n->gS0, n->g0, 16, nullptr, n->a0));
    NET_TRY(wgrad(n, S, 0, n->xs, nullptr, n->g0, st));
    n->launches += 3;
    NET_CUDA(n, cudaGetLastError());
    return FR_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------

extern "C" {

int64_t fr_aonet_num_params(void) { return kNumParams; }

int fr_aonet_set_fused(fr_aonet* net, int32_t fused)
{
    if (!net) return FR_ERR_INVALID;
    net->fused = fused != 0;
    return FR_OK;
}

int fr_aonet_get_state(fr_aonet* n, float* params, float* m, float* v, int64_t count, int64_t* step)
{
    if (!n || count != kNumParams) return net_fail(n, FR_ERR_INVALID, "get_state: bad arguments");
    DeviceGuard g(n->device);
    const size_t bytes = sizeof(float) * kNumParams;
    if (params) NET_CUDA(n, cudaMemcpy(params, n->params, bytes, cudaMemcpyDeviceToHost));
    if (m) NET_CUDA(n, cudaMemcpy(m, n->adamM, bytes, cudaMemcpyDeviceToHost));
    if (v) NET_CUDA(n, cudaMemcpy(v, n->adamV, bytes, cudaMemcpyDeviceToHost));
    if (step) *step = n->adamT;
    return FR_OK;
}

int fr_aonet_set_state(fr_aonet* n, const float* params, const float* m, const float* v, int64_t count,
                       int64_t step)
{
    if (!n || !params || !m || !v || count != kNumParams || step < 0)
        return net_fail(n, FR_ERR_INVALID, "set_state: bad arguments");
    NET_TRY(fr_aonet_set_params(n, params, count));  // the packed BF16 copies too
    DeviceGuard g(n->device);
    const size_t bytes = sizeof(float) * kNumParams;
    NET_CUDA(n, cudaMemcpy(n->adamM, m, bytes, cudaMemcpyHostToDevice));
    NET_CUDA(n, cudaMemcpy(n->adamV, v, bytes, cudaMemcpyHostToDevice));
    n->adamT = step;
    return FR_OK;
}

int fr_aonet_set_wait_limit(fr_aonet* net, uint64_t ns)
{
    if (!net) return FR_ERR_INVALID;
    net->barrierWaitNs = ns ? ns : 2000000000ull;
    return FR_OK;
}

int fr_aonet_test_absent_cta(fr_aonet* net, int32_t cta)
{
    if (!net || cta < -1) return FR_ERR_INVALID;
    net->absentCta = cta;
    return FR_OK;
}

fr_aonet* fr_aonet_create(int32_t device, uint64_t seed, char* err, size_t errlen)
{
    auto report = [&](const std::string& m) {
        if (err && errlen) std::snprintf(err, errlen, "%s", m.c_str());
    };
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    {
        report("no such CUDA device");
        return nullptr;
    }
    DeviceGuard g(device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major < 10)
    {
        report("fr_aonet needs a tcgen05 GPU (compute capability 10.x)");
        return nullptr;
    }
    fr_aonet* n = new fr_aonet();
    n->device = device;
    n->numSMs = prop.multiProcessorCount;
    int off = 0;
    for (int L = 0; L < kNumLayers; ++L)
    {
        n->paramOff[L] = off;
        off += w_count(L) + kLayers[L].cout;
    }
    n->paramOff[kNumLayers] = off;
    off += kHeadParams;
    if (off != kNumParams)
    {
        report("parameter count mismatch");
        delete n;
        return nullptr;
    }
    // He-normal weights, zero biases; head weights N(0, 1/16), head biases 1.
    std::vector<float> h(kNumParams, 0.f);
    uint64_t s = seed;
    for (int L = 0; L < kNumLayers; ++L)
    {
        const double sd = std::sqrt(2.0 / (kLayers[L].cinReal * 9.0));
        for (int i = 0; i < w_count(L); ++i) h[n->paramOff[L] + i] = static_cast<float>(gaussian(s) * sd);
    }
    for (int i = 0; i < kHeadOut * 16; ++i) h[n->paramOff[kNumLayers] + i] = static_cast<float>(gaussian(s) * 0.25);
    for (int k = 0; k < kHeadOut; ++k) h[n->paramOff[kNumLayers] + kHeadOut * 16 + k] = 1.f;
    bool ok = cudaMalloc(&n->params, sizeof(float) * kNumParams) == cudaSuccess &&
              cudaMalloc(&n->grads, sizeof(float) * kNumParams) == cudaSuccess &&
              cudaMalloc(&n->adamM, sizeof(float) * kNumParams) == cudaSuccess &&
              cudaMalloc(&n->adamV, sizeof(float) * kNumParams) == cudaSuccess &&
              cudaMalloc(&n->status, sizeof(int)) == cudaSuccess &&
              cudaMalloc(&n->unetSync, 4 * sizeof(unsigned)) == cudaSuccess &&
              cudaMalloc(&n->lossDev, sizeof(float)) == cudaSuccess;
    for (int L = 0; ok && L < kNumLayers; ++L)
    {
        const LayerSpec& sp = kLayers[L];
        const int cin = sp.c0 + sp.c1;
        n->packFwdBytes[L] = cin == 8 ? 5u * 2u * 8u * sp.cout * 2u : 9u * cin * sp.cout * 2u;
        ok = cudaMalloc(&n->packFwd[L], n->packFwdBytes[L]) == cudaSuccess;
        if (ok && L > 0) ok = cudaMalloc(&n->packBwd[L], 9u * cin * sp.cout * 2u) == cudaSuccess;
    }
    // wgrad partials: the largest layer's gridY * SMs * taps * (cin + 1) * cout
    size_t cap = 0;
    for (int L = 0; L < kNumLayers; ++L)
    {
        const LayerSpec& sp = kLayers[L];
        const int tpg = sp.cout == 64 ? 5 : 9;
        const int gy = (9 + tpg - 1) / tpg;
        cap = std::max(cap, static_cast<size_t>(gy) * n->numSMs * tpg * (sp.c0 + sp.c1 + 1) * sp.cout);
    }
    if (ok) ok = cudaMalloc(&n->partial, sizeof(float) * cap) == cudaSuccess;
    n->partialCap = cap;
    if (ok)
        ok = cudaMemcpy(n->params, h.data(), sizeof(float) * kNumParams, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(n->grads, 0, sizeof(float) * kNumParams) == cudaSuccess &&
             cudaMemset(n->adamM, 0, sizeof(float) * kNumParams) == cudaSuccess &&
             cudaMemset(n->adamV, 0, sizeof(float) * kNumParams) == cudaSuccess &&
             cudaMemset(n->status, 0, sizeof(int)) == cudaSuccess;
    if (ok) ok = pack_all(n, nullptr) == FR_OK && cudaDeviceSynchronize() == cudaSuccess;
    if (!ok)
    {
        report("device allocation or setup failed");
        fr_aonet_destroy(n);
        return nullptr;
    }
    return n;
}

void fr_aonet_destroy(fr_aonet* n)
{
    if (!n) return;
    DeviceGuard g(n->device);
    for (auto& b : n->fwdBufs) cudaFree(b.p);
    for (auto& b : n->bwdBufs) cudaFree(b.p);
    for (int L = 0; L < kNumLayers; ++L)
    {
        cudaFree(n->packFwd[L]);
        cudaFree(n->packBwd[L]);
    }
    cudaFree(n->params);
    cudaFree(n->grads);
    cudaFree(n->adamM);
    cudaFree(n->adamV);
    cudaFree(n->status);
    cudaFree(n->unetSync);
    cudaFree(n->lossDev);
    cudaFree(n->headPart);
    cudaFree(n->partial);
    delete n;
}

const char* fr_aonet_last_error(const fr_aonet* n) { return n ? n->err.c_str() : "null network"; }

int fr_aonet_get_params(fr_aonet* n, float* dst, int64_t count)
{
    if (!n || !dst || count != kNumParams) return net_fail(n, FR_ERR_INVALID, "get_params: bad arguments");
    DeviceGuard g(n->device);
    NET_CUDA(n, cudaDeviceSynchronize());
    NET_CUDA(n, cudaMemcpy(dst, n->params, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
    return FR_OK;
}

int fr_aonet_set_params(fr_aonet* n, const float* src, int64_t count)
{
    if (!n || !src || count != kNumParams) return net_fail(n, FR_ERR_INVALID, "set_params: bad arguments");
    DeviceGuard g(n->device);
    NET_CUDA(n, cudaDeviceSynchronize());
    NET_CUDA(n, cudaMemcpy(n->params, src, sizeof(float) * kNumParams, cudaMemcpyHostToDevice));
    NET_CUDA(n, cudaMemset(n->adamM, 0, sizeof(float) * kNumParams));
    NET_CUDA(n, cudaMemset(n->adamV, 0, sizeof(float) * kNumParams));
    n->adamT = 0;
    NET_TRY(pack_all(n, nullptr));
    NET_CUDA(n, cudaDeviceSynchronize());
    return FR_OK;
}

int fr_aonet_get_grads(fr_aonet* n, float* dst, int64_t count)
{
    if (!n || !dst || count != kNumParams) return net_fail(n, FR_ERR_INVALID, "get_grads: bad arguments");
    DeviceGuard g(n->device);
    NET_CUDA(n, cudaDeviceSynchronize());
    NET_CUDA(n, cudaMemcpy(dst, n->grads, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
    return FR_OK;
}

int fr_aonet_forward(fr_aonet* n, const uint16_t* in, int32_t B, int32_t H, int32_t W, float* ao, void* stream)
{
    if (!n || !in || !ao) return net_fail(n, FR_ERR_INVALID, "forward: null argument");
    NET_TRY(check_shape(n, B, H, W));
    DeviceGuard g(n->device);
    n->launches = 0;
    return forward_impl(n, in, Shape{B, H / kBlock, W / kBlock}, ao, reinterpret_cast<cudaStream_t>(stream));
}

int fr_aonet_backward(fr_aonet* n, const uint16_t* in, const float* label, int32_t B, int32_t H, int32_t W,
                      float* loss, void* stream)
{
    if (!n || !in || !label) return net_fail(n, FR_ERR_INVALID, "backward: null argument");
    NET_TRY(check_shape(n, B, H, W));
    DeviceGuard g(n->device);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    n->launches = 0;
    const Shape S{B, H / kBlock, W / kBlock};
    NET_TRY(ensure_fwd(n, static_cast<long long>(S.B) * S.H * S.W));
    NET_TRY(forward_impl(n, in, S, n->aoTmp, st));
    NET_TRY(backward_impl(n, in, label, S, st));
    if (loss)
    {
        NET_CUDA(n, cudaMemcpyAsync(loss, n->lossDev, sizeof(float), cudaMemcpyDeviceToHost, st));
        NET_TRY(fr_aonet_check(n, stream));
    }
    return FR_OK;
}

int fr_aonet_adam_step(fr_aonet* n, float lr, float beta1, float beta2, float eps, void* stream)
{
    if (!n) return FR_ERR_INVALID;
    DeviceGuard g(n->device);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    n->adamT++;
    const double bc1 = 1.0 - std::pow(static_cast<double>(beta1), static_cast<double>(n->adamT));
    const double bc2 = 1.0 - std::pow(static_cast<double>(beta2), static_cast<double>(n->adamT));
    k_adam<<<blocks_for(kNumParams, 256), 256, 0, st>>>(n->params, n->grads, n->adamM, n->adamV, kNumParams, beta1,
                                                        beta2, eps, static_cast<float>(lr / bc1),
                                                        static_cast<float>(std::sqrt(bc2)));
    n->launches++;
    NET_TRY(pack_all(n, st));
    n->launches += kNumLayers;
    NET_CUDA(n, cudaGetLastError());
    return FR_OK;
}

int fr_aonet_train_step(fr_aonet* n, const uint16_t* in, const float* label, int32_t B, int32_t H, int32_t W,
                        float lr, float* loss, void* stream)
{
    NET_TRY(fr_aonet_backward(n, in, label, B, H, W, nullptr, stream));
    NET_TRY(fr_aonet_adam_step(n, lr, 0.9f, 0.999f, 1e-8f, stream));
    if (loss)
    {
        DeviceGuard g(n->device);
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        NET_CUDA(n, cudaMemcpyAsync(loss, n->lossDev, sizeof(float), cudaMemcpyDeviceToHost, st));
        NET_TRY(fr_aonet_check(n, stream));
    }
    return FR_OK;
}

int fr_aonet_check(fr_aonet* n, void* stream)
{
    if (!n) return FR_ERR_INVALID;
    DeviceGuard g(n->device);
    NET_CUDA(n, cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
    int st = 0;
    NET_CUDA(n, cudaMemcpy(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st)
    {
        cudaMemset(n->status, 0, sizeof(int));
        return net_fail(n, FR_ERR_TIMEOUT, (st & 4) ? "a grid barrier of the fused forward timed out"
                                                    : "a tensor-core pipeline wait timed out");
    }
    return FR_OK;
}


int32_t fr_aonet_last_launch_count(const fr_aonet* n) { return n ? n->launches : 0; }

}  // extern "C"

// The network's status word, read and cleared (the renderer's synchronising calls).
int fra_take_status(fr_aonet* n)
{
    if (!n) return 0;
    DeviceGuard g(n->device);
    int st = 0;
    if (cudaMemcpy(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    if (st) cudaMemset(n->status, 0, sizeof(int));
    return st;
}

// Used by the renderer (fr_context.cu): network forward on a context stream.
int fra_forward(fr_aonet* n, const uint16_t* in, int B, int H, int W, float* ao, cudaStream_t st, int* launches)
{
    n->launches = 0;
    int rc = forward_impl(n, in, Shape{B, H / kBlock, W / kBlock}, ao, st);
    if (launches) *launches += n->launches;
    return rc;
}

int fra_forward_blocks(fr_aonet* n, const uint16_t* in_blocks, int B, int H, int W, float* ao, cudaStream_t st,
                       int* launches, const float* bgDepth, const float* bg16, bool allowFused)
{
    n->launches = 0;
    n->bgDepth = B == 1 ? bgDepth : nullptr;
    n->bg16 = B == 1 ? bg16 : nullptr;
    const Shape S{B, H / kBlock, W / kBlock};
    int rc = FR_ERR_UNSUPPORTED;
    if (allowFused && n->fused && B == 1) rc = forward_fused(n, in_blocks, S, ao, st);
    if (rc == FR_ERR_UNSUPPORTED) rc = forward_impl(n, in_blocks, S, ao, st, true);
    n->bgDepth = n->bg16 = nullptr;
    if (launches) *launches += n->launches;
    return rc;
}

int fra_reserve(fr_aonet* n, int B, int H, int W)
{
    DeviceGuard g(n->device);
    return ensure_fwd(n, static_cast<long long>(B) * (H / kBlock) * (W / kBlock));
}

int fra_device(const fr_aonet* n) { return n->device; }
