// TGA output on the GPU (include/fr_output.h): the reference's image
// conversions (Buffer1f/Buffer3f::GenerateImage, src/buffer.cpp:20-32, 113-126)
// fused into a parallel restatement of its TGA writer (TGAImage::WriteTgaFile,
// src/tgaimage.cpp:172-248, RLE packets of unloadRleData, :250-300).
//
// The RLE packer is a greedy left-to-right parse: at a packet start s the packet
// is a run if pixel s equals pixel s + 1 (it takes the following equal pixels,
// at most 128), else a raw packet that stops before a pixel equal to its
// successor, except that its 128th pixel is taken without that test. So the
// packet at s depends only on pixels s .. s + 128, but which positions start a
// packet depends on every packet before. The encoder splits each image into
// segments of kSeg pixels; the images of a batch (a frame's output files) share
// three launches:
//   1. k_tga_parse (CTA per segment): equality bits of neighbouring pixels, the
//      packet length L(s) at every position, by pointer doubling over
//      next(s) = s + L(s) inside each 128-pixel sub-block the sub-block maps,
//      and composed over the sub-blocks the segment's transfer function: for
//      each of the 128 possible offsets of its first packet start, the offset of
//      the first packet start in the next segment and the file bytes of the
//      packets on the way.
//   2. k_tga_compose (CTA per group of segments, at most 64 groups per image):
//      composes the group's transfer functions, keeping for each segment the
//      map from the group's entry offset to its own and the bytes on the way;
//      the image's last CTA chains the group functions from offset 0 and hands
//      every segment its entry offset and file offset.
//   3. k_tga_write (CTA per segment): the packet starts of the segment (its entry
//      carried through the sub-block maps of step 1, then one lane per 128-pixel
//      sub-block walks its packets), then the bytes of those packets (a packet
//      start also its header byte), placed by one block scan, staged in shared
//      memory and stored in 16-byte pieces.
// Raw (non-RLE) files are one launch, k_tga_plain.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "fr_context_internal.h"
#include "fr_device.cuh"
#include "fr_output.h"
#include "forkerrenderer.h"

using namespace frd;

namespace fro
{

constexpr int kSeg = 4096;              // pixels per segment
constexpr int kSegWords = kSeg / 32;
constexpr int kWinWords = kSeg / 32 + 4;  // + the 128-pixel look-ahead of a packet
constexpr int kParseThreads = 512;
constexpr int kParseWarps = kParseThreads / 32;
constexpr int kWalkThreads = 256;
constexpr int kWriteThreads = 256;
constexpr int kHeaderBytes = 18;
constexpr int kTailBytes = 26;          // two 4-byte area references + 18-byte footer

enum SrcKind : int
{
    kSrcBytes = 0,  // bytes in TGA order, bpp per pixel
    kSrcRgbx = 1,   // 32-bit R | G << 8 | B << 16 (the 8-bit frame and SSAA images)
    kSrcF1 = 2,     // float: Buffer1f::GenerateImage
    kSrcF3 = 3,     // float3: Buffer3f::GenerateImage
    kSrcGVec = 4,   // float4 plane of the packed G-buffer (normal or world position), as a Buffer3f
    kSrcGMat = 5,   // material field of the packed G-buffer (albedo, param: Buffer3f; shading type: Buffer1f)
    kSrcGMatLinear = 6  // the same of a bilinear-filtered frame (the G-buffer holds texture coordinates)
};

struct PixelSrc
{
    int kind, bpp, which;  // which (kSrcGMat): 3 albedo, 5 param, 6 shading type
    const void* p;
    GBuffer gb;
    DevScene S;
};

// The reference's implicit float -> std::uint8_t as its x86-64 build runs it:
// truncate to int32 (NaN / out of range: INT32_MIN), keep the low byte.
__device__ __forceinline__ uint32_t ref_u8(float v)
{
    if (!(v >= -2147483648.f && v < 2147483648.f)) return 0u;
    return (uint32_t)__float2int_rz(v) & 0xffu;
}

__device__ __forceinline__ uint32_t bgr3(F3 c)
{
    return ref_u8(c.z * 254.99f) | (ref_u8(c.y * 254.99f) << 8) | (ref_u8(c.x * 254.99f) << 16);
}

// Pixel i's bytes in TGA order, packed little-endian into 32 bits. The kind is
// a template argument so unrolled loops keep all their loads in flight.
template <int K>
__device__ __forceinline__ uint32_t pix(const PixelSrc& s, long long i)
{
    if constexpr (K == kSrcBytes)
    {
        const uint8_t* p = static_cast<const uint8_t*>(s.p) + i * s.bpp;
        uint32_t v = p[0];
        if (s.bpp >= 3) v |= ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16);
        if (s.bpp == 4) v |= (uint32_t)p[3] << 24;
        return v;
    }
    else if constexpr (K == kSrcRgbx)
    {
        const uint32_t c = static_cast<const uint32_t*>(s.p)[i];
        return ((c >> 16) & 0xffu) | (c & 0xff00u) | ((c & 0xffu) << 16);
    }
    else if constexpr (K == kSrcF1)
        return ref_u8(static_cast<const float*>(s.p)[i] * 255);
    else if constexpr (K == kSrcF3)
    {
        const float* f = static_cast<const float*>(s.p) + 3 * i;
        return bgr3(F3{f[0], f[1], f[2]});
    }
    else if constexpr (K == kSrcGVec)
    {
        const float4 v = static_cast<const float4*>(s.p)[i];
        return bgr3(F3{v.x, v.y, v.z});
    }
    else
    {
        const GDecoded g = decode_gbuffer_t<K == kSrcGMatLinear>(s.S, s.gb.c[i]);
        if (s.which == 6) return ref_u8(g.type * 255);
        return bgr3(s.which == 3 ? g.albedo : g.param);
    }
}

// Calls BODY<K>(args...) for the source kind k (uniform across a CTA). LIN: the
// kernel is instantiated for bilinear G-buffers (a compile-time flag), so the
// nearest-filtered instantiations carry none of the texture sampling code.
#define FRO_BY_KIND(LIN, k, BODY, ...)                                      \
    switch (k)                                                              \
    {                                                                       \
        case kSrcBytes: BODY<kSrcBytes>(__VA_ARGS__); break;                \
        case kSrcRgbx: BODY<kSrcRgbx>(__VA_ARGS__); break;                  \
        case kSrcF1: BODY<kSrcF1>(__VA_ARGS__); break;                      \
        case kSrcF3: BODY<kSrcF3>(__VA_ARGS__); break;                      \
        case kSrcGVec: BODY<kSrcGVec>(__VA_ARGS__); break;                  \
        default: BODY<(LIN) ? kSrcGMatLinear : kSrcGMat>(__VA_ARGS__); break; \
    }

// First position in [lo, hi] whose bit in w equals `set`, or hi + 1.
__device__ __forceinline__ int first_bit(const uint32_t* w, int lo, int hi, bool set)
{
    for (int wi = lo >> 5; wi <= (hi >> 5); ++wi)
    {
        uint32_t v = set ? w[wi] : ~w[wi];
        if (wi == (lo >> 5)) v &= ~0u << (lo & 31);
        if (v)
        {
            const int p = wi * 32 + __ffs(v) - 1;
            return p <= hi ? p : hi + 1;
        }
    }
    return hi + 1;
}

__device__ void put_header(uint8_t* o, int w, int h, int bpp, int rle, int vflip)
{
    for (int i = 0; i < kHeaderBytes; ++i) o[i] = 0;
    o[2] = (uint8_t)(bpp == 1 ? (rle ? 11 : 3) : (rle ? 10 : 2));
    o[12] = (uint8_t)(w & 0xff), o[13] = (uint8_t)((w >> 8) & 0xff);
    o[14] = (uint8_t)(h & 0xff), o[15] = (uint8_t)((h >> 8) & 0xff);
    o[16] = (uint8_t)(bpp * 8);
    o[17] = vflip ? 0x00 : 0x20;
}

__device__ void put_tail(uint8_t* o)
{
    const char footer[18] = {'T', 'R', 'U', 'E', 'V', 'I', 'S', 'I', 'O', 'N', '-', 'X', 'F', 'I', 'L', 'E', '.', '\0'};
    for (int i = 0; i < 8; ++i) o[i] = 0;
    for (int i = 0; i < 18; ++i) o[8 + i] = (uint8_t)footer[i];
}

// ---- batched encoder: one launch per stage for every image of a batch --------

constexpr int kMaxJobs = 10;
constexpr int kSubBlocks = kSeg / 128;   // 128-pixel sub-blocks of a segment
constexpr int kComposeThreads = 256;
constexpr int kMaxGroups = 64;    // groups of segments per image
constexpr int kComposeChunk = 64; // segments a compose CTA stages at a time

// One image of a batch, with its slices of the scratch buffer.
struct Job
{
    PixelSrc src;
    long long n;
    int w, h, bpp, rle, vflip;
    int S;              // segments
    int segBase;        // first CTA of this image in the per-segment launches
    int gsz, G;         // segments per group, groups (G <= kMaxGroups)
    int groupBase;      // first CTA of this image in k_tga_compose
    uint8_t* out;
    long long cap;      // bytes of out: no write goes past it
    long long* dSize;   // file size, or -1 if it would not fit in cap
    uint8_t* info;      // [n] (packet length - 1) | 0x80 for a run, at every position
    uint8_t* func;      // [S][128] transfer function: entry offset -> next segment's entry offset
    uint16_t* fbytes;   // [S][128] file bytes of the segment's packets for each entry offset
    uint8_t* sub;       // [S][kSeg] per position: the next sub-block's entry offset from it
    uint8_t* pre;       // [S][128] entry offset of segment k for each entry offset of its group
    uint32_t* preB;     // [S][128] file bytes from the group's first packet to segment k's
    uint8_t* gfun;      // [kMaxGroups][128] group transfer functions
    uint32_t* gbytes;   // [kMaxGroups][128] and their byte counts
    unsigned* counter;  // compose CTAs of this image that finished (zeroed before each batch)
    uint8_t* ent;       // [S] offset of each segment's first packet start
    long long* segOff;  // [S] file offset of each segment's first packet, after the header
};

struct Jobs
{
    int count;
    Job j[kMaxJobs];
};

__device__ __forceinline__ int job_of(const Jobs& J, int blk)
{
    int ji = 0;
    while (ji + 1 < J.count && blk >= J.j[ji + 1].segBase) ++ji;
    return ji;
}

__device__ __forceinline__ int job_of_group(const Jobs& J, int blk)
{
    int ji = 0;
    while (ji + 1 < J.count && blk >= J.j[ji + 1].groupBase) ++ji;
    return ji;
}

// Bit r of eqw: pixel seg0 + r equals its successor (r < kWinWords * 32). Warp w
// handles words w * kPer .. w * kPer + kPer - 1, every load issued before the
// first comparison; a word's last pixel finds its successor in the next word.
template <int K>
__device__ __forceinline__ void equality_bits(const Job& jb, long long seg0, uint32_t* eqw)
{
    constexpr int kPer = (kWinWords + kParseWarps - 1) / kParseWarps;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int w0 = warp * kPer;
    uint32_t av[kPer + 1];
#pragma unroll
    for (int i = 0; i <= kPer; ++i)
    {
        const long long g = seg0 + (long long)(w0 + i) * 32 + lane;
        av[i] = (i < kPer || lane == 0) && w0 + i <= kWinWords && g < jb.n ? pix<K>(jb.src, g) : 0u;
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i)
    {
        const long long g = seg0 + (long long)(w0 + i) * 32 + lane;
        uint32_t b = __shfl_down_sync(0xffffffffu, av[i], 1);
        const uint32_t next = __shfl_sync(0xffffffffu, av[i + 1], 0);
        if (lane == 31) b = next;
        const unsigned m = __ballot_sync(0xffffffffu, g + 1 < jb.n && av[i] == b);
        if (lane == 0 && w0 + i < kWinWords) eqw[w0 + i] = m;
    }
}

// Per segment: info bytes; by pointer doubling over next(s) = s + L(s) inside
// each 128-pixel sub-block (carrying the packets' file bytes) the sub-block transfer
// functions, stored for k_tga_write; composed over the 32 sub-blocks, the
// segment's transfer function and its byte counts.
template <bool kLin>
__global__ void __launch_bounds__(kParseThreads, 4) k_tga_parse(const __grid_constant__ Jobs J)
{
    __shared__ uint32_t eqw[kWinWords];
    __shared__ uint16_t Jp[kSeg];
    __shared__ uint16_t Wp[kSeg];  // bytes along a sub-block path: at most 255 pixels * 5
    const Job& jb = J.j[job_of(J, blockIdx.x)];
    const int k = blockIdx.x - jb.segBase, bpp = jb.bpp;
    const long long n = jb.n, seg0 = (long long)k * kSeg;
    FRO_BY_KIND(kLin, jb.src.kind, equality_bits, jb, seg0, eqw)
    __syncthreads();
    const int segLen = (int)min((long long)kSeg, n - seg0);
    for (int r = threadIdx.x; r < kSeg; r += kParseThreads)
    {
        if (r >= segLen)
        {
            Jp[r] = (uint16_t)((r | 127) + 1);  // past the image: terminal
            Wp[r] = 0;
            continue;
        }
        const bool run = (eqw[r >> 5] >> (r & 31)) & 1u;
        int L;
        if (run)
            L = min(128, first_bit(eqw, r, r + 127, false) - r + 1);  // r and the equal pixels after it
        else
        {
            const int j = first_bit(eqw, r + 1, r + 126, true);  // first later pixel equal to its successor
            L = j <= r + 126 ? j - r : (int)min(128ll, n - (seg0 + r));
        }
        jb.info[seg0 + r] = (uint8_t)((L - 1) | (run ? 0x80 : 0));
        Jp[r] = (uint16_t)(r + L);
        Wp[r] = (uint16_t)(run ? 1 + bpp : 1 + L * bpp);
    }
    __syncthreads();
    // pointer doubling inside each 128-pixel sub-block: 2^7 steps cover its path
    for (int round = 0; round < 7; ++round)
    {
        uint16_t ny[kSeg / kParseThreads], nw[kSeg / kParseThreads];
#pragma unroll
        for (int i = 0; i < kSeg / kParseThreads; ++i)
        {
            const int r = threadIdx.x + i * kParseThreads;
            const int x = Jp[r];
            ny[i] = (uint16_t)x, nw[i] = Wp[r];
            if (x <= (r | 127)) ny[i] = Jp[x], nw[i] = (uint16_t)(nw[i] + Wp[x]);
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kSeg / kParseThreads; ++i)
        {
            const int r = threadIdx.x + i * kParseThreads;
            Jp[r] = ny[i], Wp[r] = nw[i];
        }
        __syncthreads();
    }
    // sub-block functions: offset of the first packet start in the next sub-block
    for (int r = threadIdx.x; r < kSeg; r += kParseThreads)
        jb.sub[(size_t)k * kSeg + r] = (uint8_t)((Jp[r] - ((r | 127) + 1)) & 127);
    if (threadIdx.x < 128)
    {
        int x = threadIdx.x, bytes = 0;
        for (int sb = 0; sb < kSubBlocks; ++sb)
        {
            const int pos = 128 * sb + x;
            bytes += Wp[pos];
            x = (Jp[pos] - 128 * (sb + 1)) & 127;
        }
        jb.func[(size_t)k * 128 + threadIdx.x] = (uint8_t)x;
        jb.fbytes[(size_t)k * 128 + threadIdx.x] = (uint16_t)bytes;
    }
}

// CTA per group of gsz segments: composes the group's transfer function (and
// byte counts) segment by segment, keeping for every segment the map from the
// group's entry offset to its own (pre, preB). The last CTA of an image to
// finish chains its <= kMaxGroups group functions from offset 0 and gives every
// segment its entry offset and file offset; it writes header, footer and size.
__global__ void __launch_bounds__(kComposeThreads) k_tga_compose(const __grid_constant__ Jobs J)
{
    __shared__ __align__(16) uint8_t buf[kMaxGroups * 128 * 5];  // staged maps, then group maps
    __shared__ uint8_t xg[kMaxGroups];
    __shared__ long long go[kMaxGroups];
    __shared__ long long body;
    __shared__ bool last;
    const Job& jb = J.j[job_of_group(J, blockIdx.x)];
    const int g = blockIdx.x - jb.groupBase, tid = threadIdx.x;
    const int k0 = g * jb.gsz, k1 = min(jb.S, k0 + jb.gsz);
    uint8_t(*fs)[128] = reinterpret_cast<uint8_t(*)[128]>(buf);
    uint16_t(*fb)[128] = reinterpret_cast<uint16_t(*)[128]>(buf + kComposeChunk * 128);
    int x = tid & 127;
    uint32_t pb = 0;
    for (int c0 = k0; c0 < k1; c0 += kComposeChunk)
    {
        const int c1 = min(k1, c0 + kComposeChunk);
        for (int i = tid; i < (c1 - c0) * 128; i += kComposeThreads)
        {
            fs[i >> 7][i & 127] = jb.func[(size_t)c0 * 128 + i];
            fb[i >> 7][i & 127] = jb.fbytes[(size_t)c0 * 128 + i];
        }
        __syncthreads();
        if (tid < 128)
            for (int k = c0; k < c1; ++k)
            {
                jb.pre[(size_t)k * 128 + tid] = (uint8_t)x;
                jb.preB[(size_t)k * 128 + tid] = pb;
                pb += fb[k - c0][x];
                x = fs[k - c0][x] & 127;
            }
        __syncthreads();
    }
    if (tid < 128)
    {
        jb.gfun[g * 128 + tid] = (uint8_t)x;
        jb.gbytes[g * 128 + tid] = pb;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) last = atomicAdd(jb.counter, 1u) == (unsigned)jb.G - 1u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    uint8_t(*gf)[128] = reinterpret_cast<uint8_t(*)[128]>(buf);
    uint32_t(*gb)[128] = reinterpret_cast<uint32_t(*)[128]>(buf + kMaxGroups * 128);
    for (int i = tid; i < jb.G * 128; i += kComposeThreads)
    {
        gf[i >> 7][i & 127] = __ldcg(jb.gfun + i);
        gb[i >> 7][i & 127] = __ldcg(jb.gbytes + i);
    }
    __syncthreads();
    if (tid == 0)
    {
        int e = 0;
        long long off = 0;
        for (int q = 0; q < jb.G; ++q)
        {
            xg[q] = (uint8_t)e;
            go[q] = off;
            off += gb[q][e];
            e = gf[q][e] & 127;
        }
        body = off;
    }
    __syncthreads();
    for (int k = tid; k < jb.S; k += kComposeThreads)
    {
        const int q = k / jb.gsz, e = xg[q];
        jb.ent[k] = (uint8_t)(__ldcg(jb.pre + (size_t)k * 128 + e) & 127);
        jb.segOff[k] = go[q] + (long long)__ldcg(jb.preB + (size_t)k * 128 + e);
    }
    if (tid == 0)
    {
        if (kHeaderBytes + body + kTailBytes > jb.cap)
            *jb.dSize = -1;
        else
        {
            put_header(jb.out, jb.w, jb.h, jb.bpp, jb.rle, jb.vflip);
            put_tail(jb.out + kHeaderBytes + body);
            *jb.dSize = kHeaderBytes + body + kTailBytes;
        }
    }
}

constexpr int kWritePer = (kSeg + 128 + kWriteThreads - 1) / kWriteThreads;  // positions per thread
constexpr int kStageBytes = ((kSeg + 128) * 5 + 16 + 15) & ~15;            // a segment's packets + alignment

// The pixels of the kWritePer consecutive positions a thread owns in [a, bEnd),
// loaded together (issued before the packet walk, so their latency hides behind it).
template <int K>
__device__ __forceinline__ void prefetch_pixels(const Job& jb, long long p0, int per, long long bEnd,
                                                uint32_t (&px)[kWritePer])
{
#pragma unroll
    for (int i = 0; i < kWritePer; ++i)
    {
        const long long r = p0 + i;
        px[i] = i < per && r < bEnd ? pix<K>(jb.src, r) : 0u;
    }
}

// Bytes of the packets starting in the segment into the staging buffer
// (stg[s0 + i] is the file byte at base + i, s0 = base & 15), placed by one
// block scan over the threads' position ranges. Returns the bytes staged.
__device__ __forceinline__ int stage_segment(int bpp, long long seg0, long long p0, int per, long long bEnd, int s0,
                                             const uint32_t (&px)[kWritePer], const uint8_t* inf,
                                             const uint32_t* bits, uint8_t* stg, int* warpSum)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int mine = 0;
#pragma unroll
    for (int i = 0; i < kWritePer; ++i)
    {
        const long long r = p0 + i;
        if (i < per && r < bEnd)
        {
            const int rel = (int)(r - seg0);
            const bool start = rel < kSeg && ((bits[rel >> 5] >> (rel & 31)) & 1u);
            // a later pixel of a packet: raw packets store it, runs do not
            mine += start ? 1 + bpp : ((inf[rel - 1] & 0x80) ? 0 : bpp);
        }
    }
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warpSum[warp] = incl;
    __syncthreads();
    int before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kWriteThreads / 32; ++w)
    {
        before += w < warp ? warpSum[w] : 0;
        all += warpSum[w];
    }
    int o = s0 + before + incl - mine;
#pragma unroll
    for (int i = 0; i < kWritePer; ++i)
    {
        const long long r = p0 + i;
        if (i < per && r < bEnd)
        {
            const int rel = (int)(r - seg0);
            const bool start = rel < kSeg && ((bits[rel >> 5] >> (rel & 31)) & 1u);
            if (start)
            {
                const int v = inf[rel], L = (v & 127) + 1;
                stg[o++] = (uint8_t)((v & 0x80) ? L + 127 : L - 1);
            }
            if (start || !(inf[rel - 1] & 0x80))
                for (int c = 0; c < bpp; ++c) stg[o++] = (uint8_t)(px[i] >> (8 * c));
        }
    }
    return all;
}

// Per segment: its packet starts (the segment's entry through the 32 sub-block
// maps k_tga_parse stored, then one lane per 128-pixel sub-block walks its
// packets), then the packets' bytes, staged in shared memory and copied out in
// 16-byte stores.
template <bool kLin>
__global__ void __launch_bounds__(kWriteThreads, 4) k_tga_write(const __grid_constant__ Jobs J)
{
    __shared__ __align__(16) uint8_t inf[kSeg + 128];
    __shared__ __align__(16) uint8_t work[kStageBytes];  // sub-block maps, then the staged bytes
    __shared__ uint32_t bits[kSegWords];
    __shared__ uint8_t xs[kSubBlocks];
    __shared__ int warpSum[kWriteThreads / 32];
    const Job& jb = J.j[job_of(J, blockIdx.x)];
    const int kk = blockIdx.x - jb.segBase;
    const long long n = jb.n, seg0 = (long long)kk * kSeg;
    const int segLen = (int)min((long long)kSeg, n - seg0);
    const int avail = (int)min((long long)kSeg + 128, n - seg0);
    {
        // info and sub-block map words (scratch slices are 256-byte aligned and padded)
        const uint32_t* si = reinterpret_cast<const uint32_t*>(jb.info + seg0);
        const uint32_t* sm = reinterpret_cast<const uint32_t*>(jb.sub + (size_t)kk * kSeg);
        uint32_t* di = reinterpret_cast<uint32_t*>(inf);
        uint32_t* dm = reinterpret_cast<uint32_t*>(work);
        const int words = (avail + 3) >> 2;
        constexpr int kPer = ((kSeg + 128) / 4 + kWriteThreads - 1) / kWriteThreads;
        constexpr int kPerM = (kSeg / 4) / kWriteThreads;
        uint32_t v[kPer], m[kPerM];
#pragma unroll
        for (int i = 0; i < kPer; ++i)
        {
            const int w = threadIdx.x + i * kWriteThreads;
            v[i] = w < words ? si[w] : 0u;
        }
#pragma unroll
        for (int i = 0; i < kPerM; ++i) m[i] = sm[threadIdx.x + i * kWriteThreads];
#pragma unroll
        for (int i = 0; i < kPer; ++i)
        {
            const int w = threadIdx.x + i * kWriteThreads;
            if (w < words) di[w] = v[i];
        }
#pragma unroll
        for (int i = 0; i < kPerM; ++i) dm[threadIdx.x + i * kWriteThreads] = m[i];
    }
    for (int i = threadIdx.x; i < kSegWords; i += kWriteThreads) bits[i] = 0u;
    const long long a = seg0 + (jb.ent[kk] & 127);
    const long long bEnd = kk + 1 < jb.S ? seg0 + kSeg + (jb.ent[kk + 1] & 127) : n;
    const int per = (int)((bEnd - a + kWriteThreads - 1) / kWriteThreads);
    const long long p0 = a + (long long)threadIdx.x * per;
    uint32_t px[kWritePer];
    FRO_BY_KIND(kLin, jb.src.kind, prefetch_pixels, jb, p0, per, bEnd, px)
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int x = jb.ent[kk] & 127;
        for (int b = 0; b < kSubBlocks; ++b)
        {
            xs[b] = (uint8_t)x;
            x = work[128 * b + x];
        }
    }
    __syncthreads();
    if (threadIdx.x < kSubBlocks)
    {
        const int b = threadIdx.x, end = min(128 * (b + 1), segLen);
        for (int s = 128 * b + xs[b]; s < end; s += (inf[s] & 127) + 1) bits[s >> 5] |= 1u << (s & 31);
    }
    __syncthreads();  // the sub-block maps are done with: the buffer becomes the staging buffer
    const long long base = kHeaderBytes + jb.segOff[kk];
    const int s0 = (int)(base & 15);
    const int total = stage_segment(jb.bpp, seg0, p0, per, bEnd, s0, px, inf, bits, work, warpSum);
    __syncthreads();
    // stg[i] -> out[(base & ~15) + i] for i in [s0, s0 + total); bytes past cap - 26 are dropped
    const long long g0 = base - s0;
    const long long limit = jb.cap - kTailBytes;
    const int end = s0 + total;
    for (int c = threadIdx.x; c * 16 < end; c += kWriteThreads)
    {
        const int lo = c * 16;
        if (lo >= s0 && lo + 16 <= end && g0 + lo + 16 <= limit)
            *reinterpret_cast<uint4*>(jb.out + g0 + lo) = *reinterpret_cast<const uint4*>(work + lo);
        else
            for (int i = max(lo, s0); i < min(lo + 16, end); ++i)
                if (g0 + i < limit) jb.out[g0 + i] = work[i];
    }
}

// Raw files (and empty images): pixel bytes, header and tail.
template <bool kLin>
__global__ void k_tga_plain(const __grid_constant__ Job jb)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long body = jb.rle ? 0 : jb.n * jb.bpp;
    if (i == 0)
    {
        put_header(jb.out, jb.w, jb.h, jb.bpp, jb.rle, jb.vflip);
        put_tail(jb.out + kHeaderBytes + body);
        *jb.dSize = kHeaderBytes + body + kTailBytes;
    }
    if (jb.rle || i >= jb.n) return;
    uint32_t px = 0;
    FRO_BY_KIND(kLin, jb.src.kind, px = pix, jb.src, i)
    uint8_t* o = jb.out + kHeaderBytes + i * jb.bpp;
    for (int c = 0; c < jb.bpp; ++c) o[c] = (uint8_t)(px >> (8 * c));
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int segments(long long n) { return (int)((n + kSeg - 1) / kSeg); }

// Scratch bytes of one image of n pixels (after the batch's counter block).
size_t scratch_bytes(long long n)
{
    const size_t S = (size_t)segments(n);
    return align256((size_t)n) + align256(S * 128) + align256(S * 256) + align256(S * kSeg) + align256(S * 128) +
           align256(S * 512) + align256(kMaxGroups * 128) + align256(kMaxGroups * 512) + align256(S) +
           align256(S * 8);
}

constexpr size_t kCounterBytes = 256;  // one counter per image of a batch, zeroed per batch

struct EncodeJob
{
    PixelSrc src;
    int w, h, rle, vflip;
    uint8_t* out;
    long long* dSize;
};

// Launches the encoder for up to kMaxJobs images (scratch: kCounterBytes plus
// the sum of their scratch_bytes); returns the number of kernels launched.
int encode_batch(const EncodeJob* list, int count, void* scratch, cudaStream_t st)
{
    Jobs J{};
    int seg = 0, groups = 0, launches = 0;
    unsigned* counters = static_cast<unsigned*>(scratch);
    uint8_t* p = static_cast<uint8_t*>(scratch) + kCounterBytes;
    for (int i = 0; i < count && i < kMaxJobs; ++i)
    {
        const EncodeJob& e = list[i];
        Job jb{};
        jb.src = e.src, jb.n = (long long)e.w * e.h, jb.w = e.w, jb.h = e.h, jb.bpp = e.src.bpp;
        jb.rle = e.rle, jb.vflip = e.vflip, jb.out = e.out, jb.dSize = e.dSize;
        jb.cap = (long long)fr_tga_max_bytes(e.w, e.h, e.src.bpp);
        jb.S = segments(jb.n);
        jb.gsz = std::max(1, (jb.S + kMaxGroups - 1) / kMaxGroups);
        jb.G = (jb.S + jb.gsz - 1) / jb.gsz;
        const size_t S = (size_t)jb.S;
        uint8_t* q = p;
        jb.info = q, q += align256((size_t)jb.n);
        jb.func = q, q += align256(S * 128);
        jb.fbytes = reinterpret_cast<uint16_t*>(q), q += align256(S * 256);
        jb.sub = q, q += align256(S * kSeg);
        jb.pre = q, q += align256(S * 128);
        jb.preB = reinterpret_cast<uint32_t*>(q), q += align256(S * 512);
        jb.gfun = q, q += align256(kMaxGroups * 128);
        jb.gbytes = reinterpret_cast<uint32_t*>(q), q += align256(kMaxGroups * 512);
        jb.ent = q, q += align256(S);
        jb.segOff = reinterpret_cast<long long*>(q);
        jb.counter = counters + i;
        p += scratch_bytes(jb.n);
        if (!jb.rle || jb.n == 0)
        {
            const long long threads = jb.n > 0 && !jb.rle ? jb.n : 1;
            if (jb.src.kind == kSrcGMatLinear)
                k_tga_plain<true><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(jb);
            else
                k_tga_plain<false><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(jb);
            ++launches;
            continue;
        }
        jb.segBase = seg, seg += jb.S;
        jb.groupBase = groups, groups += jb.G;
        J.j[J.count++] = jb;
    }
    if (J.count)
    {
        cudaMemsetAsync(counters, 0, kCounterBytes, st);
        bool lin = false;
        for (int i = 0; i < J.count; ++i) lin = lin || J.j[i].src.kind == kSrcGMatLinear;
        if (lin) k_tga_parse<true><<<seg, kParseThreads, 0, st>>>(J);
        else k_tga_parse<false><<<seg, kParseThreads, 0, st>>>(J);
        k_tga_compose<<<groups, kComposeThreads, 0, st>>>(J);
        if (lin) k_tga_write<true><<<seg, kWriteThreads, 0, st>>>(J);
        else k_tga_write<false><<<seg, kWriteThreads, 0, st>>>(J);
        launches += 3;
    }
    return launches;
}

const char* const kNames[FR_OUT_COUNT] = {
    "framebuffer.tga",    "framebuffer_SSAA.tga", "shadowmap.tga",        "zbuffer.tga",
    "gbuffer_normal.tga", "gbuffer_worldpos.tga", "gbuffer_albedo.tga",   "gbuffer_param.tga",
    "gbuffer_shading_type.tga", "gbuffer_ambient_occlusion.tga"};

// An output image of the context: its source, size and bytes per pixel; false if absent.
bool image_source(fr_ctx* ctx, int image, PixelSrc& src, int& w, int& h)
{
    src = PixelSrc{};
    src.gb = ctx->gb;
    src.S = ctx->S;
    w = ctx->W, h = ctx->H;
    const int k = ctx->info.ssaa_on ? ctx->info.ssaa_kernel : 1;
    switch (image)
    {
        case FR_OUT_FRAMEBUFFER: src.kind = kSrcRgbx, src.bpp = 3, src.p = ctx->frame8; return true;
        case FR_OUT_SSAA:
            if (!ctx->info.ssaa_on) return false;
            src.kind = kSrcRgbx, src.bpp = 3, src.p = ctx->ssaa, w = ctx->W / k, h = ctx->H / k;
            return true;
        case FR_OUT_SHADOWMAP:
            if (!ctx->info.shadow_on) return false;
            src.kind = kSrcF1, src.bpp = 1, src.p = ctx->shadow, w = ctx->SW, h = ctx->SH;
            return true;
        case FR_OUT_ZBUFFER: src.kind = kSrcF1, src.bpp = 1, src.p = ctx->gb.depth; return true;
        case FR_OUT_GB_AO:
            if (!ctx->info.deferred) return false;
            src.kind = kSrcF1, src.bpp = 1, src.p = ctx->gb.ao;
            return true;
        case FR_OUT_GB_NORMAL:
        case FR_OUT_GB_WORLDPOS:
            if (!ctx->info.deferred) return false;
            src.kind = kSrcGVec, src.bpp = 3, src.p = image == FR_OUT_GB_NORMAL ? ctx->gb.b : ctx->gb.a;
            return true;
        default:
        {
            if (!ctx->info.deferred) return false;
            src.kind = ctx->S.texLinear ? kSrcGMatLinear : kSrcGMat;
            src.bpp = image == FR_OUT_GB_SHADING_TYPE ? 1 : 3;
            src.which = image == FR_OUT_GB_ALBEDO ? 3 : image == FR_OUT_GB_PARAM ? 5 : 6;
            return true;
        }
    }
}

}  // namespace fro

// Per-context output buffers (freed by fr_destroy through frout_free).
struct FrOutputState
{
    uint8_t* arena = nullptr;  // every image's file at its slot
    size_t arenaCap = 0;
    void* scratch = nullptr;
    size_t scratchCap = 0;
    long long* sizes = nullptr;  // device [FR_OUT_COUNT]
    int launches = 0;            // kernels of the last encode
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

void frout_free(fr_ctx* ctx)
{
    FrOutputState* o = ctx->output;
    if (!o) return;
    if (o->arena) cudaFree(o->arena);
    if (o->scratch) cudaFree(o->scratch);
    if (o->sizes) cudaFree(o->sizes);
    for (auto e : o->ev)
        if (e) cudaEventDestroy(e);
    delete o;
    ctx->output = nullptr;
}

namespace
{

int out_fail(fr_ctx* c, int code, const std::string& m)
{
    if (c) c->err = m;
    return code;
}

int out_cuda(fr_ctx* c, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return FR_OK;
    return out_fail(c, FR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define FRO_CUDA(call)                                   \
    do                                                   \
    {                                                    \
        int _rc = out_cuda(ctx, (call), #call);          \
        if (_rc != FR_OK) return _rc;                    \
    } while (0)

// Slot of each image in the arena and the encoder's scratch, grown to the frame.
int ensure_output(fr_ctx* ctx, size_t slot[FR_OUT_COUNT + 1])
{
    slot[0] = 0;
    size_t need = fro::kCounterBytes;
    for (int i = 0; i < FR_OUT_COUNT; ++i)
    {
        fro::PixelSrc src;
        int w = 0, h = 0;
        size_t b = 0;
        if (fro::image_source(ctx, i, src, w, h))
        {
            b = fro::align256(fr_tga_max_bytes(w, h, src.bpp));
            need += fro::scratch_bytes((long long)w * h);
        }
        slot[i + 1] = slot[i] + b;
    }
    if (!ctx->output) ctx->output = new FrOutputState();
    FrOutputState* o = ctx->output;
    if (!o->sizes)
    {
        FRO_CUDA(cudaMalloc(&o->sizes, sizeof(long long) * FR_OUT_COUNT));
        FRO_CUDA(cudaEventCreate(&o->ev[0]));
        FRO_CUDA(cudaEventCreate(&o->ev[1]));
    }
    if (o->arenaCap < slot[FR_OUT_COUNT])
    {
        if (o->arena) cudaFree(o->arena);
        o->arena = nullptr, o->arenaCap = 0;
        FRO_CUDA(cudaMalloc(&o->arena, slot[FR_OUT_COUNT]));
        o->arenaCap = slot[FR_OUT_COUNT];
    }
    if (o->scratchCap < need)
    {
        if (o->scratch) cudaFree(o->scratch);
        o->scratch = nullptr, o->scratchCap = 0;
        FRO_CUDA(cudaMalloc(&o->scratch, need));
        o->scratchCap = need;
    }
    return FR_OK;
}

// Encodes the images in `mask` into their arena slots, one batch of launches;
// sizes land in o->sizes.
int encode_images(fr_ctx* ctx, unsigned mask, int rle, const size_t* slot, bool timed)
{
    FrOutputState* o = ctx->output;
    cudaStream_t st = ctx->stream;
    fro::EncodeJob list[FR_OUT_COUNT];
    int count = 0;
    for (int i = 0; i < FR_OUT_COUNT; ++i)
    {
        if (!(mask & (1u << i))) continue;
        fro::EncodeJob& e = list[count];
        if (!fro::image_source(ctx, i, e.src, e.w, e.h)) continue;
        e.rle = rle ? 1 : 0, e.vflip = 1, e.out = o->arena + slot[i], e.dSize = o->sizes + i;
        ++count;
    }
    FRO_CUDA(cudaMemsetAsync(o->sizes, 0, sizeof(long long) * FR_OUT_COUNT, st));
    if (timed) FRO_CUDA(cudaEventRecord(o->ev[0], st));
    o->launches = fro::encode_batch(list, count, o->scratch, st);
    if (timed) FRO_CUDA(cudaEventRecord(o->ev[1], st));
    FRO_CUDA(cudaGetLastError());
    return FR_OK;
}

int check_frame(fr_ctx* ctx)
{
    if (!ctx) return FR_ERR_INVALID;
    if (ctx->W == 0) return out_fail(ctx, FR_ERR_INVALID, "no frame rendered");
    return FR_OK;
}

}  // namespace

extern "C" {

const char* fr_output_name(int32_t image)
{
    return image >= 0 && image < FR_OUT_COUNT ? fro::kNames[image] : nullptr;
}

int fr_output_present(fr_ctx* ctx, int32_t image)
{
    int rc = check_frame(ctx);
    if (rc != FR_OK) return rc;
    if (image < 0 || image >= FR_OUT_COUNT) return out_fail(ctx, FR_ERR_INVALID, "unknown output image");
    fro::PixelSrc src;
    int w, h;
    return fro::image_source(ctx, image, src, w, h) ? 1 : 0;
}

int fr_output_shape(fr_ctx* ctx, int32_t image, int32_t* width, int32_t* height, int32_t* bytespp)
{
    int rc = check_frame(ctx);
    if (rc != FR_OK) return rc;
    if (image < 0 || image >= FR_OUT_COUNT) return out_fail(ctx, FR_ERR_INVALID, "unknown output image");
    fro::PixelSrc src;
    int w = 0, h = 0;
    if (!fro::image_source(ctx, image, src, w, h)) return 0;
    if (width) *width = w;
    if (height) *height = h;
    if (bytespp) *bytespp = src.bpp;
    return 1;
}

int64_t fr_output_encode(fr_ctx* ctx, int32_t image, int32_t rle, void* dst, size_t cap)
{
    int rc = check_frame(ctx);
    if (rc != FR_OK) return rc;
    if (image < 0 || image >= FR_OUT_COUNT) return out_fail(ctx, FR_ERR_INVALID, "unknown output image");
    cudaSetDevice(ctx->cfg.device);
    size_t slot[FR_OUT_COUNT + 1];
    if ((rc = ensure_output(ctx, slot)) != FR_OK) return rc;
    if (slot[image + 1] == slot[image]) return 0;  // the reference writes no such file
    if ((rc = encode_images(ctx, 1u << image, rle, slot, false)) != FR_OK) return rc;
    long long size = 0;
    FRO_CUDA(cudaMemcpyAsync(&size, ctx->output->sizes + image, sizeof(size), cudaMemcpyDeviceToHost, ctx->stream));
    FRO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (size < 0) return out_fail(ctx, FR_ERR_INVALID, "TGA encoder exceeded the file's size bound");
    if (dst && cap >= (size_t)size)
    {
        FRO_CUDA(cudaMemcpyAsync(dst, ctx->output->arena + slot[image], (size_t)size, cudaMemcpyDeviceToHost,
                                 ctx->stream));
        FRO_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return size;
}

int64_t fr_output_encode_all(fr_ctx* ctx, int32_t rle, void* dst, size_t cap, int64_t* sizes, float* device_ms)
{
    int rc = check_frame(ctx);
    if (rc != FR_OK) return rc;
    cudaSetDevice(ctx->cfg.device);
    size_t slot[FR_OUT_COUNT + 1];
    if ((rc = ensure_output(ctx, slot)) != FR_OK) return rc;
    if ((rc = encode_images(ctx, (1u << FR_OUT_COUNT) - 1u, rle, slot, true)) != FR_OK) return rc;
    long long sz[FR_OUT_COUNT];
    FRO_CUDA(cudaMemcpyAsync(sz, ctx->output->sizes, sizeof(sz), cudaMemcpyDeviceToHost, ctx->stream));
    FRO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (device_ms) FRO_CUDA(cudaEventElapsedTime(device_ms, ctx->output->ev[0], ctx->output->ev[1]));
    long long totalBytes = 0;
    for (int i = 0; i < FR_OUT_COUNT; ++i)
    {
        if (sz[i] < 0) return out_fail(ctx, FR_ERR_INVALID, "TGA encoder exceeded the file's size bound");
        if (sizes) sizes[i] = sz[i];
        totalBytes += sz[i];
    }
    if (!dst || cap < (size_t)totalBytes) return out_fail(ctx, FR_ERR_INVALID, "destination too small");
    uint8_t* d = static_cast<uint8_t*>(dst);
    for (int i = 0; i < FR_OUT_COUNT; ++i)
    {
        if (!sz[i]) continue;
        FRO_CUDA(cudaMemcpyAsync(d, ctx->output->arena + slot[i], (size_t)sz[i], cudaMemcpyDeviceToHost, ctx->stream));
        d += sz[i];
    }
    FRO_CUDA(cudaStreamSynchronize(ctx->stream));
    return totalBytes;
}

int fr_output_write(fr_ctx* ctx, const char* dir, int32_t rle)
{
    int rc = check_frame(ctx);
    if (rc != FR_OK) return rc;
    if (!dir) return out_fail(ctx, FR_ERR_INVALID, "null directory");
    size_t slot[FR_OUT_COUNT + 1];
    if ((rc = ensure_output(ctx, slot)) != FR_OK) return rc;
    std::vector<uint8_t> host(slot[FR_OUT_COUNT]);
    int64_t sizes[FR_OUT_COUNT];
    const int64_t total = fr_output_encode_all(ctx, rle, host.data(), host.size(), sizes, nullptr);
    if (total < 0) return (int)total;
    int files = 0;
    size_t at = 0;
    for (int i = 0; i < FR_OUT_COUNT; ++i)
    {
        if (!sizes[i]) continue;
        const std::string path = std::string(dir) + "/" + fro::kNames[i];
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) return out_fail(ctx, FR_ERR_IO, "cannot open " + path);
        const size_t wrote = std::fwrite(host.data() + at, 1, (size_t)sizes[i], f);
        const bool ok = std::fclose(f) == 0 && wrote == (size_t)sizes[i];
        if (!ok) return out_fail(ctx, FR_ERR_IO, "cannot write " + path);
        at += (size_t)sizes[i];
        ++files;
    }
    return files;
}

size_t fr_tga_max_bytes(int32_t width, int32_t height, int32_t bytespp)
{
    if (width < 0 || height < 0 || bytespp < 0) return 0;
    return (size_t)fro::kHeaderBytes + fro::kTailBytes + (size_t)width * (size_t)height * (1 + (size_t)bytespp);
}

size_t fr_tga_scratch_bytes(int32_t width, int32_t height)
{
    if (width < 0 || height < 0) return 0;
    return fro::kCounterBytes + fro::scratch_bytes((long long)width * height);
}

int fr_tga_encode_device(const void* d_pixels, int32_t width, int32_t height, int32_t bytespp, int32_t rle,
                         int32_t vflip, void* d_out, int64_t* d_size, void* d_scratch, void* stream)
{
    if (width < 0 || height < 0 || (bytespp != 1 && bytespp != 3 && bytespp != 4) || !d_out || !d_size)
        return FR_ERR_INVALID;
    if ((long long)width * height > 0 && (!d_pixels || (rle && !d_scratch))) return FR_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(d_out) & 15) return FR_ERR_INVALID;  // 16-byte stores
    fro::EncodeJob e{};
    e.src.kind = fro::kSrcBytes, e.src.bpp = bytespp, e.src.p = d_pixels;
    e.w = width, e.h = height, e.rle = rle ? 1 : 0, e.vflip = vflip ? 1 : 0;
    e.out = static_cast<uint8_t*>(d_out), e.dSize = reinterpret_cast<long long*>(d_size);
    fro::encode_batch(&e, 1, d_scratch, static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? FR_OK : FR_ERR_CUDA;
}

}  // extern "C"
