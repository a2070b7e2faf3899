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
//      packet length L(s) at every position, and by pointer doubling over
//      next(s) = s + L(s) the segment's transfer function: for each of the 128
//      possible offsets of its first packet start, the offset of the first
//      packet start in the next segment and the file bytes of the packets on
//      the way.
//   2. k_tga_entries (CTA per image): a tree scan composing the transfer
//      functions gives every segment's actual first packet start; a scan of the
//      byte counts at those entries gives each segment's file offset.
//   3. k_tga_write (CTA per segment): the packet starts of the segment (the same
//      doubling on 128-pixel sub-blocks, then one lane per sub-block walks its
//      packets), then every pixel of those packets writes its bytes (a packet
//      start also its header byte) at the offset a block scan gives it.
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
    kSrcGBuf = 4    // a field of the packed G-buffer, converted as a Buffer3f / Buffer1f
};

struct PixelSrc
{
    int kind, bpp, which;  // which (kSrcGBuf): 0 normal, 1 world position, 3 albedo, 5 param, 6 shading type
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

// Pixel i's bytes in TGA order, packed little-endian into 32 bits.
__device__ __forceinline__ uint32_t src_pixel(const PixelSrc& s, long long i)
{
    switch (s.kind)
    {
        case kSrcBytes:
        {
            const uint8_t* p = static_cast<const uint8_t*>(s.p) + i * s.bpp;
            uint32_t v = p[0];
            if (s.bpp >= 3) v |= ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16);
            if (s.bpp == 4) v |= (uint32_t)p[3] << 24;
            return v;
        }
        case kSrcRgbx:
        {
            const uint32_t c = static_cast<const uint32_t*>(s.p)[i];
            return ((c >> 16) & 0xffu) | (c & 0xff00u) | ((c & 0xffu) << 16);
        }
        case kSrcF1: return ref_u8(static_cast<const float*>(s.p)[i] * 255);
        case kSrcF3:
        {
            const float* f = static_cast<const float*>(s.p) + 3 * i;
            return bgr3(F3{f[0], f[1], f[2]});
        }
        default:
        {
            if (s.which == 0 || s.which == 1)
            {
                const float4 v = s.which == 0 ? s.gb.b[i] : s.gb.a[i];  // normal / world position
                return bgr3(F3{v.x, v.y, v.z});
            }
            const GDecoded g = decode_gbuffer(s.S, s.gb.c[i]);
            if (s.which == 6) return ref_u8(g.type * 255);
            return bgr3(s.which == 3 ? g.albedo : g.param);
        }
    }
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
constexpr int kEntryThreads = 1024;
constexpr size_t kEntrySmemMax = 200 * 1024;

// One image of a batch, with its slices of the scratch buffer.
struct Job
{
    PixelSrc src;
    long long n;
    int w, h, bpp, rle, vflip;
    int S;              // segments
    int segBase;        // first CTA of this image in the per-segment launches
    uint8_t* out;
    long long cap;      // bytes of out: no write goes past it
    long long* dSize;   // file size, or -1 if it would not fit in cap
    uint8_t* info;      // [n] (packet length - 1) | 0x80 for a run, at every position
    uint8_t* func;      // [S][128] transfer function: entry offset -> next segment's entry offset
    uint16_t* fbytes;   // [S][128] file bytes of the segment's packets for each entry offset
    uint8_t* upper;     // [S + 64][128] upper tree levels, when shared memory is too small
    uint8_t* entLv;     // [2S + 64] entries of every tree level, same case
    uint8_t* ent;       // [S] offset of each segment's first packet start
    long long* segOff;  // [S] file offset of each segment's first packet, after the header
};

struct Jobs
{
    int count;
    int entrySmem;      // dynamic shared memory of the k_tga_entries launch
    Job j[kMaxJobs];
};

__device__ __forceinline__ int job_of(const Jobs& J, int blk)
{
    int ji = 0;
    while (ji + 1 < J.count && blk >= J.j[ji + 1].segBase) ++ji;
    return ji;
}

// Per segment: info bytes, and by pointer doubling over next(s) = s + L(s),
// carrying the packets' file bytes, the transfer function and its byte counts.
__global__ void __launch_bounds__(kParseThreads) k_tga_parse(const __grid_constant__ Jobs J)
{
    __shared__ uint32_t eqw[kWinWords];
    __shared__ uint16_t Jp[2][kSeg];
    __shared__ uint16_t Wp[2][kSeg];  // bytes along the path: at most 4223 pixels * 5 < 65536
    const Job& jb = J.j[job_of(J, blockIdx.x)];
    const int k = blockIdx.x - jb.segBase, bpp = jb.bpp;
    const long long n = jb.n, seg0 = (long long)k * kSeg;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // bit r of eqw: pixel seg0 + r equals its successor
    for (int w = warp; w < kWinWords; w += kParseThreads / 32)
    {
        const long long g = seg0 + w * 32 + lane;
        const uint32_t a = g < n ? src_pixel(jb.src, g) : 0u;
        uint32_t b = __shfl_down_sync(0xffffffffu, a, 1);
        if (lane == 31) b = g + 1 < n ? src_pixel(jb.src, g + 1) : 0u;
        const unsigned m = __ballot_sync(0xffffffffu, g + 1 < n && a == b);
        if (lane == 0) eqw[w] = m;
    }
    __syncthreads();
    const int segLen = (int)min((long long)kSeg, n - seg0);
    for (int r = threadIdx.x; r < kSeg; r += kParseThreads)
    {
        if (r >= segLen)
        {
            Jp[0][r] = (uint16_t)kSeg;  // past the image: terminal
            Wp[0][r] = 0;
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
        Jp[0][r] = (uint16_t)(r + L);
        Wp[0][r] = (uint16_t)(run ? 1 + bpp : 1 + L * bpp);
    }
    __syncthreads();
    int cur = 0;
    for (int round = 0; round < 12; ++round)  // 2^12 = kSeg steps
    {
        int open = 0;
        for (int r = threadIdx.x; r < kSeg; r += kParseThreads)
        {
            const int x = Jp[cur][r];
            int y = x, wv = Wp[cur][r];
            if (x < kSeg) y = Jp[cur][x], wv += Wp[cur][x];
            Jp[cur ^ 1][r] = (uint16_t)y;
            Wp[cur ^ 1][r] = (uint16_t)wv;
            open |= (r < 128 && y < kSeg);
        }
        cur ^= 1;
        if (!__syncthreads_or(open)) break;
    }
    if (threadIdx.x < 128)
    {
        jb.func[(size_t)k * 128 + threadIdx.x] = (uint8_t)(Jp[cur][threadIdx.x] - kSeg);
        jb.fbytes[(size_t)k * 128 + threadIdx.x] = Wp[cur][threadIdx.x];
    }
}

// CTA per image: tree scan of the transfer functions (in shared memory when it
// fits) -> each segment's entry offset; its bytes at that entry, scanned into
// file offsets; header, footer and file size.
__global__ void __launch_bounds__(kEntryThreads) k_tga_entries(const __grid_constant__ Jobs J)
{
    extern __shared__ __align__(16) uint8_t sm[];
    __shared__ int off[40], cnt[40], levels;
    __shared__ long long scanBuf[kEntryThreads];
    const Job& jb = J.j[blockIdx.x];
    const int S = jb.S;
    if (threadIdx.x == 0)
    {
        int L = 0;
        off[0] = 0, cnt[0] = S;
        while (cnt[L] > 1 && L < 38)
        {
            cnt[L + 1] = (cnt[L] + 1) / 2;
            off[L + 1] = off[L] + cnt[L];
            ++L;
        }
        levels = L;
    }
    __syncthreads();
    const int total = off[levels] + cnt[levels], upperCount = total - S;
    const size_t needA = (size_t)total * 128 + total, needB = (size_t)upperCount * 128 + total;
    uint8_t *lv0 = jb.func, *up = jb.upper, *entL = jb.entLv;
    if (needA <= (size_t)J.entrySmem)
    {
        lv0 = sm, up = sm + (size_t)S * 128, entL = sm + (size_t)total * 128;
        const uint4* src = reinterpret_cast<const uint4*>(jb.func);
        uint4* dst = reinterpret_cast<uint4*>(sm);
        for (int i = threadIdx.x; i < S * 8; i += kEntryThreads) dst[i] = src[i];
    }
    else if (needB <= (size_t)J.entrySmem)
        up = sm, entL = sm + (size_t)upperCount * 128;
    __syncthreads();
    auto map = [&](int l, int node) -> uint8_t* {
        return l == 0 ? lv0 + (size_t)node * 128 : up + (size_t)(off[l] - S + node) * 128;
    };
    for (int l = 0; l < levels; ++l)
    {
        for (int i = threadIdx.x; i < cnt[l + 1] * 128; i += kEntryThreads)
        {
            const int j = i >> 7, e = i & 127, a = 2 * j;
            int x = map(l, a)[e] & 127;
            if (a + 1 < cnt[l]) x = map(l, a + 1)[x] & 127;
            map(l + 1, j)[e] = (uint8_t)x;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) entL[off[levels]] = 0;
    __syncthreads();
    for (int l = levels; l >= 1; --l)
    {
        for (int j = threadIdx.x; j < cnt[l]; j += kEntryThreads)
        {
            const int x = entL[off[l] + j] & 127;
            entL[off[l - 1] + 2 * j] = (uint8_t)x;
            if (2 * j + 1 < cnt[l - 1]) entL[off[l - 1] + 2 * j + 1] = map(l - 1, 2 * j)[x];
        }
        __syncthreads();
    }
    // bytes of each segment at its entry; exclusive scan over contiguous slices
    const int per = (S + kEntryThreads - 1) / kEntryThreads;
    const int lo = threadIdx.x * per, hi = min(S, lo + per);
    long long mine = 0;
    for (int k = lo; k < hi; ++k)
    {
        const int e = entL[k] & 127;
        jb.ent[k] = (uint8_t)e;
        mine += jb.fbytes[(size_t)k * 128 + e];
    }
    scanBuf[threadIdx.x] = mine;
    __syncthreads();
    for (int d = 1; d < kEntryThreads; d <<= 1)
    {
        const long long v = threadIdx.x >= d ? scanBuf[threadIdx.x - d] : 0;
        __syncthreads();
        scanBuf[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = scanBuf[threadIdx.x] - mine;
    for (int k = lo; k < hi; ++k)
    {
        jb.segOff[k] = run;
        run += jb.fbytes[(size_t)k * 128 + (entL[k] & 127)];
    }
    if (threadIdx.x == kEntryThreads - 1)
    {
        const long long body = scanBuf[kEntryThreads - 1];
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

// Per segment: its packet starts (sub-block transfer functions by pointer
// doubling, then one lane per 128-pixel sub-block walks its packets), then
// every pixel of the segment's packets writes its bytes at the offset a block
// scan gives it (a packet start also its header byte).
__global__ void __launch_bounds__(kWriteThreads) k_tga_write(const __grid_constant__ Jobs J)
{
    __shared__ uint8_t inf[kSeg + 128];
    __shared__ uint16_t Jb[2][kSeg];
    __shared__ uint32_t bits[kSegWords];
    __shared__ uint8_t xs[kSubBlocks];
    __shared__ int warpSum[kWriteThreads / 32];
    const Job& jb = J.j[job_of(J, blockIdx.x)];
    const int kk = blockIdx.x - jb.segBase, bpp = jb.bpp;
    const long long n = jb.n, seg0 = (long long)kk * kSeg;
    const int segLen = (int)min((long long)kSeg, n - seg0);
    const int avail = (int)min((long long)kSeg + 128, n - seg0);
    for (int i = threadIdx.x; i < avail; i += kWriteThreads) inf[i] = jb.info[seg0 + i];
    for (int i = threadIdx.x; i < kSegWords; i += kWriteThreads) bits[i] = 0u;
    __syncthreads();
    for (int r = threadIdx.x; r < kSeg; r += kWriteThreads)
        Jb[0][r] = (uint16_t)(r < segLen ? r + (inf[r] & 127) + 1 : (r | 127) + 1);
    __syncthreads();
    int cur = 0;
    for (int round = 0; round < 7; ++round)  // 2^7 = 128 steps: a sub-block's path
    {
        for (int r = threadIdx.x; r < kSeg; r += kWriteThreads)
        {
            const int x = Jb[cur][r];
            Jb[cur ^ 1][r] = (uint16_t)(x <= (r | 127) ? Jb[cur][x] : x);
        }
        cur ^= 1;
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        int x = jb.ent[kk] & 127;
        for (int b = 0; b < kSubBlocks; ++b)
        {
            xs[b] = (uint8_t)x;
            x = (Jb[cur][128 * b + x] - 128 * (b + 1)) & 127;
        }
    }
    __syncthreads();
    if (threadIdx.x < kSubBlocks)
    {
        const int b = threadIdx.x, end = min(128 * (b + 1), segLen);
        for (int s = 128 * b + xs[b]; s < end; s += (inf[s] & 127) + 1) bits[s >> 5] |= 1u << (s & 31);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long a = seg0 + (jb.ent[kk] & 127);
    const long long bEnd = kk + 1 < jb.S ? seg0 + kSeg + (jb.ent[kk + 1] & 127) : n;
    long long base = kHeaderBytes + jb.segOff[kk];
    for (long long r0 = a; r0 < bEnd; r0 += kWriteThreads)
    {
        const long long r = r0 + threadIdx.x;
        int bytes = 0;
        bool start = false;
        int rel = 0;
        if (r < bEnd)
        {
            rel = (int)(r - seg0);
            start = rel < kSeg && ((bits[rel >> 5] >> (rel & 31)) & 1u);
            // a later pixel of a packet: raw packets store it, runs do not
            bytes = start ? 1 + bpp : ((inf[rel - 1] & 0x80) ? 0 : bpp);
        }
        int incl = bytes;
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
        if (bytes && base + before + incl <= jb.cap - kTailBytes)
        {
            uint8_t* o = jb.out + base + before + incl - bytes;
            if (start)
            {
                const int v = inf[rel], L = (v & 127) + 1;
                *o++ = (uint8_t)((v & 0x80) ? L + 127 : L - 1);
            }
            const uint32_t px = src_pixel(jb.src, r);
            for (int c = 0; c < bpp; ++c) o[c] = (uint8_t)(px >> (8 * c));
        }
        base += all;
        __syncthreads();
    }
}

// Raw files (and empty images): pixel bytes, header and tail.
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
    const uint32_t px = src_pixel(jb.src, i);
    uint8_t* o = jb.out + kHeaderBytes + i * jb.bpp;
    for (int c = 0; c < jb.bpp; ++c) o[c] = (uint8_t)(px >> (8 * c));
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int segments(long long n) { return (int)((n + kSeg - 1) / kSeg); }

// Scratch bytes of one image of n pixels.
size_t scratch_bytes(long long n)
{
    const size_t S = (size_t)segments(n);
    return align256((size_t)n) + align256(S * 128) + align256(S * 256) + align256((S + 64) * 128) +
           align256(2 * S + 64) + align256(S) + align256(S * 8);
}

// Entry-scan shared memory one image wants (0: it runs from global memory).
size_t entry_smem(long long n)
{
    int S = segments(n), total = 0;
    for (int c = S; ; c = (c + 1) / 2)
    {
        total += c;
        if (c <= 1) break;
    }
    const size_t needA = (size_t)total * 128 + total, needB = (size_t)(total - S) * 128 + total;
    return needA <= kEntrySmemMax ? needA : needB <= kEntrySmemMax ? needB : 0;
}

struct EncodeJob
{
    PixelSrc src;
    int w, h, rle, vflip;
    uint8_t* out;
    long long* dSize;
};

// Launches the encoder for up to kMaxJobs images (scratch: the sum of their
// scratch_bytes); returns the number of kernels launched.
int encode_batch(const EncodeJob* list, int count, void* scratch, cudaStream_t st)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_tga_entries, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kEntrySmemMax);
        attr = true;
    }
    Jobs J{};
    int seg = 0, launches = 0;
    size_t smem = 0;
    uint8_t* p = static_cast<uint8_t*>(scratch);
    for (int i = 0; i < count && i < kMaxJobs; ++i)
    {
        const EncodeJob& e = list[i];
        Job jb{};
        jb.src = e.src, jb.n = (long long)e.w * e.h, jb.w = e.w, jb.h = e.h, jb.bpp = e.src.bpp;
        jb.rle = e.rle, jb.vflip = e.vflip, jb.out = e.out, jb.dSize = e.dSize;
        jb.cap = (long long)fr_tga_max_bytes(e.w, e.h, e.src.bpp);
        jb.S = segments(jb.n);
        const size_t S = (size_t)jb.S;
        uint8_t* q = p;
        jb.info = q, q += align256((size_t)jb.n);
        jb.func = q, q += align256(S * 128);
        jb.fbytes = reinterpret_cast<uint16_t*>(q), q += align256(S * 256);
        jb.upper = q, q += align256((S + 64) * 128);
        jb.entLv = q, q += align256(2 * S + 64);
        jb.ent = q, q += align256(S);
        jb.segOff = reinterpret_cast<long long*>(q);
        p += scratch_bytes(jb.n);
        if (!jb.rle || jb.n == 0)
        {
            const long long threads = jb.n > 0 && !jb.rle ? jb.n : 1;
            k_tga_plain<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(jb);
            ++launches;
            continue;
        }
        jb.segBase = seg;
        seg += jb.S;
        smem = std::max(smem, entry_smem(jb.n));
        J.j[J.count++] = jb;
    }
    if (J.count)
    {
        J.entrySmem = (int)smem;
        k_tga_parse<<<seg, kParseThreads, 0, st>>>(J);
        k_tga_entries<<<J.count, kEntryThreads, smem, st>>>(J);
        k_tga_write<<<seg, kWriteThreads, 0, st>>>(J);
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
        default:
        {
            if (!ctx->info.deferred) return false;
            static const int which[FR_OUT_COUNT] = {-1, -1, -1, -1, 0, 1, 3, 5, 6, -1};
            src.kind = kSrcGBuf, src.which = which[image], src.bpp = image == FR_OUT_GB_SHADING_TYPE ? 1 : 3;
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
    size_t need = 0;
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
    return fro::scratch_bytes((long long)width * height);
}

int fr_tga_encode_device(const void* d_pixels, int32_t width, int32_t height, int32_t bytespp, int32_t rle,
                         int32_t vflip, void* d_out, int64_t* d_size, void* d_scratch, void* stream)
{
    if (width < 0 || height < 0 || (bytespp != 1 && bytespp != 3 && bytespp != 4) || !d_out || !d_size)
        return FR_ERR_INVALID;
    if ((long long)width * height > 0 && (!d_pixels || (rle && !d_scratch))) return FR_ERR_INVALID;
    fro::EncodeJob e{};
    e.src.kind = fro::kSrcBytes, e.src.bpp = bytespp, e.src.p = d_pixels;
    e.w = width, e.h = height, e.rle = rle ? 1 : 0, e.vflip = vflip ? 1 : 0;
    e.out = static_cast<uint8_t*>(d_out), e.dSize = reinterpret_cast<long long*>(d_size);
    fro::encode_batch(&e, 1, d_scratch, static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? FR_OK : FR_ERR_CUDA;
}

}  // extern "C"
