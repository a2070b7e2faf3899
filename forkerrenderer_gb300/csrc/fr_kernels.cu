// The frame's CUDA kernels for sm_103a.
//
// Visibility is resolved exactly as the reference's sequential, in-order,
// strict-less depth test (forkergl.cpp:165-234) would leave it, but in parallel:
// every covered fragment forms a 64-bit key (order-preserving depth bits, draw
// index) and the per-pixel unsigned minimum survives (frx::make_key). Triangles
// are drawn by one thread (tiny bounding boxes), one warp (medium) or through
// 16 x 16 tile bins with one CTA per tile (large), all feeding the same keys.
// Shading then runs once per pixel on the surviving triangle, which is what the
// reference's overwrite-on-pass leaves in its buffers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <float.h>
#include <algorithm>

#include "fr_kernels.cuh"
#include "fr_ssao.cuh"
#include "forkerrenderer.h"

using namespace frd;

namespace frk
{

namespace
{

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(hi, max(v, lo)); }

__device__ __forceinline__ void load_rtri(const int4* __restrict__ scr, int4 tv, frx::RTri& r, bool withRecip = true)
{
    int4 a = scr[tv.x], b = scr[tv.y], c = scr[tv.z];
    r.x[0] = a.x, r.x[1] = b.x, r.x[2] = c.x;
    r.y[0] = a.y, r.y[1] = b.y, r.y[2] = c.y;
    r.d[0] = __int_as_float(a.z), r.d[1] = __int_as_float(b.z), r.d[2] = __int_as_float(c.z);
    frx::classify(r, withRecip);
}

// Resolve record of a fast-class triangle with small coordinates (every
// coordinate within +-kSmallLimit, so each fits 16 bits): the packed vertices,
// bz and RN(1 / bz), and the per-vertex .w screen data. rec[2t] = (x0|y0, x1|y1,
// x2|y2, bz), rec[2t + 1] = (w0, w1, w2, rbz) as bits; bz = 0 marks a triangle
// without a record (any other class). With it a resolve rebuilds the RTri that
// bary() needs (the same fields load_rtri derives) in one load round trip.
__device__ __forceinline__ int pack_xy(int x, int y) { return (x & 0xffff) | (y << 16); }

__device__ __forceinline__ void store_tri_record(int4* rec, int t, const frx::RTri& r, int w0, int w1, int w2)
{
    const bool ok = r.cls == frx::kTriFast && r.small;
    rec[2 * (size_t)t] = make_int4(pack_xy(r.x[0], r.y[0]), pack_xy(r.x[1], r.y[1]), pack_xy(r.x[2], r.y[2]),
                                   ok ? (int)r.bz : 0);
    rec[2 * (size_t)t + 1] = make_int4(w0, w1, w2, __float_as_int(r.rbz));
}

// The RTri of a record (false: the triangle has none). d[] is not restored.
__device__ __forceinline__ bool load_tri_record(const int4* __restrict__ rec, int t, frx::RTri& r, int4& wv)
{
    const int4 a = __ldg(rec + 2 * (size_t)t);
    wv = __ldg(rec + 2 * (size_t)t + 1);
    if (a.w == 0) return false;
    r.x[0] = (a.x << 16) >> 16, r.y[0] = a.x >> 16;
    r.x[1] = (a.y << 16) >> 16, r.y[1] = a.y >> 16;
    r.x[2] = (a.z << 16) >> 16, r.y[2] = a.z >> 16;
    r.d[0] = r.d[1] = r.d[2] = 0.f;
    r.cls = frx::kTriFast;
    r.bz = a.w;
    r.fbz = (float)a.w;
    r.rbz = __int_as_float(wv.w);
    r.s53 = 0, r.m53 = 0;  // the on-edge weight derives its reciprocal when needed
    r.small = 1;
    return true;
}

// BoundBox::GenerateBoundBox (forkergl.cpp:154-162)
__device__ __forceinline__ void bbox(const frx::RTri& r, int W, int H, int& x0, int& x1, int& y0, int& y1)
{
    x0 = clampi(min(r.x[0], min(r.x[1], r.x[2])), 0, W - 1);
    y0 = clampi(min(r.y[0], min(r.y[1], r.y[2])), 0, H - 1);
    x1 = clampi(max(r.x[0], max(r.x[1], r.x[2])), 0, W - 1);
    y1 = clampi(max(r.y[0], max(r.y[1], r.y[2])), 0, H - 1);
}

template <int kOnly = 0>
__device__ __forceinline__ void fragment_key(const frx::RTri& r, int t, int px, int py, int W,
                                             unsigned long long* __restrict__ keys)
{
    float b0, b1, b2;
    if (!frx::bary<kOnly, false>(r, px, py, b0, b1, b2)) return;
    float d = frx::depth_of(r, b0, b1, b2);
    if (!frx::depth_passes_clear(d)) return;
    atomicMin(keys + (size_t)py * W + px, frx::make_key(d, (unsigned)t));  // result unused: RED.MIN
}

// ---- vertex stages ------------------------------------------------------------------------

// Camera vertex shader (gshader.h:41-92 / phongshader.h:35-85 / pbrshader.h:35-85)
// per unique vertex, then the viewport transform and int snap of DrawTriangle
// (forkergl.cpp:244-249). Normals are transformed per unique normal.
__global__ void k_transform_camera(DevScene S, FrameConst F, VertexOut vo)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < S.numVerts)
    {
        const DevModel& Md = S.models[S.vmodel[v]];
        float4 p = S.pos[v];
        F4 posWS = mul4(Md.M, F4{p.x, p.y, p.z, 1.f});
        F4 posVS = mul4(F.V, posWS);
        F4 posCS = mul4(F.P, posVS);
        F4 lndc{0.f, 0.f, 0.f, 0.f};
        if (F.shadowOn)
        {
            lndc = mul4(F.L, posWS);
            lndc = div4(lndc, lndc.w);
        }
        float ow = 1.f / posCS.w;
        posWS = scale4(posWS, ow);
        F3 tw{0.f, 0.f, 0.f};
        if (Md.has_tangents)
        {
            float4 t = S.tan[v];
            tw = mul3(Md.N3, normalize(F3{t.x, t.y, t.z})) * ow;
        }
        if (F.shadowOn) lndc = scale4(lndc, ow);
        F4 ndc = div4(posCS, posCS.w);
        F4 c = mul4(F.VPort, ndc);
        vo.scr[v] = make_int4(frx::f2i_sat(c.x), frx::f2i_sat(c.y), __float_as_int(c.z), 0);
        vo.pw[v] = make_float4(posWS.x, posWS.y, posWS.z, ow);
        vo.lw[v] = make_float4(lndc.x, lndc.y, lndc.z, 0.f);
        vo.tw[v] = make_float4(tw.x, tw.y, tw.z, 0.f);
    }
    if (v < S.numNormals)
    {
        const DevModel& Md = S.models[S.nmodel[v]];
        float4 n = S.nrm[v];
        F3 nn = mul3(Md.N3, normalize(F3{n.x, n.y, n.z}));
        vo.npre[v] = make_float4(nn.x, nn.y, nn.z, 0.f);
    }
}

// DepthShader::ProcessVertex (depthshader.h:21-28): (L * M) * v, / w, then the
// shadow viewport. .w keeps NDC z for the shadow-map value.
__global__ void k_transform_light(DevScene S, FrameConst F, int4* scrL)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= S.numVerts) return;
    const DevModel& Md = S.models[S.vmodel[v]];
    float4 p = S.pos[v];
    F4 cs = mul4(Md.LM, F4{p.x, p.y, p.z, 1.f});
    F4 ndc = div4(cs, cs.w);
    F4 c = mul4(F.SVPort, ndc);
    scrL[v] = make_int4(frx::f2i_sat(c.x), frx::f2i_sat(c.y), __float_as_int(c.z), __float_as_int(ndc.z));
}

// ---- raster ----------------------------------------------------------------------------------

// Triangle setup and the small-triangle raster. Each thread classifies one
// triangle. Triangles whose clamped bounding box has at most smallArea pixels
// are drawn right here, cooperatively by the warp: the 32 boxes are flattened
// (warp prefix sum of their areas) and dealt out pixel by pixel to the lanes,
// so every lane stays busy whatever the mix of triangle sizes. Larger fast
// triangles go to the medium list (one warp each), the rest to the tile bins.
constexpr int kSetupThreads = 256;

// Five CTAs per SM (at most 51 registers a thread; 48 without spills): with the two
// queues, an unbounded allocation took 52 and four CTAs, and in the concurrent frame
// the extra resident warps let the shadow setup overlap the camera chain better.
__global__ void __launch_bounds__(kSetupThreads, 5) k_setup(DevScene S, const int4* __restrict__ scr, RasterParams rp,
                                                         RasterScratch rs)
{
    // the warp's small triangles, compacted in draw order (slot = rank among them)
    __shared__ frx::RTri sh[kSetupThreads];
    __shared__ int4 shb[kSetupThreads];  // (x0, y0, w, triangle)
    __shared__ float shr[kSetupThreads]; // 1 / w
    __shared__ int shs[kSetupThreads];   // first pixel in the warp's flattened pixel list
    __shared__ int shq[2][kSetupThreads / 32][64];  // per-warp queues of covered pixels (slot, y, x):
                                                    // off edge BC, on edge BC
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, wbase = threadIdx.x & ~31;
    int area = 0;
    frx::RTri r;
    int sx0 = 0, sy0 = 0, sw = 1;
    if (t < S.numTris)
    {
        const int4 tv = S.triV[t];
        load_rtri(scr, tv, r);
        if (rs.triRec) store_tri_record(rs.triRec, t, r, scr[tv.x].w, scr[tv.y].w, scr[tv.z].w);
        if (r.cls != frx::kTriEmpty)
        {
            int x0, x1, y0, y1;
            bbox(r, rp.W, rp.H, x0, x1, y0, y1);
            long long a = (long long)(x1 - x0 + 1) * (y1 - y0 + 1);
            if (r.cls == frx::kTriFast && a <= rp.smallArea && rp.W <= 8192 && rp.H <= 8192)
            {
                area = (int)a;
                sx0 = x0, sy0 = y0, sw = x1 - x0 + 1;
            }
            else if (r.cls == frx::kTriFast && a <= rp.mediumArea)
            {
                int i = atomicAdd(&rs.counters[0], 1);
                if (i < rs.triCap)
                {
                    rs.mediumTris[i] = r;
                    rs.mediumIdx[i] = t;
                }
                else
                    atomicOr(&rs.counters[3], kStatusListOverflow);
            }
            else
            {
                int i = atomicAdd(&rs.counters[1], 1);
                if (i < rs.triCap)
                {
                    rs.largeTris[i] = r;
                    rs.largeIdx[i] = t;
                    rs.largeAux[i] = make_float4(__int_as_float(scr[tv.x].w), __int_as_float(scr[tv.y].w),
                                                 __int_as_float(scr[tv.z].w), 0.f);
                }
                else
                    atomicOr(&rs.counters[3], kStatusListOverflow);
            }
        }
    }
    int incl = area;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int slot = __popc(__ballot_sync(0xffffffffu, area > 0) & ((1u << lane) - 1u));
    if (area > 0)
    {
        sh[wbase + slot] = r;
        shb[wbase + slot] = make_int4(sx0, sy0, sw, t);
        shr[wbase + slot] = 1.f / (float)sw;
        shs[wbase + slot] = incl - area;
    }
    __syncwarp();
    // Pixels that pass the cheap integer coverage pre-test are queued (per warp,
    // in shared memory) and the exact evaluation runs on full 32-pixel batches,
    // so the expensive path never idles lanes on uncovered pixels. Pixels on edge
    // BC (whose weight takes the exact on-edge path) have a queue of their own, so
    // neither batch form carries the other's code path.
    int* queue = shq[0][threadIdx.x >> 5];
    int* queueE = shq[1][threadIdx.x >> 5];
    int qn = 0, qe = 0;
    // The owner of pixel p of the flattened list is the last triangle that starts
    // at or before p: one OR-reduction marks the triangles starting in this
    // 32-pixel step, and the owner is the previous step's last owner plus the
    // starts up to the lane (slots follow the start order).
    int owner = -1;
    const int rel0 = incl - area;
    for (int base = 0; base < total; base += 32)
    {
        const int p = base + lane;
        const int rel = rel0 - base;
        const unsigned starts = __reduce_or_sync(0xffffffffu, (area > 0 && (unsigned)rel < 32u) ? 1u << rel : 0u);
        const int j = owner + __popc(starts & ((2u << lane) - 1u));
        owner += __popc(starts);
        int kind = 0;
        int px = 0, py = 0;
        if (p < total)
        {
            int local = p - shs[wbase + j];
            int4 b = shb[wbase + j];
            int q = (int)((float)local * shr[wbase + j]);
            int rem = local - q * b.z;
            if (rem < 0) --q, rem += b.z;
            else if (rem >= b.z) ++q, rem -= b.z;
            px = b.x + rem, py = b.y + q;
            kind = frx::pretest_kind(sh[wbase + j], px, py);
        }
        const unsigned lt = (1u << lane) - 1u;
        const unsigned m = __ballot_sync(0xffffffffu, kind == 1), me = __ballot_sync(0xffffffffu, kind == 2);
        const int entry = (j << 26) | (py << 13) | px;
        if (kind == 1) queue[qn + __popc(m & lt)] = entry;
        if (kind == 2) queueE[qe + __popc(me & lt)] = entry;
        qn += __popc(m);
        qe += __popc(me);
        __syncwarp();
        if (qn >= 32)
        {
            int e = queue[lane];
            int jj = e >> 26;
            fragment_key<1>(sh[wbase + jj], shb[wbase + jj].w, e & 8191, (e >> 13) & 8191, rp.W, rs.keys);
            __syncwarp();
            if (lane < qn - 32) queue[lane] = queue[32 + lane];
            qn -= 32;
            __syncwarp();
        }
        if (qe >= 32)
        {
            int e = queueE[lane];
            int jj = e >> 26;
            fragment_key<2>(sh[wbase + jj], shb[wbase + jj].w, e & 8191, (e >> 13) & 8191, rp.W, rs.keys);
            __syncwarp();
            if (lane < qe - 32) queueE[lane] = queueE[32 + lane];
            qe -= 32;
            __syncwarp();
        }
    }
    if (lane < qn)
    {
        int e = queue[lane];
        int jj = e >> 26;
        fragment_key<1>(sh[wbase + jj], shb[wbase + jj].w, e & 8191, (e >> 13) & 8191, rp.W, rs.keys);
    }
    if (lane < qe)
    {
        int e = queueE[lane];
        int jj = e >> 26;
        fragment_key<2>(sh[wbase + jj], shb[wbase + jj].w, e & 8191, (e >> 13) & 8191, rp.W, rs.keys);
    }
}

// One warp per medium triangle; lanes stride over its bounding box.
__global__ void k_raster_medium(RasterParams rp, RasterScratch rs)
{
    int n = min(rs.counters[0], rs.triCap);
    int lane = threadIdx.x & 31;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int i = warp; i < n; i += nwarps)
    {
        frx::RTri r = rs.mediumTris[i];
        int t = rs.mediumIdx[i];
        int x0, x1, y0, y1;
        bbox(r, rp.W, rp.H, x0, x1, y0, y1);
        int w = x1 - x0 + 1, area = w * (y1 - y0 + 1);
        for (int p = lane; p < area; p += 32) fragment_key(r, t, x0 + p % w, y0 + p / w, rp.W, rs.keys);
    }
}

// Tile binning of large triangles: pass 0 counts (triangle, tile) pairs, pass 1
// scatters triangle list indices into the per-tile ranges. Work items are
// (triangle, tile row) pairs, one warp each, so a triangle spanning thousands
// of tiles is binned by many warps at once. With at most kDirectLarge large
// triangles the fine raster takes them all (each gated by its box per pixel,
// the same pixels the bins would give it) and the binning kernels do nothing.
constexpr int kDirectLarge = 8;

__device__ __forceinline__ bool large_direct(const RasterScratch& rs)
{
    return min(rs.counters[1], rs.triCap) <= kDirectLarge;
}

__global__ void k_bin(RasterParams rp, RasterScratch rs, int scatter)
{
    if (large_direct(rs)) return;
    int n = min(rs.counters[1], rs.triCap);
    int lane = threadIdx.x & 31;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nwarps = (gridDim.x * blockDim.x) >> 5;
    int ntx = (rp.W + kTile - 1) / kTile;
    int maxRows = (rp.H + kTile - 1) / kTile;
    long long items = (long long)n * maxRows;
    for (long long it = warp; it < items; it += nwarps)
    {
        int i = (int)(it / maxRows), row = (int)(it % maxRows);
        const frx::RTri& r = rs.largeTris[i];
        int x0, x1, y0, y1;
        bbox(r, rp.W, rp.H, x0, x1, y0, y1);
        int ty = y0 / kTile + row;
        if (ty > y1 / kTile) continue;
        int tx0 = x0 / kTile, tx1 = x1 / kTile;
        for (int tx = tx0 + lane; tx <= tx1; tx += 32)
        {
            int tile = ty * ntx + tx;
            if (!scatter)
                atomicAdd(&rs.tileCount[tile], 1);
            else
            {
                long long pos = (long long)rs.tileStart[tile] + atomicAdd(&rs.tileFill[tile], 1);
                if (pos < rs.binCap) rs.binTri[pos] = i;
            }
        }
    }
}

// Exclusive scan of the tile counts: one CTA walks the array in coalesced
// chunks of 1024, scanning each chunk with warp shuffles and carrying the total.
__global__ void __launch_bounds__(1024) k_bin_scan(RasterScratch rs, int tiles)
{
    if (large_direct(rs)) return;  // uniform across the block
    // Each thread scans kScanPer consecutive tiles in registers, so one pass of
    // the block covers 16,384 tiles (a 2048^2 map) with one block-wide scan.
    constexpr int kScanPer = 16;
    __shared__ long long warpSum[32];
    __shared__ long long carry;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < tiles; base += 1024 * kScanPer)
    {
        const int i0 = base + tid * kScanPer;
        int v[kScanPer];
        if (i0 + kScanPer <= tiles)
        {
            const int4* src = reinterpret_cast<const int4*>(rs.tileCount + i0);  // 64-byte aligned
#pragma unroll
            for (int q = 0; q < kScanPer / 4; ++q)
            {
                const int4 w = src[q];
                v[4 * q] = w.x, v[4 * q + 1] = w.y, v[4 * q + 2] = w.z, v[4 * q + 3] = w.w;
            }
        }
        else
        {
#pragma unroll
            for (int k = 0; k < kScanPer; ++k) v[k] = i0 + k < tiles ? rs.tileCount[i0 + k] : 0;
        }
        long long local = 0;
#pragma unroll
        for (int k = 0; k < kScanPer; ++k) local += v[k];
        long long x = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warpSum[wid] = x;
        __syncthreads();
        if (wid == 0)
        {
            long long w = warpSum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warpSum[lane] = w;  // inclusive
        }
        __syncthreads();
        long long run = carry + (wid ? warpSum[wid - 1] : 0) + (x - local);
        if (i0 + kScanPer <= tiles)
        {
            int st[kScanPer];
#pragma unroll
            for (int k = 0; k < kScanPer; ++k)
            {
                st[k] = (int)min(run, (long long)0x7fffffff);
                run += v[k];
            }
            int4* dst = reinterpret_cast<int4*>(rs.tileStart + i0);
            int4* fill = reinterpret_cast<int4*>(rs.tileFill + i0);
#pragma unroll
            for (int q = 0; q < kScanPer / 4; ++q)
            {
                dst[q] = make_int4(st[4 * q], st[4 * q + 1], st[4 * q + 2], st[4 * q + 3]);
                fill[q] = make_int4(0, 0, 0, 0);
            }
        }
        else
        {
            for (int k = 0; k < kScanPer && i0 + k < tiles; ++k)
            {
                rs.tileStart[i0 + k] = (int)min(run, (long long)0x7fffffff);
                rs.tileFill[i0 + k] = 0;
                run += v[k];
            }
        }
        __syncthreads();
        if (tid == 0) carry += warpSum[31];
        __syncthreads();
    }
    if (tid == 0)
    {
        long long total = carry;
        rs.tileStart[tiles] = (int)min(total, (long long)0x7fffffff);
        rs.counters[2] = (int)min(total, (long long)0x7fffffff);
        if (total > rs.binCap) atomicOr(&rs.counters[3], kStatusBinOverflow);
    }
}

// One CTA per 16 x 16 tile: the tile's triangles are staged in shared memory
// in batches, each thread keeps the minimum key of its pixel in a register and
// publishes it once. The body is shared by the single-view launch (one CTA per
// tile) and the persistent multi-view launch ((view, tile) work queue).
constexpr int kTileBatch = 64;

template <int CAP>
__device__ __forceinline__ void tile_raster_body(const RasterParams& rp, const RasterScratch& rs, int tile,
                                                 frx::RTri* sh, int* shIdx, int4* shBox)
{
    const bool direct = large_direct(rs);
    long long start = direct ? 0 : rs.tileStart[tile];
    long long end = direct ? min(rs.counters[1], rs.triCap) : min((long long)rs.tileStart[tile + 1], rs.binCap);
    if (start >= end) return;  // uniform across the CTA
    int ntx = (rp.W + kTile - 1) / kTile;
    int px = (tile % ntx) * kTile + (threadIdx.x & 15);
    int py = (tile / ntx) * kTile + (threadIdx.x >> 4);
    bool inside = px < rp.W && py < rp.H;
    unsigned long long best = frx::kEmptyKey;
    for (long long base = start; base < end; base += CAP)
    {
        int cnt = (int)min((long long)CAP, end - base);
        for (int i = threadIdx.x; i < cnt; i += blockDim.x)
        {
            int li = direct ? (int)(base + i) : rs.binTri[base + i];
            frx::RTri r = rs.largeTris[li];
            sh[i] = r;
            shIdx[i] = rs.largeIdx[li];
            int x0, x1, y0, y1;
            bbox(r, rp.W, rp.H, x0, x1, y0, y1);
            shBox[i] = make_int4(x0, x1, y0, y1);
        }
        __syncthreads();
        // every thread runs the loop so the warp-wide ballot sees full warps
        for (int j = 0; j < cnt; ++j)
        {
            int4 bb = shBox[j];
            bool inb = inside && px >= bb.x && px <= bb.y && py >= bb.z && py <= bb.w;
            if (__ballot_sync(0xffffffffu, inb) == 0u) continue;
            if (!inb) continue;
            float b0, b1, b2;
            if (!frx::bary<0, false>(sh[j], px, py, b0, b1, b2)) continue;
            float d = frx::depth_of(sh[j], b0, b1, b2);
            if (!frx::depth_passes_clear(d)) continue;
            unsigned long long key = frx::make_key(d, (unsigned)shIdx[j]);
            best = key < best ? key : best;
        }
        __syncthreads();
    }
    if (inside && best != frx::kEmptyKey) atomicMin(rs.keys + (size_t)py * rp.W + px, best);
}

__global__ void __launch_bounds__(256) k_tile_raster(RasterParams rp, RasterScratch rs)
{
    __shared__ frx::RTri sh[kTileBatch];
    __shared__ int shIdx[kTileBatch];
    __shared__ int4 shBox[kTileBatch];
    tile_raster_body<kTileBatch>(rp, rs, blockIdx.x, sh, shIdx, shBox);
}

// Shadow-map value of texel p from its visibility key: the winning triangle's
// interpolated NDC z mapped to [0, 1] (render.cpp:83-93), 0 where nothing covers it.
// rec: the pass's resolve records, or null.
__device__ __forceinline__ float shadow_texel(const DevScene& S, const int4* __restrict__ scrL,
                                              const int4* __restrict__ rec, unsigned long long key, int px, int py)
{
    float out = 0.f;
    if (key != frx::kEmptyKey)
    {
        int t = (int)(key & 0xffffffffu);
        if (rec)
        {
            frx::RTri r;
            int4 wv;
            if (load_tri_record(rec, t, r, wv))
            {
                float b0, b1, b2;
                if (frx::bary<0, false>(r, px, py, b0, b1, b2))
                    out = interp(__int_as_float(wv.x), __int_as_float(wv.y), __int_as_float(wv.z), b0, b1, b2) * 0.5f +
                          0.5f;
                return out;
            }
        }
        int4 tv = S.triV[t];
        frx::RTri r;
        load_rtri(scrL, tv, r, false);
        float b0, b1, b2;
        if (frx::bary<0, false>(r, px, py, b0, b1, b2))
        {
            float z = interp(__int_as_float(scrL[tv.x].w), __int_as_float(scrL[tv.y].w),
                             __int_as_float(scrL[tv.z].w), b0, b1, b2);
            out = z * 0.5f + 0.5f;
        }
    }
    return out;
}

// The shadow pass's fine raster with the shadow-map resolve fused in. The setup
// and medium passes ran before, and no other CTA touches this tile, so each
// thread reads its texel's key once up front and resolves it at once (the
// winner among the small and medium triangles: its vertex gathers overlap the
// tile's staging), keeps the minimum with the tile's binned triangles in a
// register and writes it back with a plain store. A texel won by a binned
// triangle takes its shadow value from the weights of the winning evaluation
// (the bary() the resolve would repeat) and the vertices' NDC z staged beside
// the triangle.
__global__ void __launch_bounds__(256, 5) k_tile_raster_shadow(RasterParams rp, RasterScratch rs, DevScene S,
                                                            const int4* __restrict__ scrL, float* __restrict__ shadow)
{
    __shared__ frx::RTri sh[kTileBatch];
    __shared__ int shIdx[kTileBatch];
    __shared__ int4 shBox[kTileBatch];
    __shared__ float4 shZ[kTileBatch];
    const int tile = blockIdx.x;
    const int ntx = (rp.W + kTile - 1) / kTile;
    const int px = (tile % ntx) * kTile + (threadIdx.x & 15);
    const int py = (tile / ntx) * kTile + (threadIdx.x >> 4);
    const bool inside = px < rp.W && py < rp.H;
    const size_t p = inside ? (size_t)py * rp.W + px : 0;
    const unsigned long long k0 = inside ? __ldcg(rs.keys + p) : frx::kEmptyKey;
    const float out0 = shadow_texel(S, scrL, rs.triRec, k0, px, py);
    unsigned long long best = k0;
    float w0 = 0.f, w1 = 0.f, w2 = 0.f;
    float4 wz = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool direct = large_direct(rs);
    const long long start = direct ? 0 : rs.tileStart[tile];
    const long long end = direct ? min(rs.counters[1], rs.triCap) : min((long long)rs.tileStart[tile + 1], rs.binCap);
    for (long long base = start; base < end; base += kTileBatch)
    {
        const int cnt = (int)min((long long)kTileBatch, end - base);
        for (int i = threadIdx.x; i < cnt; i += blockDim.x)
        {
            const int li = direct ? (int)(base + i) : rs.binTri[base + i];
            const frx::RTri r = rs.largeTris[li];
            sh[i] = r;
            shIdx[i] = rs.largeIdx[li];
            shZ[i] = rs.largeAux[li];
            int x0, x1, y0, y1;
            bbox(r, rp.W, rp.H, x0, x1, y0, y1);
            shBox[i] = make_int4(x0, x1, y0, y1);
        }
        __syncthreads();
        // every thread runs the loop so the warp-wide ballot sees full warps
        for (int j = 0; j < cnt; ++j)
        {
            const int4 bb = shBox[j];
            const bool inb = inside && px >= bb.x && px <= bb.y && py >= bb.z && py <= bb.w;
            if (__ballot_sync(0xffffffffu, inb) == 0u) continue;
            if (!inb) continue;
            float b0, b1, b2;
            if (!frx::bary<0, false>(sh[j], px, py, b0, b1, b2)) continue;
            const float d = frx::depth_of(sh[j], b0, b1, b2);
            if (!frx::depth_passes_clear(d)) continue;
            const unsigned long long key = frx::make_key(d, (unsigned)shIdx[j]);
            if (key < best)
            {
                best = key;
                w0 = b0, w1 = b1, w2 = b2;
                wz = shZ[j];
            }
        }
        __syncthreads();
    }
    if (!inside) return;
    if (best != k0)
    {
        rs.keys[p] = best;
        shadow[p] = interp(wz.x, wz.y, wz.z, w0, w1, w2) * 0.5f + 0.5f;
    }
    else
        shadow[p] = out0;
}

// Index of the work-queue entry holding item `it`: the last e with start[e] <= it.
__device__ __forceinline__ int queue_entry(const int* __restrict__ start, int n, int it)
{
    int lo = 0, hi = n - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= it) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Persistent fine raster of many views (camera views and shadow maps): CTAs
// take (view, tile) items from one atomic queue until it runs dry. CAP
// triangles are staged in shared memory per batch.
template <int CAP>
__global__ void __launch_bounds__(256) k_tile_raster_views(const ViewRaster* __restrict__ vr,
                                                           const int* __restrict__ itemStart, int nEntries, int total,
                                                           int* __restrict__ queue)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    frx::RTri* sh = reinterpret_cast<frx::RTri*>(dsm);
    int* shIdx = reinterpret_cast<int*>(sh + CAP);
    int4* shBox = reinterpret_cast<int4*>(shIdx + CAP);
    __shared__ int sItem, sEntry;
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            int it = atomicAdd(queue, 1);
            sItem = it;
            sEntry = it < total ? queue_entry(itemStart, nEntries, it) : 0;
        }
        __syncthreads();
        const int it = sItem;
        if (it >= total) break;
        const int e = sEntry;
        const RasterParams rp = vr[e].rp;
        const RasterScratch rs = vr[e].rs;
        tile_raster_body<CAP>(rp, rs, it - itemStart[e], sh, shIdx, shBox);
        __syncthreads();  // sItem is rewritten next
    }
}

// ---- fragment inputs (gshader.h:95-143) --------------------------------------------------
struct FragIn
{
    F3 pos, normal, lndc;
    float u, v;
    int material, model;
};

__device__ __forceinline__ F3 ld3(float4 a) { return F3{a.x, a.y, a.z}; }

__device__ bool fragment_inputs(const DevScene& S, const FrameConst& F, const VertexOut& vo, int t, int px,
                                int py, FragIn& f)
{
    int4 tv = S.triV[t], tt = S.triT[t], tn = S.triN[t];
    frx::RTri r;
    load_rtri(vo.scr, tv, r, false);
    float b0, b1, b2;
    if (!frx::bary<0, false>(r, px, py, b0, b1, b2)) return false;
    f.material = tt.w;
    f.model = tn.w;
    float4 A0 = vo.pw[tv.x], A1 = vo.pw[tv.y], A2 = vo.pw[tv.z];
    float2 T0 = S.uv[tt.x], T1 = S.uv[tt.y], T2 = S.uv[tt.z];
    float4 N0 = vo.npre[tn.x], N1 = vo.npre[tn.y], N2 = vo.npre[tn.z];
    // per-corner varyings of the vertex stage (texCoord *= ow, normalWS *= ow)
    float u0 = T0.x * A0.w, v0 = T0.y * A0.w, u1 = T1.x * A1.w, v1 = T1.y * A1.w;
    float u2 = T2.x * A2.w, v2 = T2.y * A2.w;
    F3 n0 = ld3(N0) * A0.w, n1 = ld3(N1) * A1.w, n2 = ld3(N2) * A2.w;
    F3 pos{interp(A0.x, A1.x, A2.x, b0, b1, b2), interp(A0.y, A1.y, A2.y, b0, b1, b2),
           interp(A0.z, A1.z, A2.z, b0, b1, b2)};
    float u = interp(u0, u1, u2, b0, b1, b2), v = interp(v0, v1, v2, b0, b1, b2);
    F3 n{interp(n0.x, n1.x, n2.x, b0, b1, b2), interp(n0.y, n1.y, n2.y, b0, b1, b2),
         interp(n0.z, n1.z, n2.z, b0, b1, b2)};
    float w = 1.f / interp(A0.w, A1.w, A2.w, b0, b1, b2);
    pos = pos * w;
    u = u * w;
    v = v * w;
    n = n * w;
    F3 N = normalize(n);
    F3 normal = N;
    const DevMaterial& mat = S.materials[f.material];
    if (S.models[f.model].has_tangents && mat.map_bump >= 0)
    {
        float4 G0 = vo.tw[tv.x], G1 = vo.tw[tv.y], G2 = vo.tw[tv.z];
        F3 tg{interp(G0.x, G1.x, G2.x, b0, b1, b2), interp(G0.y, G1.y, G2.y, b0, b1, b2),
              interp(G0.z, G1.z, G2.z, b0, b1, b2)};
        tg = tg * w;
        F3 Tn = normalize(tg + f3(0.001f));
        Tn = normalize(Tn - N * dot(Tn, N));
        F3 B = normalize(cross(N, Tn));
        float tbn[9] = {Tn.x, B.x, N.x, Tn.y, B.y, N.y, Tn.z, B.z, N.z};
        F3 s = tex_sample(S, mat.map_bump, u, v);
        s = normalize(s * 2.f - f3(1.f));
        normal = normalize(mul3(tbn, s));
    }
    F3 l{0.f, 0.f, 0.f};
    if (F.shadowOn)
    {
        float4 L0 = vo.lw[tv.x], L1 = vo.lw[tv.y], L2 = vo.lw[tv.z];
        l = F3{interp(L0.x, L1.x, L2.x, b0, b1, b2), interp(L0.y, L1.y, L2.y, b0, b1, b2),
               interp(L0.z, L1.z, L2.z, b0, b1, b2)};
        l = l * w;
    }
    f.pos = pos;
    f.normal = normal;
    f.lndc = l;
    f.u = u;
    f.v = v;
    return true;
}

__device__ __forceinline__ unsigned pack_rgb(unsigned r, unsigned g, unsigned b) { return r | (g << 8) | (b << 16); }

// ---- resolves --------------------------------------------------------------------------------

// DepthShader::ProcessFragment (depthshader.h:30-36) of the surviving triangle.
__global__ void k_resolve_shadow(DevScene S, const int4* __restrict__ scrL, const unsigned long long* __restrict__ keys,
                                 int SW, int SH, float* __restrict__ shadow)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= SW * SH) return;
    shadow[p] = shadow_texel(S, scrL, nullptr, keys[p], p % SW, p / SW);
}

// GShader::ProcessFragment (gshader.h:95-202) of the surviving triangle, into the
// packed G-buffer; background pixels get the cleared values (forkergl.cpp:70-81).
__global__ void k_resolve_gbuffer(DevScene S, FrameConst F, VertexOut vo, const unsigned long long* __restrict__ keys,
                                  GBuffer gb)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= F.W * F.H) return;
    unsigned long long key = keys[p];
    FragIn f;
    if (key == frx::kEmptyKey || !fragment_inputs(S, F, vo, (int)(key & 0xffffffffu), p % F.W, p / F.W, f))
    {
        gb.a[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        gb.b[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        gb.c[p] = make_uint4(0u, 0u, 0u, 0u);
        gb.depth[p] = FLT_MAX;
        gb.ao[p] = 1.f;
        return;
    }
    const DevMaterial& mat = S.materials[f.material];
    gb.a[p] = make_float4(f.pos.x, f.pos.y, f.pos.z, f.lndc.x);
    gb.b[p] = make_float4(f.normal.x, f.normal.y, f.normal.z, f.lndc.y);
    gb.depth[p] = frx::key_depth(key);
    gb.ao[p] = 1.f;
    if (S.texLinear)
    {
        // bilinear texels are not bytes: keep the texture coordinate, decode_gbuffer samples
        unsigned flags = kGCovered;
        if (mat.map_kd >= 0) flags |= kGAlbedoMap;
        if (mat.map_ke >= 0) flags |= kGEmissiveMap;
        if (S.models[f.model].support_pbr)
        {
            flags |= kGPbr;
            if (mat.map_ao >= 0) flags |= kGP0Map;
            if (mat.map_pm >= 0) flags |= kGP1Map;
            if (mat.map_pr >= 0) flags |= kGP2Map;
        }
        else if (mat.map_ks >= 0)
            flags |= kGP2Map;
        gb.c[p] = make_uint4(__float_as_uint(f.lndc.z), ((unsigned)f.material & 0xffffffu) | (flags << 24),
                             __float_as_uint(f.u), __float_as_uint(f.v));
        return;
    }
    unsigned flags = kGCovered, alb = 0, emi = 0, p0 = 0, p1 = 0, p2 = 0, r8, g8, b8;
    if (mat.map_kd >= 0)
    {
        texel_rgb(S, mat.map_kd, f.u, f.v, r8, g8, b8);
        alb = pack_rgb(r8, g8, b8);
        flags |= kGAlbedoMap;
    }
    if (mat.map_ke >= 0)
    {
        texel_rgb(S, mat.map_ke, f.u, f.v, r8, g8, b8);
        emi = pack_rgb(r8, g8, b8);
        flags |= kGEmissiveMap;
    }
    if (S.models[f.model].support_pbr)
    {
        flags |= kGPbr;
        if (mat.map_ao >= 0)
        {
            texel_rgb(S, mat.map_ao, f.u, f.v, r8, g8, b8);
            p0 = b8;
            flags |= kGP0Map;
        }
        if (mat.map_pm >= 0)
        {
            texel_rgb(S, mat.map_pm, f.u, f.v, r8, g8, b8);
            p1 = b8;
            flags |= kGP1Map;
        }
        if (mat.map_pr >= 0)
        {
            texel_rgb(S, mat.map_pr, f.u, f.v, r8, g8, b8);
            p2 = b8;
            flags |= kGP2Map;
        }
    }
    else if (mat.map_ks >= 0)
    {
        texel_rgb(S, mat.map_ks, f.u, f.v, r8, g8, b8);
        p2 = b8;
        flags |= kGP2Map;
    }
    unsigned m = (unsigned)f.material;
    gb.c[p] = make_uint4(__float_as_uint(f.lndc.z), alb | (flags << 24), p0 | (p1 << 8) | (p2 << 16) | ((m & 0xffu) << 24),
                         emi | (((m >> 8) & 0xffu) << 24));
}

// The frame's 8 raster counters and status words into host memory the device
// can address (both raster passes are done when the frame's shading runs), so
// the host reads them after the frame's last event without a copy of its own.
__device__ __forceinline__ void publish_status(const int* __restrict__ counters, int* __restrict__ statusOut)
{
    if (statusOut && blockIdx.x == 0 && threadIdx.x < 8) statusOut[threadIdx.x] = counters[threadIdx.x];
}

// ForkerGL::DrawScreenSpacePixels (forkergl.cpp:326-380) for one pixel.
template <bool kLinear>
__global__ void k_lighting(DevScene S, FrameConst F, GBuffer gb, const float* __restrict__ shadow,
                           unsigned* __restrict__ frame8, float* __restrict__ frameF, const int* __restrict__ counters,
                           int* __restrict__ statusOut)
{
    publish_status(counters, statusOut);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= F.W * F.H) return;
    uint4 C = gb.c[p];
    if (F.bgBlack && !((C.y >> 24) & kGCovered))
    {
        // zero G-buffer: albedo, emissive, ks and shininess 0 make every term of
        // the Blinn-Phong sum exactly 0 (pow(0, 0) = 1 times ks = 0), so the
        // reference's result is black
        frame8[p] = 0u;
        if (frameF) frameF[3 * (size_t)p] = frameF[3 * (size_t)p + 1] = frameF[3 * (size_t)p + 2] = 0.f;
        return;
    }
    float4 A = gb.a[p], B = gb.b[p];
    GDecoded g = decode_gbuffer_t<kLinear>(S, C);
    F3 pos = ld3(A), n = ld3(B), l{A.w, B.w, __uint_as_float(C.x)};
    F3 param = g.param;
    param.x *= gb.ao[p];
    F3 eye{F.eye[0], F.eye[1], F.eye[2]}, lp{F.lightPos[0], F.lightPos[1], F.lightPos[2]};
    F3 lc{F.lightColor[0], F.lightColor[1], F.lightColor[2]};
    F3 L = normalize(lp - pos);
    F3 Vd = normalize(eye - pos);
    float vis = 0.f;
    if (F.shadowOn) vis = shadow_visibility(F, shadow, l, n, L);
    F3 c;
    if (g.type < 0.5f) c = blinn_phong_lin(F.shadowOn, L, Vd, n, vis, g.albedoLin, g.emissiveLin, param, lc);
    else c = pbr_lin(F.shadowOn, L, Vd, normalize(L + Vd), n, vis, g.albedoLin, g.emissiveLin, param, lc);
    frame8[p] = quantize_rgb(c);
    if (frameF)
    {
        frameF[3 * (size_t)p] = c.x;
        frameF[3 * (size_t)p + 1] = c.y;
        frameF[3 * (size_t)p + 2] = c.z;
    }
}

// Shade one pixel of a batch view with the batch's lights (PBR: the lights'
// direct terms summed, then ambient / emission / tone mapping once; with one
// light this is exactly k_lighting's arithmetic).
template <bool kLinear>
__device__ __forceinline__ unsigned shade_batch_pixel(const DevScene& S, const ViewShade& VS, int p,
                                                      const BatchLight* __restrict__ lights, int nLights)
{
    const FrameConst& F = VS.F;
    const uint4 C = VS.gb.c[p];
    if (!((C.y >> 24) & kGCovered)) return 0u;  // background: black, as the reference's lit frame
    const float4 A = VS.gb.a[p], B = VS.gb.b[p];
    GDecoded g = decode_gbuffer_t<kLinear>(S, C);
    const F3 pos = ld3(A), n = ld3(B), lg{A.w, B.w, __uint_as_float(C.x)};
    F3 param = g.param;
    param.x *= VS.gb.ao[p];
    const F3 eye{F.eye[0], F.eye[1], F.eye[2]};
    const F3 Vd = normalize(eye - pos);
    const bool pbrMat = g.type >= 0.5f;
    F3 Lo{0.f, 0.f, 0.f}, al{0.f, 0.f, 0.f}, el{0.f, 0.f, 0.f}, c;
    if (pbrMat)
    {
        al = g.albedoLin;
        el = g.emissiveLin;
    }
    for (int k = 0; k < nLights; ++k)
    {
        const BatchLight& Lk = lights[k];
        const F3 lc{Lk.color[0], Lk.color[1], Lk.color[2]};
        F3 L;
        if (Lk.type == 0) L = normalize(F3{Lk.pos[0], Lk.pos[1], Lk.pos[2]} - pos);
        else L = F3{-Lk.dir[0], -Lk.dir[1], -Lk.dir[2]};
        float vis = 0.f;
        if (F.shadowOn)
        {
            F3 l = lg;
            if (k != VS.ndcLight)
            {
                const F4 q = mul4(Lk.S.L, F4{pos.x, pos.y, pos.z, 1.f});
                l = F3{q.x / q.w, q.y / q.w, q.z / q.w};
            }
            vis = shadow_visibility(Lk.S, Lk.shadow, l, n, L);
        }
        if (pbrMat)
        {
            const F3 d = pbr_direct(F.shadowOn, L, Vd, normalize(L + Vd), n, vis, al, param.y, param.z, lc);
            Lo = (k == 0) ? d : Lo + d;
        }
        else if (k == 0)
            c = blinn_phong_lin(F.shadowOn, L, Vd, n, vis, g.albedoLin, g.emissiveLin, param, lc);
    }
    if (pbrMat) c = pbr_finish(Lo, al, el, param.x);
    return quantize_rgb(c);
}

template <int T, bool kLinear>
__global__ void __launch_bounds__(256) k_lighting_views(DevScene S, const ViewShade* __restrict__ views,
                                                        const int* __restrict__ itemStart, int nViews, int total,
                                                        const BatchLight* __restrict__ lights, int nLights,
                                                        int* __restrict__ queue)
{
    __shared__ int sItem, sView;
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            int it = atomicAdd(queue, 1);
            sItem = it;
            sView = it < total ? queue_entry(itemStart, nViews, it) : 0;
        }
        __syncthreads();
        const int it = sItem;
        if (it >= total) break;
        const ViewShade& VS = views[sView];
        const int W = VS.F.W, H = VS.F.H;
        const int tile = it - itemStart[sView];
        const int ntx = (W + T - 1) / T;
        const int x0 = (tile % ntx) * T, y0 = (tile / ntx) * T;
        for (int k = threadIdx.x; k < T * T; k += blockDim.x)
        {
            const int px = x0 + k % T, py = y0 + k / T;
            if (px < W && py < H)
            {
                const int p = py * W + px;
                VS.frame8[p] = shade_batch_pixel<kLinear>(S, VS, p, lights, nLights);
            }
        }
        __syncthreads();
    }
}

// Forward pass (render.cpp:99-157): the surviving fragment's Blinn-Phong or PBR
// shading (phongshader.h:292-371, pbrshader.h:90-180); ClearColor elsewhere.
__global__ void k_forward_shade(DevScene S, FrameConst F, VertexOut vo, const unsigned long long* __restrict__ keys,
                                const float* __restrict__ shadow, float* __restrict__ depth,
                                unsigned* __restrict__ frame8, float* __restrict__ frameF,
                                const int* __restrict__ counters, int* __restrict__ statusOut)
{
    publish_status(counters, statusOut);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= F.W * F.H) return;
    unsigned long long key = keys[p];
    F3 c = f3(0.12f);
    FragIn f;
    if (key != frx::kEmptyKey && fragment_inputs(S, F, vo, (int)(key & 0xffffffffu), p % F.W, p / F.W, f))
    {
        depth[p] = frx::key_depth(key);
        const DevMaterial& mat = S.materials[f.material];
        F3 eye{F.eye[0], F.eye[1], F.eye[2]}, lp{F.lightPos[0], F.lightPos[1], F.lightPos[2]};
        F3 lc{F.lightColor[0], F.lightColor[1], F.lightColor[2]};
        F3 L = normalize(lp - f.pos);
        F3 Vd = normalize(eye - f.pos);
        F3 Hd = normalize(L + Vd);
        float vis = 0.f;
        if (F.shadowOn) vis = shadow_visibility(F, shadow, f.lndc, f.normal, L);
        F3 emissive = F3{mat.ke[0], mat.ke[1], mat.ke[2]};
        if (mat.map_ke >= 0) emissive = tex_sample(S, mat.map_ke, f.u, f.v);
        if (!S.models[f.model].support_pbr)
        {
            F3 diffuse = F3{mat.kd[0], mat.kd[1], mat.kd[2]};
            if (mat.map_kd >= 0) diffuse = tex_sample(S, mat.map_kd, f.u, f.v);
            float shin = 1.f;
            if (mat.map_ks >= 0) shin = tex_sample_float(S, mat.map_ks, f.u, f.v) + 5;
            c = blinn_phong(F.shadowOn, L, Hd, f.normal, vis, diffuse, emissive, F3{mat.ka[0], mat.ks[0], shin}, lc);
        }
        else
        {
            F3 albedo = F3{mat.pbr_albedo[0], mat.pbr_albedo[1], mat.pbr_albedo[2]};
            if (mat.map_kd >= 0) albedo = tex_sample(S, mat.map_kd, f.u, f.v);
            float rough = mat.roughness, metal = mat.metalness, ao = 1.f;
            if (mat.map_pr >= 0) rough = tex_sample_float(S, mat.map_pr, f.u, f.v);
            if (mat.map_pm >= 0) metal = tex_sample_float(S, mat.map_pm, f.u, f.v);
            if (mat.map_ao >= 0) ao = tex_sample_float(S, mat.map_ao, f.u, f.v);
            c = pbr(F.shadowOn, L, Vd, Hd, f.normal, vis, albedo, emissive, F3{ao, metal, rough}, lc);
        }
    }
    else
    {
        depth[p] = FLT_MAX;
    }
    frame8[p] = quantize_rgb(c);
    if (frameF)
    {
        frameF[3 * (size_t)p] = c.x;
        frameF[3 * (size_t)p + 1] = c.y;
        frameF[3 * (size_t)p + 2] = c.z;
    }
}

// ---- SSAO (render.cpp:214-286) ---------------------------------------------------------------
// Per sample the reference draws a unit-ball vector k, flips it into the normal's
// hemisphere, scales it by Lerp(0.1, 1, |k|^2) and by the radius, projects the
// offset point and compares depths. Length, Lerp and both scalings depend on k
// only (|-k| == |k| and negation commutes with rounding), so each CTA first
// builds, for the 16 noise-cell kernels, the table (k, (k * sc) * radius) in
// shared memory with the reference's operations (two 16-byte entries per sample,
// cells padded apart so the four cells a warp row touches use distinct banks).
//
// Background pixels (no triangle) have a zero position and normal and the
// cleared depth, so their result depends on the noise cell only: the 16 values
// are computed once per frame (k_ssao_background) and copied.
// Entry e = cell * N + s of the table: the kernel vector k and its offset (k * sc) * radius.
__device__ __forceinline__ void ssao_kernel_offset(const FrameConst& F, const float* __restrict__ table, int e, F3& k,
                                                   F3& o)
{
    k = F3{table[3 * e], table[3 * e + 1], table[3 * e + 2]};
    float sc = length(k);
    sc = (1 - 0.1f) * 1.0f + 0.1f * (sc * sc);  // Lerp(0.1f, 1.0f, sc * sc) (utility.h:26-29)
    o = (k * sc) * F.ssaoRadius;
}

__device__ __forceinline__ void ssao_build_table(const FrameConst& F, const float* __restrict__ table, float4* tbl,
                                                 int stride)
{
    const int N = F.ssaoN;
    for (int e = threadIdx.x; e < 16 * N; e += blockDim.x)
    {
        F3 k, o;
        ssao_kernel_offset(F, table, e, k, o);
        int cell = e / N, s = e % N;
        tbl[cell * stride + 2 * s] = make_float4(k.x, k.y, k.z, 0.f);
        tbl[cell * stride + 2 * s + 1] = make_float4(o.x, o.y, o.z, 0.f);
    }
}

// The depth the reference's SSAO reads for pixel (ix, iy) of the depth buffer.
__device__ __forceinline__ float ssao_cached(const FrameConst& F, const float* __restrict__ depth, int ix, int iy)
{
    if ((unsigned)ix < (unsigned)F.W && (unsigned)iy < (unsigned)F.H) return __ldg(depth + (iy * F.W + ix));
    // unchecked DepthBuffer.GetValue(x, y) (render.cpp:255): the linear index
    // reads wherever it lands inside the buffer; outside, nothing occludes
    const long long li = (long long)ix + (long long)iy * F.W;
    return (li >= 0 && li < (long long)F.W * F.H) ? __ldg(depth + li) : FLT_MAX;
}

// The flip of a kernel vector into the normal's hemisphere (render.cpp:244-246):
// +1 when Dot(k, n) > 0, else -1 (the leading "0 +" of the Dot cannot change the sign).
__device__ __forceinline__ float ssao_flip(float4 kk, F3 nrm)
{
    return (kk.x * nrm.x + kk.y * nrm.y) + kk.z * nrm.z > 0.f ? 1.f : -1.f;
}

// One SSAO sample (render.cpp:240-277): 1 when it occludes (depth test and range
// check pass), else 0; the reference adds kernelScale * this (adding kernelScale
// * 0 = +0 to a non-negative sum is exact, so the caller may always add). Every
// value is used only through a sign test, a float->int truncation or a
// comparison, none of which can see the sign of a zero, so the leading "0 +" of
// each Dot is dropped; all other operations and roundings are the reference's
// (frx::ssao_project).
__device__ __forceinline__ float ssao_sample(const FrameConst& F, const float* __restrict__ depth, float4 kk,
                                             float4 oo, F3 pos, F3 nrm, float fragDepth)
{
    const frx::SsaoProj q = frx::ssao_project(F.VP, F.VPort, F.vportSimple != 0, pos.x, pos.y, pos.z,
                                              ssao_flip(kk, nrm), oo.x, oo.y, oo.z);
    const float cached = ssao_cached(F, depth, frx::f2i_sat(q.x), frx::f2i_sat(q.y));
    if (q.z >= cached + F.ssaoBias) return fabsf(fragDepth - cached) < F.ssaoRange ? 1.f : 0.f;
    return 0.f;
}

__device__ __forceinline__ float ssao_result(const FrameConst& F, int hits)
{
    // The reference adds kernelScale * rangeCheck per sample in order
    // (render.cpp:262-268). A sample that does not occlude adds +0 to a
    // non-negative sum, which leaves it unchanged, so the sum is kernelScale
    // added once per occluding sample, whichever they are: count them, then add.
    const float kernelScale = 1.f / F.ssaoN;
    float occ = 0.f;
    for (int i = 0; i < hits; ++i) occ += kernelScale;
    occ = 1.f - occ;
    return powf(occ, 3.f);
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The frame kernel's table: per (cell, sample) three float4: (k, Q.w), (Q.xyz, 0),
// (o, 0), with o built as in ssao_build_table and Q = VP (o, 0) (frx::ssao_q).
// Cells are 3N + 1 float4 apart: the four cells a warp row reads start 4 banks apart.
__host__ __device__ constexpr int ssao_q_stride(int N) { return 3 * N + 1; }
__device__ __forceinline__ void ssao_build_table_q(const FrameConst& F, const float* __restrict__ table, float4* tbl,
                                                   int stride)
{
    const int N = F.ssaoN;
    for (int e = threadIdx.x; e < 16 * N; e += blockDim.x)
    {
        F3 k, o;
        ssao_kernel_offset(F, table, e, k, o);
        float Q[4];
        frx::ssao_q(F.VP, o.x, o.y, o.z, Q);
        int cell = e / N, s = e % N;
        tbl[cell * stride + 3 * s] = make_float4(k.x, k.y, k.z, Q[3]);
        tbl[cell * stride + 3 * s + 1] = make_float4(Q[0], Q[1], Q[2], 0.f);
        tbl[cell * stride + 3 * s + 2] = make_float4(o.x, o.y, o.z, 0.f);
    }
}

// One pixel's SSAO through the estimate (frx::ssao_plane): a sample whose
// estimated pixel and depth comparison lie outside the error bound of every
// rounding boundary is decided by the estimate; the others (about 1 % on the
// benchmark frame) are marked and evaluated exactly afterwards. The result is
// the exact path's for every sample.
__device__ __forceinline__ float ssao_pixel_filtered(const FrameConst& F, const float* __restrict__ depth,
                                                     const float4* k, F3 pos, F3 nrm, float fragDepth)
{
    const frx::SsaoPlane q = frx::ssao_plane(F.VP, F.VPort, F.vportSimple != 0, F.ssaoRadius, pos.x, pos.y, pos.z);
    const int N = F.ssaoN;
    int hits = 0;
    if (!q.ok)
    {
        for (int s = 0; s < N; ++s) hits += ssao_sample(F, depth, k[3 * s], k[3 * s + 2], pos, nrm, fragDepth) > 0.f;
        return ssao_result(F, hits);
    }
    const float V0 = F.VPort[0], V3 = F.VPort[3], V5 = F.VPort[5], V7 = F.VPort[7], V10 = F.VPort[10],
                V11 = F.VPort[11];
    // one sample by the estimate: adds its hit when decided, else marks it
    auto fast = [&](int s, unsigned bit, unsigned& unsure) {
        const float4 kq = k[3 * s], qq = k[3 * s + 1];
        const float sg = ssao_flip(kq, nrm);
        const float r = rcp_approx(__fmaf_rn(sg, kq.w, q.P[3]));
        const float ex = __fmaf_rn(V0, __fmul_rn(__fmaf_rn(sg, qq.x, q.P[0]), r), V3);
        const float ey = __fmaf_rn(V5, __fmul_rn(__fmaf_rn(sg, qq.y, q.P[1]), r), V7);
        const float ez = __fmaf_rn(V10, __fmul_rn(__fmaf_rn(sg, qq.z, q.P[2]), r), V11);
        const int ix = frx::f2i_sat(ex - q.dx), iy = frx::f2i_sat(ey - q.dy);
        const bool xyok = (ix == frx::f2i_sat(ex + q.dx)) & (iy == frx::f2i_sat(ey + q.dy));
        const float cached = ssao_cached(F, depth, ix, iy);
        const float thr = cached + F.ssaoBias;
        const bool above = ez - q.dz >= thr, below = ez + q.dz < thr;
        const bool sure = xyok & (above | below);
        hits += (int)(sure & above & (fabsf(fragDepth - cached) < F.ssaoRange));
        unsure |= sure ? 0u : bit;
    };
    for (int base = 0; base < N; base += 32)
    {
        unsigned unsure = 0u;
        const int cnt = min(32, N - base);
        if (cnt == 32)
        {
#pragma unroll 2
            for (int j = 0; j < 32; ++j) fast(base + j, 1u << j, unsure);
        }
        else if (cnt == 16)  // the learned-AO input's sample count
        {
#pragma unroll 2
            for (int j = 0; j < 16; ++j) fast(base + j, 1u << j, unsure);
        }
        else
            for (int j = 0; j < cnt; ++j) fast(base + j, 1u << j, unsure);
        while (unsure)
        {
            const int s = base + __ffs(unsure) - 1;
            unsure &= unsure - 1u;
            hits += ssao_sample(F, depth, k[3 * s], k[3 * s + 2], pos, nrm, fragDepth) > 0.f;
        }
    }
    return ssao_result(F, hits);
}

// The 16 background values by one CTA: one thread per (cell, sample), then each
// cell's contributions are summed in sample order as the reference does.
// rc: 16 N floats of shared memory.
__device__ __forceinline__ void ssao_background_cta(const FrameConst& F, const float* __restrict__ depth,
                                                    const float* __restrict__ table, float* rc, float* __restrict__ out16)
{
    const int N = F.ssaoN;
    for (int e = threadIdx.x; e < 16 * N; e += blockDim.x)
    {
        F3 k, o;
        ssao_kernel_offset(F, table, e, k, o);
        rc[e] = ssao_sample(F, depth, make_float4(k.x, k.y, k.z, 0.f), make_float4(o.x, o.y, o.z, 0.f),
                            F3{0.f, 0.f, 0.f}, F3{0.f, 0.f, 0.f}, FLT_MAX);
    }
    __syncthreads();
    if (threadIdx.x < 16)
    {
        const float kernelScale = 1.f / N;
        float occ = 0.f;
        for (int s = 0; s < N; ++s) occ += kernelScale * rc[threadIdx.x * N + s];
        occ = 1.f - occ;
        out16[threadIdx.x] = powf(occ, 3.f);
    }
}

__global__ void __launch_bounds__(1024) k_ssao_background(FrameConst F, const float* __restrict__ depth,
                                                           const float* __restrict__ table, float* __restrict__ out16,
                                                           const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    extern __shared__ float rcb[];
    ssao_background_cta(F, depth, table, rcb, out16);
}

// 512-thread CTAs, three per SM (40 registers a thread; the 16-cell sample table
// is 49 KB at 64 samples).
constexpr int kSsaoThreads = 512;

__global__ void __launch_bounds__(kSsaoThreads, 3) k_ssao(FrameConst F, GBuffer gb, const float* __restrict__ table,
                                               const float* __restrict__ bg16, const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    extern __shared__ float4 tbl4[];
    const int stride = ssao_q_stride(F.ssaoN);
    ssao_build_table_q(F, table, tbl4, stride);
    __syncthreads();
    const int n = F.W * F.H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    {
        int x = p % F.W, y = p / F.W;
        int cell = (y & 3) * 4 + (x & 3);
        // a covered pixel's depth passed the depth test (< FLT_MAX); the resolve
        // writes FLT_MAX everywhere else, so the depth stands in for the covered flag
        const float fragDepth = gb.depth[p];
        if (!(fragDepth < FLT_MAX))
        {
            gb.ao[p] = bg16[cell];
            continue;
        }
        float4 A = gb.a[p], B = gb.b[p];
        gb.ao[p] = ssao_pixel_filtered(F, gb.depth, tbl4 + cell * stride, ld3(A), ld3(B), fragDepth);
    }
}

// ---- learned AO: network input and probe -----------------------------------------------------

__device__ __forceinline__ unsigned pack_bf16_pair(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned*>(&v);
}

// Channel 3 of the network input: the view normal's z, the depth residual (K < 0) or (K > 0) a K-sample
// SSAO of the pixel (the reference's sampling with the K-sample table, no blur).
// FK.ssaoN < 0 (kAoInputDepthResidual): channel 3 is the depth channel's BF16
// rounding residual times 256, so channels 0 and 3 carry view depth to about 16
// mantissa bits (the network's input stays view depth and normal).
__device__ __forceinline__ float ao_input_ch3(const FrameConst& FK, const GBuffer& gb, const float4* tbl, int x, int y,
                                              float4 A, float4 B, float nz, float d, float fragDepth)
{
    if (FK.ssaoN == 0) return nz;
    if (FK.ssaoN < 0) return (d - __bfloat162float(__float2bfloat16_rn(d))) * 256.f;
    const int cell = (y & 3) * 4 + (x & 3);
    return ssao_pixel_filtered(FK, gb.depth, tbl + cell * ssao_q_stride(FK.ssaoN), ld3(A), ld3(B), fragDepth);
}

// The K-sample table of ao_input_ch3 in shared memory (FK: the frame constants
// with ssaoN = K), in the layout of the frame's estimated SSAO.
__device__ __forceinline__ FrameConst ao_input_table(const FrameConst& F, const float* table, int K, float4* tbl)
{
    FrameConst FK = F;
    FK.ssaoN = K;
    if (K > 0) ssao_build_table_q(FK, table, tbl, ssao_q_stride(K));
    __syncthreads();
    return FK;
}

// Network input of one pixel: view-space depth / 8 (positive in front of the
// camera), the view-space normal's x and y, and channel 3 (ao_input_ch3), BF16
// in channels 0..3 of an 8-channel vector; all zero where no triangle covers
// the pixel.
__global__ void k_ao_features(FrameConst F, GBuffer gb, uint4* __restrict__ out, const float* __restrict__ table, int K)
{
    extern __shared__ float4 tbl[];
    const FrameConst FK = ao_input_table(F, table, K, tbl);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= F.W * F.H) return;
    const float fragDepth = gb.depth[p];  // < FLT_MAX exactly where a triangle covers the pixel
    uint4 o = make_uint4(0u, 0u, 0u, 0u);
    if (fragDepth < FLT_MAX)
    {
        const float4 A = gb.a[p], B = gb.b[p];
        const float* V = F.V;
        const float z = ((V[8] * A.x + V[9] * A.y) + V[10] * A.z) + V[11];
        const float nx = (V[0] * B.x + V[1] * B.y) + V[2] * B.z;
        const float ny = (V[4] * B.x + V[5] * B.y) + V[6] * B.z;
        const float nz = (V[8] * B.x + V[9] * B.y) + V[10] * B.z;
        const float d = -z * 0.125f;
        o.x = pack_bf16_pair(d, nx);
        o.y = pack_bf16_pair(ny, ao_input_ch3(FK, gb, tbl, p % F.W, p / F.W, A, B, nz, d, fragDepth));
    }
    out[p] = o;
}

// The same input already rearranged for the network's 2x2-block level 0: block
// (X, Y) of the output [1][2][H/2][W/2][8] holds, in chunk r, row 2Y + r as
// [pixel 2X ch0..3 | pixel 2X+1 ch0..3]. One pixel per thread: the two pixels of
// an output vector are neighbouring lanes, and the even lane stores the pair.
// With bg16, block 0 computes the 16 background values of the frame's SSAO
// (ssao_background_cta, from frameTable) beside the others.
__global__ void __launch_bounds__(256, 6) k_ao_features_blocks(FrameConst F, GBuffer gb, uint4* __restrict__ out,
                                                            const float* __restrict__ table, int K,
                                                            const float* __restrict__ frameTable, float* __restrict__ bg16)
{
    extern __shared__ float4 tbl[];
    if (bg16 && blockIdx.x == 0)
    {
        ssao_background_cta(F, gb.depth, frameTable, reinterpret_cast<float*>(tbl), bg16);
        return;
    }
    const FrameConst FK = ao_input_table(F, table, K, tbl);
    const int w = F.W / 2, h = F.H / 2;
    const int t = (blockIdx.x - (bg16 ? 1 : 0)) * blockDim.x + threadIdx.x;
    const int i = t >> 1, dx = t & 1;
    const bool live = i < 2 * w * h;
    uint32_t v0 = 0u, v1 = 0u;
    if (live)
    {
        const int X = i % w, r = (i / w) % h, c8 = i / (w * h);
        const int px = 2 * X + dx, py = 2 * r + c8, p = py * F.W + px;
        const float fragDepth = gb.depth[p];  // < FLT_MAX exactly where a triangle covers the pixel
        if (fragDepth < FLT_MAX)
        {
            const float4 A = gb.a[p], B = gb.b[p];
            const float* V = F.V;
            const float z = ((V[8] * A.x + V[9] * A.y) + V[10] * A.z) + V[11];
            const float nx = (V[0] * B.x + V[1] * B.y) + V[2] * B.z;
            const float ny = (V[4] * B.x + V[5] * B.y) + V[6] * B.z;
            const float nz = (V[8] * B.x + V[9] * B.y) + V[10] * B.z;
            const float d = -z * 0.125f;
            v0 = pack_bf16_pair(d, nx);
            v1 = pack_bf16_pair(ny, ao_input_ch3(FK, gb, tbl, px, py, A, B, nz, d, fragDepth));
        }
    }
    // every lane of the warp reaches the exchange (blocks are whole warps)
    const uint32_t u0 = __shfl_xor_sync(0xffffffffu, v0, 1), u1 = __shfl_xor_sync(0xffffffffu, v1, 1);
    if (live && dx == 0) out[i] = make_uint4(v0, v1, u0, u1);
}

// The per-cell sample table of ssao_build_table, built once into global memory
// (16 cells x (2N + 2) float4) for kernels that read it from L1 instead.
__global__ void k_ssao_table_global(FrameConst F, const float* __restrict__ table, float4* __restrict__ out)
{
    ssao_build_table(F, table, out, 2 * F.ssaoN + 2);
}

// The probe: plain SSAO (the frame's sample count, no blur) on one pixel in 64 --
// (8i + 4, 8j + 4) -- against the network's AO there. Its plain values depend on
// the G-buffer only, so they are computed beside the network (k_ao_probe_plain);
// k_ao_probe_compare then reads the network's AO.

// plain[probe] = the plain SSAO of probe pixel `probe`, NaN where no triangle
// covers it; one warp per probe pixel, its lanes the samples.
__global__ void __launch_bounds__(256) k_ao_probe_plain(FrameConst F, GBuffer gb, const float4* __restrict__ tbl,
                                                         float* __restrict__ plain)
{
    const int pw = F.W / 8, ph = F.H / 8;
    const int lane = threadIdx.x & 31;
    const int probe = blockIdx.x * 8 + (threadIdx.x >> 5);  // uniform in the warp
    if (probe >= pw * ph) return;
    const int x = (probe % pw) * 8 + 4, y = (probe / pw) * 8 + 4;
    const int p = y * F.W + x;
    const float fragDepth = gb.depth[p];  // < FLT_MAX exactly where a triangle covers the pixel
    if (!(fragDepth < FLT_MAX))
    {
        if (lane == 0) plain[probe] = __int_as_float(0x7fc00000);
        return;
    }
    const int cell = (y & 3) * 4 + (x & 3);
    const float4* k = tbl + cell * (2 * F.ssaoN + 2);
    const F3 pos = ld3(gb.a[p]), nrm = ld3(gb.b[p]);
    int occluded = 0;
    for (int s0 = 0; s0 < F.ssaoN; s0 += 32)
    {
        const int s = s0 + lane;
        const bool hit = s < F.ssaoN && ssao_sample(F, gb.depth, k[2 * s], k[2 * s + 1], pos, nrm, fragDepth) > 0.f;
        occluded += __popc(__ballot_sync(0xffffffffu, hit));
    }
    // occ = kernelScale added once per occluding sample, in order (render.cpp:277)
    if (lane == 0) plain[probe] = ssao_result(F, occluded);
}

// The decision: one thread per probe pixel; part[2b], part[2b + 1] = block b's sum
// of squared differences and its count of covered probe pixels, summed in a fixed
// order; the last block to finish takes the mean over all blocks and sets *gate
// when it exceeds `threshold`.
__global__ void __launch_bounds__(256) k_ao_probe_compare(FrameConst F, const float* __restrict__ ao,
                                                           const float* __restrict__ plain, float* __restrict__ part,
                                                           unsigned* __restrict__ done, float threshold,
                                                           int* __restrict__ gate, float* __restrict__ mean)
{
    const int pw = F.W / 8, ph = F.H / 8;
    const int probe = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f, cnt = 0.f;
    if (probe < pw * ph)
    {
        const float pl = plain[probe];
        if (pl == pl)
        {
            const int x = (probe % pw) * 8 + 4, y = (probe / pw) * 8 + 4;
            const float dlt = ao[y * F.W + x] - pl;
            d2 = dlt * dlt;
            cnt = 1.f;
        }
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    __shared__ float red[2][8];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[0][wid] = d2, red[1][wid] = cnt;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        float a = 0.f, c = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[0][w], c += red[1][w];
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = c;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block: mean over all blocks in a fixed order (strided partial sums,
    // then a pairwise tree: 8 dependent FP64 adds, not a 256-long chain)
    __threadfence();
    double a = 0.0, c = 0.0;
    for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
    {
        a += __ldcg(part + 2 * b);
        c += __ldcg(part + 2 * b + 1);
    }
    __shared__ double ra[256], rc[256];
    ra[threadIdx.x] = a;
    rc[threadIdx.x] = c;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1)  // blockDim.x == 256
    {
        if (threadIdx.x < h)
        {
            ra[threadIdx.x] += ra[threadIdx.x + h];
            rc[threadIdx.x] += rc[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        const double sa = ra[0], sc = rc[0];
        const float m = sc > 0.0 ? static_cast<float>(sa / sc) : 0.f;
        *mean = m;
        *gate = m > threshold ? 1 : 0;
        *done = 0u;  // ready for the next frame (and graph replays)
    }
}

// ---- blur (buffer.cpp:59-98) -----------------------------------------------------------------
__constant__ float c_blurW[5] = {0.227027f, 0.1945946f, 0.1216216f, 0.054054f, 0.016216f};

// In-place two-pass Gaussian, bit-exact: one thread walks one row (then one
// column) in order, carrying the already-updated left / upper neighbours in
// registers as the reference's in-place reads see them. The lines a CTA walks
// are first staged in shared memory (padded stride: conflict-free column
// access), so the sequential walk only waits on its own 9-tap recurrence and
// never on global memory; results go back with coalesced stores.
template <int LINES>
__global__ void __launch_bounds__(256) k_blur_inplace(float* a, int W, int H, int vertical, const int* gate)
{
    if (gate && *gate == 0) return;
    extern __shared__ float strip[];
    const int n = vertical ? H : W;          // length of a line
    const int lines = vertical ? W : H;      // number of lines
    const int first = blockIdx.x * LINES;
    const int cnt = min(LINES, lines - first);
    const int stride = vertical ? LINES + 1 : n + 1;  // floats between consecutive elements / lines
    // stage: horizontal -> strip[l * (n + 1) + i]; vertical -> strip[i * (LINES + 1) + l].
    // Element e of the strip is line e / n, position e % n (horizontal) or position
    // e / LINES, line e % LINES (vertical); each thread keeps kStageU loads in flight.
    const int total = n * LINES;
    auto gaddr = [&](int e, bool& ok) -> size_t {
        if (!vertical)
        {
            const int l = e / n, i = e - l * n;
            ok = l < cnt;
            return (size_t)(first + l) * W + i;
        }
        const int i = e / LINES, c = e - i * LINES;
        ok = c < cnt;
        return (size_t)i * W + first + c;
    };
    auto saddr = [&](int e) -> int {
        if (!vertical)
        {
            const int l = e / n;
            return l * stride + (e - l * n);
        }
        const int i = e / LINES;
        return i * stride + (e - i * LINES);
    };
    constexpr int kStageU = 8;
    for (int base = threadIdx.x; base < total; base += blockDim.x * kStageU)
    {
        float v[kStageU];
#pragma unroll
        for (int u = 0; u < kStageU; ++u)
        {
            const int e = base + u * blockDim.x;
            bool ok = false;
            const size_t g = e < total ? gaddr(e, ok) : 0;
            v[u] = (e < total && ok) ? a[g] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kStageU; ++u)
        {
            const int e = base + u * blockDim.x;
            if (e < total) strip[saddr(e)] = v[u];
        }
    }
    __syncthreads();
    const int l = threadIdx.x;
    if (l < cnt)
    {
        float* s = vertical ? strip + l : strip + l * stride;
        const int step = vertical ? stride : 1;
        const float w0 = c_blurW[0], w1 = c_blurW[1], w2 = c_blurW[2], w3 = c_blurW[3], w4 = c_blurW[4];
        auto at = [&](int i) -> float { return s[min(i, n - 1) * step]; };
        float x0 = at(0), x1 = at(1), x2 = at(2), x3 = at(3), x4 = at(4);
        float p5 = at(5), p6 = at(6), p7 = at(7);  // prefetched originals
        float l1 = x0, l2 = x0, l3 = x0, l4 = x0;  // clamped left reads of index 0 before its update
        // One step: the reference's sum order (buffer.cpp:66-74); the running sum
        // first needs the previous result at its third term.
        auto step_once = [&](int i) -> float {
            float p8 = at(i + 8);
            float r = x0 * w0;
            r += x1 * w1;
            r += l1 * w1;
            r += x2 * w2;
            r += l2 * w2;
            r += x3 * w3;
            r += l3 * w3;
            r += x4 * w4;
            r += l4 * w4;
            s[i * step] = r;
            x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = p5, p5 = p6, p6 = p7, p7 = p8;
            return r;
        };
        if (n > 0)
        {
            // index 0: its left neighbours are the clamped index 0 itself, updated in place
            const float r0 = step_once(0);
            l1 = l2 = l3 = l4 = r0;
        }
        // groups of 8 steps unrolled: the rotations of the window become register renaming
        int i = 1;
        for (; i + 8 <= n; i += 8)
        {
#pragma unroll
            for (int u = 0; u < 8; ++u)
            {
                const float r = step_once(i + u);
                l4 = l3;
                l3 = l2;
                l2 = l1;
                l1 = r;
            }
        }
        for (; i < n; ++i)
        {
            const float r = step_once(i);
            l4 = l3;
            l3 = l2;
            l2 = l1;
            l1 = r;
        }
    }
    __syncthreads();
    if (!vertical)
    {
        for (int l2 = 0; l2 < cnt; ++l2)
            for (int i = threadIdx.x; i < n; i += blockDim.x) a[(size_t)(first + l2) * W + i] = strip[l2 * stride + i];
    }
    else
    {
        for (int e = threadIdx.x; e < n * LINES; e += blockDim.x)
        {
            int i = e / LINES, c = e % LINES;
            if (c < cnt) a[(size_t)i * W + first + c] = strip[i * stride + c];
        }
    }
}

// ---- the in-place blur in parallel, bit-exact --------------------------------------------------
// One pass of the in-place blur is the recurrence r_i = f(x_i .. x_{i+4}, r_{i-1} .. r_{i-4})
// over the originals x and the results r, evaluated in the reference's float
// order. Its state is the four previous results, and a difference in that state
// shrinks by about 0.61 per step (the largest root of z^4 = w1 z^3 + w2 z^2 +
// w3 z + w4), so two evaluations started from different states become the same
// floats after a few dozen steps. Each line is cut into chunks of kBlurChunk
// positions, one thread per chunk. A thread starts `warm` steps before its
// chunk from a guessed state (the originals there) and runs to the chunk's end;
// the four results it holds when it reaches the chunk are its entry state. The
// chunk is right exactly when that entry state equals, bit for bit, the last
// four results of the chunk before it, and the first chunk starts at position
// 0 from the true state, so by induction every chunk whose check passes holds
// the reference's floats. A chunk whose check fails is recomputed from the
// previous chunk's results, in order along the line, and the chunk after a
// recomputed one is checked again. Any warm-up length gives the same bits;
// short ones only make more chunks fall back to the sequential repair.
constexpr int kBlurChunk = 32;
constexpr int kBlurWarmDefault = 64;

__device__ __forceinline__ float blur_step(float x0, float x1, float x2, float x3, float x4, float l1, float l2,
                                           float l3, float l4, const float* w)
{
    // buffer.cpp:66-74: the running sum, right (original) tap before left (updated) tap
    float r = x0 * w[0];
    r += x1 * w[1];
    r += l1 * w[1];
    r += x2 * w[2];
    r += l2 * w[2];
    r += x3 * w[3];
    r += l3 * w[3];
    r += x4 * w[4];
    r += l4 * w[4];
    return r;
}

// Shared-memory index of position i of line l. Horizontal (lines are rows):
// one float of padding after every chunk, so the threads of consecutive chunks
// of a row read distinct banks. Vertical (lines are columns, L per CTA): the L
// columns of a position are adjacent, and the chunk stride 32 (L + 1) + L puts
// the 32 / L chunks a warp covers in different banks.
template <bool VERT>
__device__ __forceinline__ int blur_sidx(int l, int i, int rowStride, int L)
{
    if (!VERT) return l * rowStride + i + (i >> 5);
    return (i >> 5) * (32 * (L + 1) + L) + (i & 31) * (L + 1) + l;
}

// The same index split into a base (position s, a multiple of 32) and an offset of
// position s + tt, so that with tt a compile-time constant the offset is one too.
template <bool VERT>
__device__ __forceinline__ int blur_base(int l, int s, int rowStride, int L)
{
    return VERT ? (s >> 5) * (32 * (L + 1) + L) + l : l * rowStride + s + (s >> 5);
}
template <bool VERT, int LV>
__device__ __forceinline__ constexpr int blur_off(int tt)
{
    return VERT ? (tt >> 5) * (32 * (LV + 1) + LV) + (tt & 31) * (LV + 1) : tt + (tt >> 5);
}

// VERT: LV columns per CTA (a compile-time constant); horizontal: L rows per CTA.
template <bool VERT, int LV>
__global__ void __launch_bounds__(512) k_blur_spec(float* a, int W, int H, int Lrows, int warm, const int* gate)
{
    if (gate && *gate == 0) return;
    extern __shared__ float sm[];
    const float* w = c_blurW;
    const int L = VERT ? LV : Lrows;
    constexpr int lgL = LV == 16 ? 4 : LV == 8 ? 3 : LV == 4 ? 2 : 0;
    const int n = VERT ? H : W;
    const int lines = VERT ? W : H;
    const int first = blockIdx.x * L;
    const int cnt = min(L, lines - first);
    const int nch = (n + kBlurChunk - 1) / kBlurChunk;
    const int rowStride = n + nch + 1;
    const int items = L * nch;
    const int smLine = VERT ? nch * (32 * (L + 1) + L) : L * rowStride;
    float4* chk = reinterpret_cast<float4*>(sm + ((smLine + 3) & ~3));
    int* bad = reinterpret_cast<int*>(chk + items);
    auto gidx = [&](int l, int i) -> size_t {
        return VERT ? (size_t)i * W + first + l : (size_t)(first + l) * W + i;
    };
    // Stage the lines, coalesced, kStage loads in flight per thread. Horizontal: a
    // row at a time, consecutive threads on consecutive pixels. Vertical (blockDim
    // a multiple of L, L = 2^lgL): thread t takes column t mod L of rows t / L,
    // t / L + blockDim / L, ...
    constexpr int kStage = 8;
    const int lane0 = VERT ? (threadIdx.x & (L - 1)) : 0;
    const int row0 = VERT ? (threadIdx.x >> lgL) : threadIdx.x;
    const int rstep = VERT ? (blockDim.x >> lgL) : blockDim.x;
    for (int l = VERT ? lane0 : 0; l < cnt; l += VERT ? L : 1)
        for (int i0 = row0; i0 < n; i0 += kStage * rstep)
        {
            float v[kStage];
#pragma unroll
            for (int u = 0; u < kStage; ++u)
            {
                const int i = i0 + u * rstep;
                v[u] = i < n ? a[gidx(l, i)] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < kStage; ++u)
            {
                const int i = i0 + u * rstep;
                if (i < n) sm[blur_sidx<VERT>(l, i, rowStride, L)] = v[u];
            }
        }
    __syncthreads();

    // Work items: the interior chunks (those the unrolled path takes at the default
    // warm-up, jlo <= j <= jlo + nInt - 1) on consecutive threads first, the chunks at
    // the two ends of the lines after them, so that a warp runs one of the two paths.
    // Vertical: the L columns of a chunk index are adjacent threads.
    const int jlo = (kBlurWarmDefault + 4 + kBlurChunk - 1) / kBlurChunk;
    const int nInt = warm == kBlurWarmDefault ? max(0, min(nch, (n - kBlurChunk - 5) / kBlurChunk + 1) - jlo) : 0;
    const int nEdge = nch - nInt;
    const int t = threadIdx.x;
    int l, j;
    {
        int q, k;
        if (VERT)
        {
            l = t % L;
            q = t / L;
        }
        else
        {
            const bool in = t < L * nInt;
            const int e2 = in ? t : t - L * nInt;
            const int per = in ? nInt : nEdge;
            l = per > 0 ? e2 / per : 0;
            q = in ? e2 % max(per, 1) : nInt + e2 % max(per, 1);
        }
        k = q - nInt;
        j = q < nInt ? jlo + q : (k < jlo ? k : k + nInt);
    }
    const bool active = t < items && l < cnt;
    const int b = j * kBlurChunk, e = min(b + kBlurChunk, n);
    float res[kBlurChunk];
    float c1 = 0.f, c2 = 0.f, c3 = 0.f, c4 = 0.f;
    const bool fast = active && warm == kBlurWarmDefault && b - warm >= 4 && b + kBlurChunk + 4 < n;
    if (fast)
    {
        // An interior chunk at the default warm-up: its first position is a multiple
        // of 32, so every read is a fixed offset from one base and the 96 steps unroll
        // into straight-line code.
        const float* base = sm + blur_base<VERT>(l, b - kBlurWarmDefault, rowStride, L);
        float l1 = base[blur_off<VERT, LV>(-1)], l2 = base[blur_off<VERT, LV>(-2)];
        float l3 = base[blur_off<VERT, LV>(-3)], l4 = base[blur_off<VERT, LV>(-4)];
        float x0 = base[blur_off<VERT, LV>(0)], x1 = base[blur_off<VERT, LV>(1)], x2 = base[blur_off<VERT, LV>(2)];
        float x3 = base[blur_off<VERT, LV>(3)], x4 = base[blur_off<VERT, LV>(4)];
#pragma unroll
        for (int u = 0; u < kBlurWarmDefault + kBlurChunk; ++u)
        {
            if (u == kBlurWarmDefault) c1 = l1, c2 = l2, c3 = l3, c4 = l4;
            const float r = blur_step(x0, x1, x2, x3, x4, l1, l2, l3, l4, w);
            if (u >= kBlurWarmDefault) res[u - kBlurWarmDefault] = r;
            l4 = l3, l3 = l2, l2 = l1, l1 = r;
            x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = base[blur_off<VERT, LV>(u + 5)];
        }
    }
    else if (active)
    {
        auto X = [&](int i) -> float { return sm[blur_sidx<VERT>(l, min(i, n - 1), rowStride, L)]; };
        int i = b - warm;
        float l1, l2, l3, l4, x0, x1, x2, x3, x4;
        if (i <= 0)
        {
            // from the line's start, exactly: position 0's left reads are itself, original
            x0 = X(0), x1 = X(1), x2 = X(2), x3 = X(3), x4 = X(4);
            const float r0 = blur_step(x0, x1, x2, x3, x4, x0, x0, x0, x0, w);
            res[0] = r0;
            l1 = l2 = l3 = l4 = r0;
            x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = X(5);
            i = 1;
        }
        else
        {
            l1 = X(i - 1), l2 = X(i - 2), l3 = X(i - 3), l4 = X(i - 4);
            x0 = X(i), x1 = X(i + 1), x2 = X(i + 2), x3 = X(i + 3), x4 = X(i + 4);
        }
        for (; i < b; ++i)  // warm-up: results not kept
        {
            const float r = blur_step(x0, x1, x2, x3, x4, l1, l2, l3, l4, w);
            l4 = l3, l3 = l2, l2 = l1, l1 = r;
            x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = X(i + 5);
        }
        c1 = l1, c2 = l2, c3 = l3, c4 = l4;
#pragma unroll
        for (int u = 0; u < kBlurChunk; ++u)
        {
            if (b + u >= i && b + u < e)
            {
                const float r = blur_step(x0, x1, x2, x3, x4, l1, l2, l3, l4, w);
                res[u] = r;
                l4 = l3, l3 = l2, l2 = l1, l1 = r;
                x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = X(b + u + 5);
            }
        }
    }
    __syncthreads();  // every original has been read: results may replace them
    if (active)
    {
#pragma unroll
        for (int u = 0; u < kBlurChunk; ++u)
            if (b + u < e) sm[blur_sidx<VERT>(l, b + u, rowStride, L)] = res[u];
        chk[t] = make_float4(c1, c2, c3, c4);
    }
    __syncthreads();
    int mismatch = 0;
    if (active && j > 0)
    {
        const float p1 = sm[blur_sidx<VERT>(l, b - 1, rowStride, L)], p2 = sm[blur_sidx<VERT>(l, b - 2, rowStride, L)];
        const float p3 = sm[blur_sidx<VERT>(l, b - 3, rowStride, L)], p4 = sm[blur_sidx<VERT>(l, b - 4, rowStride, L)];
        mismatch = (__float_as_uint(c1) != __float_as_uint(p1)) | (__float_as_uint(c2) != __float_as_uint(p2)) |
                   (__float_as_uint(c3) != __float_as_uint(p3)) | (__float_as_uint(c4) != __float_as_uint(p4));
    }
    if (t < items) bad[t] = mismatch;
    if (__syncthreads_or(mismatch))
    {
        // sequential repair, one thread per line, with the originals from global
        // memory (this CTA stores its lines only at the end)
        if (active && j == 0)
        {
            auto S = [&](int i) -> float& { return sm[blur_sidx<VERT>(l, i, rowStride, L)]; };
            auto Xg = [&](int i) -> float { return a[gidx(l, min(i, n - 1))]; };
            bool prevRedone = false;
            for (int c = 1; c < nch; ++c)
            {
                const int cb = c * kBlurChunk, ce = min(cb + kBlurChunk, n);
                // the work item of chunk c of this line (the inverse of the mapping above)
                const bool inner = c >= jlo && c < jlo + nInt;
                const int qq = inner ? c - jlo : nInt + (c < jlo ? c : c - nInt);
                const int it = VERT ? qq * L + l : (inner ? l * nInt + qq : L * nInt + l * nEdge + (qq - nInt));
                float l1 = S(cb - 1), l2 = S(cb - 2), l3 = S(cb - 3), l4 = S(cb - 4);
                bool ok;
                if (prevRedone)
                {
                    const float4 q = chk[it];
                    ok = __float_as_uint(q.x) == __float_as_uint(l1) && __float_as_uint(q.y) == __float_as_uint(l2) &&
                         __float_as_uint(q.z) == __float_as_uint(l3) && __float_as_uint(q.w) == __float_as_uint(l4);
                }
                else
                {
                    ok = bad[it] == 0;
                }
                prevRedone = !ok;
                if (ok) continue;
                float x0 = Xg(cb), x1 = Xg(cb + 1), x2 = Xg(cb + 2), x3 = Xg(cb + 3), x4 = Xg(cb + 4);
                for (int i = cb; i < ce; ++i)
                {
                    const float r = blur_step(x0, x1, x2, x3, x4, l1, l2, l3, l4, w);
                    S(i) = r;
                    l4 = l3, l3 = l2, l2 = l1, l1 = r;
                    x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = Xg(i + 5);
                }
            }
        }
        __syncthreads();
    }
    for (int ll = VERT ? lane0 : 0; ll < cnt; ll += VERT ? L : 1)
        for (int i = row0; i < n; i += rstep) a[gidx(ll, i)] = sm[blur_sidx<VERT>(ll, i, rowStride, L)];
}

// Shared memory of k_blur_spec for L lines of length n (0 if more than the
// per-CTA limit).
size_t blur_spec_smem(int n, int L, bool vert)
{
    const int nch = (n + kBlurChunk - 1) / kBlurChunk;
    const size_t line = vert ? (size_t)nch * (32 * (L + 1) + L) : (size_t)L * (n + nch + 1);
    const size_t items = (size_t)L * nch;
    if (items > 512) return 0;
    const size_t bytes = ((line + 3) & ~(size_t)3) * sizeof(float) + items * (sizeof(float4) + sizeof(int));
    return bytes <= 200 * 1024 ? bytes : 0;
}

// pow(b / 255, 2.2) for every byte b with the device's own powf, the values the
// shaders compute from 8-bit texels (DevScene::gamma8).
__global__ void k_gamma8_table(float* __restrict__ out)
{
    const unsigned b = threadIdx.x;
    if (b < 256) out[b] = powf(rgb_to_f3(b, b, b).x, 2.2f);
}

// Ping-pong separable Gaussian (same taps, reads only the previous sweep).
__global__ void k_blur_sep(const float* __restrict__ src, float* __restrict__ dst, int W, int H, int vertical,
                           const int* __restrict__ gate)
{
    if (gate && *gate == 0) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= W * H) return;
    int x = p % W, y = p / W;
    const float* w = c_blurW;
    float r;
    if (!vertical)
    {
        const float* row = src + (size_t)y * W;
        r = row[x] * w[0];
        for (int i = 1; i < 5; ++i)
        {
            r += row[min(W - 1, x + i)] * w[i];
            r += row[max(0, x - i)] * w[i];
        }
    }
    else
    {
        r = src[p] * w[0];
        for (int i = 1; i < 5; ++i)
        {
            r += src[(size_t)min(H - 1, y + i) * W + x] * w[i];
            r += src[(size_t)max(0, y - i) * W + x] * w[i];
        }
    }
    dst[p] = r;
}

// ---- SSAA (render.cpp:291-345) ---------------------------------------------------------------
// R, G, B bytes of n 32-bit R | G << 8 | B << 16 pixels (the 8-bit images'
// download layout), 4 pixels (12 bytes) per thread.
// RGBA8 words -> R, G, B bytes. A CTA packs 1,024 pixels in shared memory and stores
// its 3,072 bytes as contiguous 16-byte pieces (the destination may be host memory
// written across the chip-to-chip link, where wide contiguous stores matter).
constexpr int kPackPixels = 1024;
__global__ void __launch_bounds__(256) k_pack_rgb(const unsigned* __restrict__ in, uint8_t* __restrict__ out, int n)
{
    __shared__ __align__(16) uint32_t sb[3 * kPackPixels / 4];
    const int p0 = blockIdx.x * kPackPixels;
    const int cnt = min(kPackPixels, n - p0);
    const bool full = cnt == kPackPixels && (reinterpret_cast<uintptr_t>(out) & 15u) == 0u;
    if (full)
    {
        // thread t: pixels 4t .. 4t+3 -> words 3t .. 3t+2
        const int t = threadIdx.x;
        const uint4 v = *reinterpret_cast<const uint4*>(in + p0 + 4 * t);
        sb[3 * t] = (v.x & 0xffffffu) | (v.y << 24);
        sb[3 * t + 1] = ((v.y >> 8) & 0xffffu) | (v.z << 16);
        sb[3 * t + 2] = ((v.z >> 16) & 0xffu) | (v.w << 8);
        __syncthreads();
        uint4* o = reinterpret_cast<uint4*>(out + 3 * (size_t)p0);
        const uint4* sv = reinterpret_cast<const uint4*>(sb);
        for (int q = threadIdx.x; q < 3 * kPackPixels / 16; q += blockDim.x) o[q] = sv[q];
        return;
    }
    for (int p = p0 + threadIdx.x; p < p0 + cnt; p += blockDim.x)
    {
        const unsigned c = in[p];
        out[3 * (size_t)p] = (uint8_t)(c & 0xffu);
        out[3 * (size_t)p + 1] = (uint8_t)((c >> 8) & 0xffu);
        out[3 * (size_t)p + 2] = (uint8_t)((c >> 16) & 0xffu);
    }
}

__global__ void k_ssaa(int W, int H, int k, const unsigned* __restrict__ frame8, unsigned* __restrict__ out)
{
    int ow = W / k, oh = H / k;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ow * oh) return;
    int x = p % ow, y = p / ow;
    int R = 0, G = 0, B = 0;
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j)
        {
            unsigned c = frame8[(size_t)(y * k + j) * W + x * k + i];
            R += c & 0xff, G += (c >> 8) & 0xff, B += (c >> 16) & 0xff;
        }
    float kk = (float)(k * k);
    R = (int)(R / kk);
    G = (int)(G / kk);
    B = (int)(B / kk);
    out[p] = (unsigned)(R & 0xff) | ((unsigned)(G & 0xff) << 8) | ((unsigned)(B & 0xff) << 16);
}

// ---- read-back helpers ----------------------------------------------------------------------
__global__ void k_unpack(DevScene S, GBuffer gb, int n, int which, float* out)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float4 A = gb.a[p], B = gb.b[p];
    uint4 C = gb.c[p];
    F3 v{0.f, 0.f, 0.f};
    if (which == 0) v = ld3(B);
    else if (which == 1) v = ld3(A);
    else if (which == 2) v = F3{A.w, B.w, __uint_as_float(C.x)};
    else
    {
        GDecoded g = decode_gbuffer(S, C);
        if (which == 3) v = g.albedo;
        else if (which == 4) v = g.emissive;
        else if (which == 5) v = g.param;
        else
        {
            out[p] = g.type;
            return;
        }
    }
    out[3 * (size_t)p] = v.x;
    out[3 * (size_t)p + 1] = v.y;
    out[3 * (size_t)p + 2] = v.z;
}

__global__ void k_tri_ids(const unsigned long long* keys, int n, int* out)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    unsigned long long k = keys[p];
    out[p] = k == frx::kEmptyKey ? -1 : (int)(k & 0xffffffffu);
}

inline int blocks(long long n, int bs) { return (int)((n + bs - 1) / bs); }

}  // namespace

// ---- launchers -------------------------------------------------------------------------------
void launch_transform_camera(const DevScene& S, const FrameConst& F, VertexOut vo, cudaStream_t st)
{
    int n = max(S.numVerts, S.numNormals);
    if (n > 0) k_transform_camera<<<blocks(n, 256), 256, 0, st>>>(S, F, vo);
}

void launch_transform_light(const DevScene& S, const FrameConst& F, int4* scrL, cudaStream_t st)
{
    if (S.numVerts > 0) k_transform_light<<<blocks(S.numVerts, 256), 256, 0, st>>>(S, F, scrL);
}

void launch_raster(const DevScene& S, const int4* scr, const RasterParams& rp, RasterScratch& rs, cudaStream_t st,
                   int& launches, bool tileRaster, float* shadowOut)
{
    const int tiles = ((rp.W + kTile - 1) / kTile) * ((rp.H + kTile - 1) / kTile);
    cudaMemsetAsync(rs.keys, 0xff, sizeof(unsigned long long) * (size_t)rp.W * rp.H, st);
    cudaMemsetAsync(rs.counters, 0, sizeof(int) * 4, st);
    cudaMemsetAsync(rs.tileCount, 0, sizeof(int) * tiles, st);
    if (S.numTris <= 0)
    {
        if (shadowOut) cudaMemsetAsync(shadowOut, 0, sizeof(float) * (size_t)rp.W * rp.H, st);
        return;
    }
    k_setup<<<blocks(S.numTris, kSetupThreads), kSetupThreads, 0, st>>>(S, scr, rp, rs);
    int sms = 152;
    k_raster_medium<<<sms * 8, 256, 0, st>>>(rp, rs);
    k_bin<<<sms * 4, 256, 0, st>>>(rp, rs, 0);
    k_bin_scan<<<1, 1024, 0, st>>>(rs, tiles);
    k_bin<<<sms * 4, 256, 0, st>>>(rp, rs, 1);
    if (tileRaster && shadowOut) k_tile_raster_shadow<<<tiles, 256, 0, st>>>(rp, rs, S, scr, shadowOut);
    else if (tileRaster) k_tile_raster<<<tiles, 256, 0, st>>>(rp, rs);
    launches += tileRaster ? 6 : 5;
}

void launch_tile_raster_views(const ViewRaster* vr, const int* itemStart, int nEntries, int total, int* queue,
                              int cap, int grid, cudaStream_t st)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_tile_raster_views<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    const size_t smem = (size_t)cap * (sizeof(frx::RTri) + sizeof(int) + sizeof(int4));
    cudaMemsetAsync(queue, 0, sizeof(int), st);
    if (cap >= 1024) k_tile_raster_views<1024><<<grid, 256, smem, st>>>(vr, itemStart, nEntries, total, queue);
    else if (cap >= 256) k_tile_raster_views<256><<<grid, 256, smem, st>>>(vr, itemStart, nEntries, total, queue);
    else k_tile_raster_views<64><<<grid, 256, smem, st>>>(vr, itemStart, nEntries, total, queue);
}

template <bool kLinear>
void launch_lighting_views_t(const DevScene& S, const ViewShade* views, const int* itemStart, int nViews, int total,
                             const BatchLight* lights, int nLights, int* queue, int T, int grid, cudaStream_t st)
{
    if (T <= 8)
        k_lighting_views<8, kLinear><<<grid, 256, 0, st>>>(S, views, itemStart, nViews, total, lights, nLights, queue);
    else if (T <= 16)
        k_lighting_views<16, kLinear><<<grid, 256, 0, st>>>(S, views, itemStart, nViews, total, lights, nLights, queue);
    else
        k_lighting_views<32, kLinear><<<grid, 256, 0, st>>>(S, views, itemStart, nViews, total, lights, nLights, queue);
}

void launch_lighting_views(const DevScene& S, const ViewShade* views, const int* itemStart, int nViews, int total,
                           const BatchLight* lights, int nLights, int* queue, int T, int grid, cudaStream_t st)
{
    cudaMemsetAsync(queue, 0, sizeof(int), st);
    if (S.texLinear)
        launch_lighting_views_t<true>(S, views, itemStart, nViews, total, lights, nLights, queue, T, grid, st);
    else
        launch_lighting_views_t<false>(S, views, itemStart, nViews, total, lights, nLights, queue, T, grid, st);
}

void launch_resolve_shadow(const DevScene& S, const int4* scrL, const unsigned long long* keys, int SW, int SH,
                           float* shadow, cudaStream_t st)
{
    k_resolve_shadow<<<blocks((long long)SW * SH, 256), 256, 0, st>>>(S, scrL, keys, SW, SH, shadow);
}

void launch_resolve_gbuffer(const DevScene& S, const FrameConst& F, VertexOut vo, const unsigned long long* keys,
                            GBuffer gb, cudaStream_t st)
{
    k_resolve_gbuffer<<<blocks((long long)F.W * F.H, 128), 128, 0, st>>>(S, F, vo, keys, gb);
}

void launch_forward_shade(const DevScene& S, const FrameConst& F, VertexOut vo, const unsigned long long* keys,
                          const float* shadow, float* depth, unsigned* frame8, float* frameF, cudaStream_t st,
                          const int* counters, int* statusOut)
{
    k_forward_shade<<<blocks((long long)F.W * F.H, 128), 128, 0, st>>>(S, F, vo, keys, shadow, depth, frame8, frameF,
                                                                       counters, statusOut);
}

void ssao_attributes()
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_ssao, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_ssao_background, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_ao_features, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_ao_features_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
}

void launch_ssao(const FrameConst& F, GBuffer gb, const float* table, float* bg16, cudaStream_t st, const int* gate,
                 bool withBackground)
{
    const size_t smem = sizeof(float4) * 16 * ssao_q_stride(F.ssaoN);
    ssao_attributes();
    if (withBackground)
        k_ssao_background<<<1, 1024, sizeof(float) * 16 * F.ssaoN, st>>>(F, gb.depth, table, bg16, gate);
    // gated (learned-AO fallback): a small grid-stride grid, so a skipped pass costs little
    const int grid = gate ? std::min(blocks((long long)F.W * F.H, kSsaoThreads), 2 * 152)
                          : blocks((long long)F.W * F.H, kSsaoThreads);
    k_ssao<<<grid, kSsaoThreads, smem, st>>>(F, gb, table, bg16, gate);
}

void launch_ssao_background(const FrameConst& F, const float* depth, const float* table, float* bg16, cudaStream_t st)
{
    ssao_attributes();
    k_ssao_background<<<1, 1024, sizeof(float) * 16 * F.ssaoN, st>>>(F, depth, table, bg16, nullptr);
}

size_t ao_input_smem(int K) { return K > 0 ? sizeof(float4) * 16 * (size_t)ssao_q_stride(K) : 0; }

void launch_ao_features(const FrameConst& F, GBuffer gb, uint4* out, cudaStream_t st, const float* inputTable, int K)
{
    ssao_attributes();
    k_ao_features<<<blocks((long long)F.W * F.H, 256), 256, ao_input_smem(K), st>>>(F, gb, out, inputTable, K);
}

void launch_ao_features_blocks(const FrameConst& F, GBuffer gb, uint4* out, cudaStream_t st, const float* inputTable,
                               int K, const float* frameTable, float* bg16)
{
    ssao_attributes();
    const size_t smem = std::max(ao_input_smem(K), bg16 ? sizeof(float) * 16 * F.ssaoN : (size_t)0);
    k_ao_features_blocks<<<blocks((long long)F.W * F.H, 256) + (bg16 ? 1 : 0), 256, smem, st>>>(F, gb, out, inputTable,
                                                                                             K, frameTable, bg16);
}

void launch_ssao_table_global(const FrameConst& F, const float* table, float4* out, cudaStream_t st)
{
    k_ssao_table_global<<<1, 256, 0, st>>>(F, table, out);
}

int ao_probe_blocks(int W, int H) { return blocks((long long)(W / 8) * (H / 8), 256); }

void launch_ao_probe_plain(const FrameConst& F, GBuffer gb, const float4* tbl, float* plain, cudaStream_t st)
{
    const long long n = (long long)(F.W / 8) * (F.H / 8);
    if (n > 0) k_ao_probe_plain<<<blocks(n, 8), 256, 0, st>>>(F, gb, tbl, plain);
}

void launch_ao_probe_compare(const FrameConst& F, const float* ao, const float* plain, float threshold, float* part,
                             unsigned* done, int* gate, float* mean, cudaStream_t st)
{
    k_ao_probe_compare<<<ao_probe_blocks(F.W, F.H), 256, 0, st>>>(F, ao, plain, part, done, threshold, gate, mean);
}


int launch_blur(int mode, int W, int H, float* ao, float* tmp, cudaStream_t st, int& launches, const int* gate,
                int warm)
{
    if (mode == 0)
    {
        // the parallel form when both passes' lines fit a CTA, else the sequential walk below
        static bool specAttr = false;
        if (!specAttr)
        {
            cudaFuncSetAttribute(k_blur_spec<false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            cudaFuncSetAttribute(k_blur_spec<true, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            cudaFuncSetAttribute(k_blur_spec<true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            specAttr = true;
        }
        const int wsteps = warm > 0 ? warm : kBlurWarmDefault;
        const int nchH = (W + kBlurChunk - 1) / kBlurChunk;
        // few lines per CTA: more CTAs than SMs, each a short chain of warm-up + chunk steps
        int sh = 4;
        while (sh > 1 && (sh * nchH > 512 || blur_spec_smem(W, sh, false) == 0)) --sh;
        const int sv = blur_spec_smem(H, 8, true) ? 8 : 4;
        const size_t smSpecH = blur_spec_smem(W, sh, false), smSpecV = blur_spec_smem(H, sv, true);
        if (smSpecH && smSpecV)
        {
            k_blur_spec<false, 0><<<blocks(H, sh), sh * nchH, smSpecH, st>>>(ao, W, H, sh, wsteps, gate);
            const int nchV = (H + kBlurChunk - 1) / kBlurChunk;
            if (sv == 8)
                k_blur_spec<true, 8><<<blocks(W, 8), 8 * nchV, smSpecV, st>>>(ao, W, H, 8, wsteps, gate);
            else
                k_blur_spec<true, 4><<<blocks(W, 4), 4 * nchV, smSpecV, st>>>(ao, W, H, 4, wsteps, gate);
            launches += 2;
            return FR_OK;
        }
        static bool attr = false;
        if (!attr)
        {
            cudaFuncSetAttribute(k_blur_inplace<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
            cudaFuncSetAttribute(k_blur_inplace<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
            cudaFuncSetAttribute(k_blur_inplace<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
            cudaFuncSetAttribute(k_blur_inplace<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
            attr = true;
        }
        // The sequential walk: strips of rows (a row is W + 1 floats of shared memory),
        // then strips of columns (H (lines + 1) floats); the launch's template count of
        // lines is the one the strip was sized for.
        constexpr size_t kStrip = 220 * 1024;
        int lh = 8;
        while (lh > 0 && sizeof(float) * (size_t)lh * (W + 1) > kStrip) lh >>= 1;
        int lv = 8;
        while (lv > 0 && sizeof(float) * (size_t)H * (lv + 1) > kStrip) lv >>= 1;
        if (lh == 0 || lv == 0) return FR_ERR_UNSUPPORTED;  // a line longer than one CTA's shared memory
        const size_t smh = sizeof(float) * (size_t)lh * (W + 1), smv = sizeof(float) * (size_t)H * (lv + 1);
        auto walk = [&](int lines, int count, size_t smem, int vertical) {
            if (lines == 8) k_blur_inplace<8><<<blocks(count, 8), 256, smem, st>>>(ao, W, H, vertical, gate);
            else if (lines == 4) k_blur_inplace<4><<<blocks(count, 4), 256, smem, st>>>(ao, W, H, vertical, gate);
            else if (lines == 2) k_blur_inplace<2><<<blocks(count, 2), 256, smem, st>>>(ao, W, H, vertical, gate);
            else k_blur_inplace<1><<<blocks(count, 1), 256, smem, st>>>(ao, W, H, vertical, gate);
        };
        walk(lh, H, smh, 0);
        walk(lv, W, smv, 1);
        launches += 2;
    }
    else if (mode == 1)
    {
        k_blur_sep<<<blocks((long long)W * H, 256), 256, 0, st>>>(ao, tmp, W, H, 0, gate);
        k_blur_sep<<<blocks((long long)W * H, 256), 256, 0, st>>>(tmp, ao, W, H, 1, gate);
        launches += 2;
    }
    return FR_OK;
}

void launch_gamma8_table(float* out, cudaStream_t st) { k_gamma8_table<<<1, 256, 0, st>>>(out); }

// A kernel's argument count, from its signature.
template <typename... A>
constexpr int kernel_arg_count(void (*)(A...))
{
    return (int)sizeof...(A);
}

// The kernels of a frame that take the frame constants by value: the position of
// that argument and the kernel's argument count.
bool frame_const_param(const void* func, int& index, int& nargs)
{
    struct Entry
    {
        const void* f;
        int index, nargs;
    };
#define FR_FC_ENTRY(k, i) {reinterpret_cast<const void*>(k), i, kernel_arg_count(k)}
    static const Entry table[] = {
        FR_FC_ENTRY(k_transform_camera, 1),
        FR_FC_ENTRY(k_transform_light, 1),
        FR_FC_ENTRY(k_resolve_gbuffer, 1),
        FR_FC_ENTRY(k_lighting<false>, 1),
        FR_FC_ENTRY(k_lighting<true>, 1),
        FR_FC_ENTRY(k_forward_shade, 1),
        FR_FC_ENTRY(k_ssao_background, 0),
        FR_FC_ENTRY(k_ssao, 0),
        FR_FC_ENTRY(k_ao_features, 0),
        FR_FC_ENTRY(k_ao_features_blocks, 0),
        FR_FC_ENTRY(k_ssao_table_global, 0),
        FR_FC_ENTRY(k_ao_probe_plain, 0),
        FR_FC_ENTRY(k_ao_probe_compare, 0),
    };
#undef FR_FC_ENTRY
    for (const Entry& e : table)
        if (e.f == func)
        {
            index = e.index, nargs = e.nargs;
            return true;
        }
    return false;
}

void launch_lighting(const DevScene& S, const FrameConst& F, GBuffer gb, const float* shadow, unsigned* frame8,
                     float* frameF, cudaStream_t st, const int* counters, int* statusOut)
{
    const int g = blocks((long long)F.W * F.H, 128);
    if (S.texLinear) k_lighting<true><<<g, 128, 0, st>>>(S, F, gb, shadow, frame8, frameF, counters, statusOut);
    else k_lighting<false><<<g, 128, 0, st>>>(S, F, gb, shadow, frame8, frameF, counters, statusOut);
}

void launch_ssaa(int W, int H, int k, const unsigned* frame8, unsigned* out, cudaStream_t st)
{
    long long n = (long long)(W / k) * (H / k);
    if (n > 0) k_ssaa<<<blocks(n, 256), 256, 0, st>>>(W, H, k, frame8, out);
}

void launch_unpack_gbuffer(const DevScene& S, GBuffer gb, int W, int H, int which, float* out, cudaStream_t st)
{
    k_unpack<<<blocks((long long)W * H, 256), 256, 0, st>>>(S, gb, W * H, which, out);
}

void launch_pack_rgb(const unsigned* in, uint8_t* out, int n, cudaStream_t st)
{
    if (n > 0) k_pack_rgb<<<blocks(n, kPackPixels), 256, 0, st>>>(in, out, n);
}

void launch_triangle_ids(const unsigned long long* keys, int n, int* out, cudaStream_t st)
{
    k_tri_ids<<<blocks(n, 256), 256, 0, st>>>(keys, n, out);
}

void set_shadow_tables(const float* blocker, int nb, const float* pcfxy, int np, cudaStream_t st)
{
    cudaMemcpyToSymbolAsync(c_blocker, blocker, sizeof(float) * 2 * nb, 0, cudaMemcpyHostToDevice, st);
    cudaMemcpyToSymbolAsync(c_pcf, pcfxy, sizeof(float) * 2 * np, 0, cudaMemcpyHostToDevice, st);
}

}  // namespace frk
