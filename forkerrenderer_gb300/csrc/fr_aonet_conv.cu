// tcgen05 BF16 implicit-GEMM 3x3 convolutions of the learned-AO U-Net:
// forward / backward-data (k_conv3x3) and backward-weights (k_wgrad).
//
// Both kernels are persistent and warp-specialised (192 threads):
//   warp 0      TMA producer (one lane): halo tiles into a shared-memory ring
//   warp 1      MMA issuer (one lane) and TMEM owner
//   warps 2..5  epilogue: TMEM -> registers -> global
#include <cfloat>
#include <cuda_bf16.h>

#include "fr_aonet_conv.cuh"
#include "fr_aonet_ew.cuh"
#include "fr_tc.cuh"

namespace fra
{
namespace
{

constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s: far above any legitimate wait
constexpr uint32_t kSleepHintNs = 100000;     // longest hardware sleep of one poll
constexpr int kHeadParamsMax = 68;            // 1x1 head: w[4][16], b[4]

struct SyncState
{
    uint64_t full[kMaxStages];
    uint64_t empty[kMaxStages];
    uint64_t tfull[2];
    uint64_t tempty[2];
    uint64_t wbar;
    uint64_t done;
    uint32_t tmem;
    int abort;
};

// Bounded wait. Gives up when another thread of the CTA aborted, or after kWaitNs
// (then it aborts the CTA and sets status bit 2).
__device__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort, int* status)
{
    if (frtc::mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = frtc::global_timer_ns();
    // sleep in hardware between polls so waiting threads leave the issue slots to the others
    while (!frtc::mbar_try_wait_sleep(bar, parity, kSleepHintNs))
    {
        if (*abort) return false;
        if (frtc::global_timer_ns() - t0 > kWaitNs)
        {
            *abort = 1;
            atomicOr(status, 2);
            return false;
        }
    }
    return true;
}

// Barriers of one CTA: the halo ring, the two TMEM buffers, weights, done.
__device__ __forceinline__ void init_sync(SyncState& sy)
{
    if (threadIdx.x == 0)
    {
        for (int s = 0; s < kMaxStages; ++s)
        {
            frtc::mbar_init(&sy.full[s], 1);
            frtc::mbar_init(&sy.empty[s], 1);
        }
        for (int b = 0; b < 2; ++b)
        {
            frtc::mbar_init(&sy.tfull[b], 1);
            frtc::mbar_init(&sy.tempty[b], 4);
        }
        frtc::mbar_init(&sy.wbar, 1);
        frtc::mbar_init(&sy.done, 1);
        sy.abort = 0;
        frtc::fence_mbar_init();
    }
}

__device__ __forceinline__ uint32_t tmem_cols(int cols)
{
    return cols <= 32 ? 32u : cols <= 64 ? 64u : cols <= 128 ? 128u : cols <= 256 ? 256u : 512u;
}

__device__ __forceinline__ void decode_tile(int tile, int tilesX, int tilesY, int& b, int& tx, int& ty)
{
    const int per = tilesX * tilesY;
    b = tile / per;
    const int r = tile - b * per;
    ty = r / tilesX;
    tx = r - ty * tilesX;
}

__device__ __forceinline__ int tap_offset(int t)  // byte offset of tap t inside a halo plane
{
    return ((t / 3) * kHaloW + (t % 3)) * 16;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// Paired-tap schedule for an 8-channel input: K step p covers taps kPairA[p] and
// kPairB[p] (the second 8 K-elements read the pixel that tap B reads). The last
// step repeats tap 7 with zero weights.
__constant__ int kPairA[5] = {0, 2, 4, 6, 7};
__constant__ int kPairB[5] = {1, 3, 5, 7, 8};

__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Tiles are 8 x (16 * mb) pixels: mb M-blocks of 128 rows share one halo load,
// one pipeline stage and one accumulator buffer (mb * cout TMEM columns).

// The shared-memory ring of halo tiles, after the weight region.
struct ConvRing
{
    unsigned char* sW;      // the layer's packed weights
    unsigned char* sStage;  // ring slot i at sStage + i * stageBytes
    uint32_t stageBytes;
    int stages;
};

// Each role's running count of tiles (ring slots, TMEM buffers and barrier
// phases follow from it); kept across the layers of one CTA.
struct RoleCounters
{
    int issued = 0;  // TMA producer lane
    int mma = 0;     // MMA lane
    int epi = 0;     // epilogue threads
};

// One layer's tiles on this CTA: warp 0 lane 0 loads halo tiles, warp 1 lane 0
// issues the MMAs (after the weights, wbar phase wParity), warps 2..5 run the
// epilogue. The weights are already being loaded, bias / head are in shared memory.
__device__ __forceinline__ void conv_layer(const CUtensorMap* map0, const CUtensorMap* map1, const ConvArgs& a,
                                           const ConvRing& R, SyncState& sy, uint32_t tmem, uint32_t wParity,
                                           const float* sBias, const float* sHead, RoleCounters& rc)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cin = a.c0 + a.c1;
    const bool paired = (cin == 8);
    const int MB = a.mb;
    const int tileH = kTileH * MB;
    const uint32_t planeBytes = static_cast<uint32_t>(kHaloW * (tileH + 2) * 16);
    const uint32_t loadBytes = static_cast<uint32_t>(cin / 8) * planeBytes;
    const uint32_t accCols = static_cast<uint32_t>(MB * a.cout);
    volatile int* abortp = &sy.abort;

    if (warp == 0)
    {
        if (lane == 0)
        {
            for (int tile = blockIdx.x; tile < a.numTiles; tile += gridDim.x, ++rc.issued)
            {
                const int s = rc.issued % R.stages;
                const uint32_t ph = (rc.issued / R.stages) & 1;
                if (rc.issued >= R.stages && !wait_or_abort(&sy.empty[s], ph ^ 1, abortp, a.status)) break;
                int b, tx, ty;
                decode_tile(tile, a.tilesX, a.tilesY, b, tx, ty);
                unsigned char* dst = R.sStage + s * R.stageBytes;
                frtc::mbar_expect_tx(&sy.full[s], loadBytes);
                frtc::tma_load_3d(dst, map0, 8 * (tx * kTileW - 1), ty * tileH - 1, b * (a.c0 / 8), &sy.full[s]);
                if (a.c1)
                    frtc::tma_load_3d(dst + (a.c0 / 8) * planeBytes, map1, 8 * (tx * kTileW - 1), ty * tileH - 1,
                                      b * (a.c1 / 8), &sy.full[s]);
            }
        }
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            const uint32_t idesc = frtc::idesc_bf16_f32(128, a.cout, 0, 0);
            const uint32_t wBase = frtc::smem_u32(R.sW);
            const uint32_t bLbo = static_cast<uint32_t>(a.cout) * 16u;
            // Descriptor constants hoisted out of the tile loop: per MMA only the
            // start addresses change (a few integer ops, so issue keeps up with
            // the tensor pipe).
            const uint64_t bHi = frtc::smem_desc_hi(bLbo, 128);
            const uint64_t aHi = frtc::smem_desc_hi(planeBytes, kRowBytes);
            const uint32_t bTapStride = static_cast<uint32_t>(cin / 8) * bLbo;
            const int kc = cin / 16;
            bool ok = wait_or_abort(&sy.wbar, wParity, abortp, a.status);
            for (int tile = blockIdx.x; ok && tile < a.numTiles; tile += gridDim.x, ++rc.mma)
            {
                const int it = rc.mma;
                const int s = it % R.stages;
                if (!wait_or_abort(&sy.full[s], (it / R.stages) & 1, abortp, a.status)) break;
                const int buf = it & 1;
                if (it >= 2 && !wait_or_abort(&sy.tempty[buf], ((it >> 1) & 1) ^ 1, abortp, a.status)) break;
                frtc::tc_fence_after();
                const uint32_t stageAddr = frtc::smem_u32(R.sStage + s * R.stageBytes);
                for (int mb = 0; mb < MB; ++mb)
                {
                    const uint32_t d = tmem + static_cast<uint32_t>(buf) * accCols + static_cast<uint32_t>(mb * a.cout);
                    const uint32_t aBase = stageAddr + static_cast<uint32_t>(mb * kTileH) * kRowBytes;
                    if (paired)
                    {
#pragma unroll
                        for (int p = 0; p < 5; ++p)
                        {
                            constexpr int pa[5] = {0, 2, 4, 6, 7};
                            constexpr int pb[5] = {1, 3, 5, 7, 8};
                            const uint32_t oa = ((pa[p] / 3) * kHaloW + pa[p] % 3) * 16;
                            const uint32_t ob = ((pb[p] / 3) * kHaloW + pb[p] % 3) * 16;
                            const uint64_t ad = frtc::smem_desc_hi(ob - oa, kRowBytes) | ((aBase + oa) >> 4);
                            const uint64_t bd = bHi | ((wBase + static_cast<uint32_t>(p * 2) * bLbo) >> 4);
                            frtc::mma_bf16(d, ad, bd, idesc, p > 0);
                        }
                    }
                    else
                    {
#pragma unroll
                        for (int t = 0; t < 9; ++t)
                        {
                            const uint32_t aTap = aBase + static_cast<uint32_t>(((t / 3) * kHaloW + t % 3) * 16);
                            const uint32_t bTap = wBase + static_cast<uint32_t>(t) * bTapStride;
                            for (int j = 0; j < kc; ++j)
                            {
                                const uint64_t ad = aHi | ((aTap + static_cast<uint32_t>(2 * j) * planeBytes) >> 4);
                                const uint64_t bd = bHi | ((bTap + static_cast<uint32_t>(2 * j) * bLbo) >> 4);
                                frtc::mma_bf16(d, ad, bd, idesc, (t | j) != 0);
                            }
                        }
                    }
                }
                frtc::mma_commit(&sy.empty[s]);
                frtc::mma_commit(&sy.tfull[buf]);
            }
        }
    }
    else
    {
        const int q = warp & 3;  // TMEM lane quarter of this warp
        const int row = q * 32 + lane;
        const int lx = row & 7, ly = row >> 3;
        const int co8 = a.co0 / 8;
        const int c1n = (a.cout - a.co0) / 8;
        const uint32_t HW = static_cast<uint32_t>(a.H) * static_cast<uint32_t>(a.W);
        for (int tile = blockIdx.x; tile < a.numTiles; tile += gridDim.x, ++rc.epi)
        {
            const int it = rc.epi;
            const int buf = it & 1;
            int ok = 1;
            if (lane == 0) ok = wait_or_abort(&sy.tfull[buf], (it >> 1) & 1, abortp, a.status);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            frtc::tc_fence_after();
            int b, tx, ty;
            decode_tile(tile, a.tilesX, a.tilesY, b, tx, ty);
            const int x = tx * kTileW + lx;
            for (int mb = 0; mb < MB; ++mb)
            {
                const int y = ty * tileH + mb * kTileH + ly;
                const bool valid = x < a.W && y < a.H;
                const uint32_t pix = static_cast<uint32_t>(y) * static_cast<uint32_t>(a.W) + static_cast<uint32_t>(x);
                const uint32_t tb = tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(buf) * accCols +
                                    static_cast<uint32_t>(mb * a.cout);
                float z[4] = {0.f, 0.f, 0.f, 0.f};
                for (int g = 0; g < a.cout / 16; ++g)
                {
                    float v[16];
                    frtc::tmem_ld16(tb + g * 16, v);
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                    {
                        const int cc = 2 * g + h;
                        float o[8];
                        if (!a.backward)
                        {
#pragma unroll
                            for (int e = 0; e < 8; ++e) o[e] = fmaxf(v[8 * h + e] + sBias[cc * 8 + e], 0.f);
                        }
                        else
                        {
#pragma unroll
                            for (int e = 0; e < 8; ++e) o[e] = v[8 * h + e];
                            if (a.mask && valid)
                            {
                                const uint32_t moff = ((static_cast<uint32_t>(b) * (a.cout / 8) + cc) * HW + pix) * 8;
                                const uint4 m = *reinterpret_cast<const uint4*>(a.mask + moff);
                                const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
                                for (int e = 0; e < 8; ++e)
                                {
                                    const float mv = (e & 1) ? bf16_hi(mw[e >> 1]) : bf16_lo(mw[e >> 1]);
                                    if (!(mv > 0.f)) o[e] = 0.f;
                                }
                            }
                        }
                        uint4 pk;
                        pk.x = pack_bf16x2(o[0], o[1]);
                        pk.y = pack_bf16x2(o[2], o[3]);
                        pk.z = pack_bf16x2(o[4], o[5]);
                        pk.w = pack_bf16x2(o[6], o[7]);
                        if (a.head)
                        {
                            const uint32_t pw[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
                            for (int e = 0; e < 8; ++e)
                            {
                                const float hv = (e & 1) ? bf16_hi(pw[e >> 1]) : bf16_lo(pw[e >> 1]);
#pragma unroll
                                for (int k = 0; k < 4; ++k) z[k] += sHead[k * 16 + cc * 8 + e] * hv;
                            }
                        }
                        if (valid)
                        {
                            if (cc < co8)
                                *reinterpret_cast<uint4*>(
                                    a.out0 + ((static_cast<uint32_t>(b) * co8 + cc) * HW + pix) * 8) = pk;
                            else if (a.out1)
                                *reinterpret_cast<uint4*>(
                                    a.out1 + ((static_cast<uint32_t>(b) * c1n + (cc - co8)) * HW + pix) * 8) = pk;
                        }
                    }
                }
                if (a.head && valid)
                {
                    // the block's four sub-pixels of the full-resolution AO
                    const uint32_t W2 = 2u * static_cast<uint32_t>(a.W);
                    float* o = a.ao + static_cast<uint32_t>(b) * 4u * HW + (2u * static_cast<uint32_t>(y)) * W2 +
                               2u * static_cast<uint32_t>(x);
                    float v[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) v[k] = 1.f / (1.f + expf(-(z[k] + sHead[64 + k])));
                    if (a.bg16)
                    {
                        // background pixels: the plain SSAO's per-noise-cell value
                        const uint32_t X0 = 2u * static_cast<uint32_t>(x), Y0 = 2u * static_cast<uint32_t>(y);
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                        {
                            const uint32_t px = X0 + (k & 1), py = Y0 + (k >> 1);
                            if (a.bgDepth[py * W2 + px] == FLT_MAX) v[k] = a.bg16[(py & 3u) * 4u + (px & 3u)];
                        }
                    }
                    o[0] = v[0];
                    o[1] = v[1];
                    o[W2] = v[2];
                    o[W2 + 1] = v[3];
                }
            }
            frtc::tc_fence_before();
            __syncwarp();
            if (lane == 0) frtc::mbar_arrive(&sy.tempty[buf]);
        }
    }
}

__global__ void __launch_bounds__(192) k_conv3x3(const __grid_constant__ CUtensorMap map0,
                                                 const __grid_constant__ CUtensorMap map1, const ConvArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ SyncState sy;
    __shared__ float sBias[128];
    __shared__ float sHead[kHeadParamsMax];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cin = a.c0 + a.c1;
    const int tileH = kTileH * a.mb;
    const uint32_t planeBytes = static_cast<uint32_t>(kHaloW * (tileH + 2) * 16);
    const uint32_t wAligned = (a.wbytes + 1023u) & ~1023u;
    const uint32_t stageBytes = ((static_cast<uint32_t>(cin / 8) * planeBytes) + 1023u) & ~1023u;
    const ConvRing R{smem, smem + wAligned, stageBytes, a.stages};
    const uint32_t allocCols = tmem_cols(2 * a.mb * a.cout);

    // Prologue, independent of the previous kernel's outputs: barriers, TMEM,
    // the weights (never written by the kernel launched just before).
    init_sync(sy);
    if (warp == 1) frtc::tmem_alloc(&sy.tmem, allocCols);
    frtc::tc_fence_before();
    __syncthreads();
    frtc::tc_fence_after();
    if (threadIdx.x == 0)
    {
        frtc::mbar_expect_tx(&sy.wbar, a.wbytes);
        frtc::bulk_load(R.sW, a.wpacked, a.wbytes, &sy.wbar);
    }
    // From here on the previous kernel's outputs are read (no-op without a programmatic launch).
    griddep_wait();
    for (int i = threadIdx.x; i < a.cout; i += blockDim.x) sBias[i] = a.bias ? a.bias[i] : 0.f;
    if (a.head && threadIdx.x < kHeadParamsMax) sHead[threadIdx.x] = a.head[threadIdx.x];
    __syncthreads();
    const uint32_t tmem = sy.tmem;
    RoleCounters rc;
    conv_layer(&map0, &map1, a, R, sy, tmem, 0, sBias, sHead, rc);
    if (warp == 0 && lane == 0)
    {
        // Every issued copy must land before the CTA exits.
        for (int i = rc.issued - R.stages; i < rc.issued; ++i)
            if (i >= 0) frtc::mbar_wait(&sy.full[i % R.stages], (i / R.stages) & 1, kWaitNs);
        frtc::mbar_wait(&sy.wbar, 0, kWaitNs);
    }
    else if (warp == 1 && lane == 0)
    {
        // All MMAs of this thread complete before TMEM is released.
        frtc::mma_commit(&sy.done);
        frtc::mbar_wait(&sy.done, 0, kWaitNs);
        griddep_launch();
    }
    frtc::tc_fence_before();
    __syncthreads();
    if (warp == 1)
    {
        frtc::tc_fence_after();
        frtc::tmem_dealloc(tmem, allocCols);
    }
}

// Grid-wide barrier of the fused forward (all CTAs co-resident: cooperative
// launch). A CTA whose pipeline gave up raises the failure flag before it
// arrives; a barrier that waits longer than waitNs raises it too. Returns false
// when the flag is set (every CTA then leaves the stage loop).
__device__ bool grid_barrier(unsigned* sync, int* status, volatile int* abortp, uint64_t waitNs)
{
    __shared__ int failed;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        if (*abortp) atomicExch(sync + 2, 1u);
        // this CTA's stores are ordered before the other CTAs' later TMA reads
        frtc::fence_proxy_async_global();
        __threadfence();
        volatile unsigned* gen = sync + 1;
        const unsigned g = *gen;
        __threadfence();  // the generation is read before this CTA arrives
        if (atomicAdd(sync, 1u) == gridDim.x - 1)
        {
            atomicExch(sync, 0u);
            __threadfence();
            atomicAdd(sync + 1, 1u);
        }
        else
        {
            const uint64_t t0 = frtc::global_timer_ns();
            while (*gen == g)
            {
                __nanosleep(256);
                if (frtc::global_timer_ns() - t0 > waitNs)
                {
                    atomicOr(status, 4);
                    atomicExch(sync + 2, 1u);
                    break;
                }
            }
        }
        __threadfence();
        frtc::fence_proxy_async_global();
        failed = *reinterpret_cast<volatile unsigned*>(sync + 2) != 0u;
    }
    __syncthreads();
    return !failed;
}

// The whole U-Net forward in one launch: one CTA per SM runs every stage of
// U.stage in order, with a grid barrier after each.
__global__ void __launch_bounds__(192, 1) k_unet_fwd(const __grid_constant__ UnetArgs U)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ SyncState sy;
    __shared__ float sBias[128];
    __shared__ float sHead[kHeadParamsMax];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    init_sync(sy);
    if (warp == 1) frtc::tmem_alloc(&sy.tmem, U.tmemCols);
    frtc::tc_fence_before();
    __syncthreads();
    frtc::tc_fence_after();
    const uint32_t tmem = sy.tmem;
    const ConvRing R{smem, smem + U.wRegion, U.stageBytes, U.ringStages};
    RoleCounters rc;
    int convs = 0;
    const int nthreads = gridDim.x * blockDim.x;
    for (int st = 0; st < U.nStages; ++st)
    {
        const UnetStage& S = U.stage[st];
        if (S.kind == kStageConv)
        {
            const UnetConv& C = U.conv[S.conv];
            // the previous layer's MMAs have all completed (its epilogue ran): the
            // weight region is free
            if (threadIdx.x == 0)
            {
                frtc::mbar_expect_tx(&sy.wbar, C.a.wbytes);
                frtc::bulk_load(R.sW, C.a.wpacked, C.a.wbytes, &sy.wbar);
            }
            for (int i = threadIdx.x; i < C.a.cout; i += blockDim.x) sBias[i] = C.a.bias ? C.a.bias[i] : 0.f;
            if (C.a.head && threadIdx.x < kHeadParamsMax) sHead[threadIdx.x] = C.a.head[threadIdx.x];
            __syncthreads();
            conv_layer(&C.map0, &C.map1, C.a, R, sy, tmem, static_cast<uint32_t>(convs & 1), sBias, sHead, rc);
            ++convs;
        }
        else
        {
            for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += nthreads)
            {
                if (S.kind == kStagePool)
                    pool_vec(S.in, S.out, i, S.H, S.W);
                else
                    up_vec(S.in, S.out, i, S.H, S.W);
            }
        }
        // the test hook: a CTA that never arrives (its stage is complete, nothing in flight)
        if (st == 0 && static_cast<int>(blockIdx.x) == U.absentCta) break;
        if (!grid_barrier(U.sync, U.status, &sy.abort, U.waitNs)) break;
    }
    if (warp == 0 && lane == 0)
    {
        // every issued copy has landed before the CTA exits
        for (int i = rc.issued - R.stages; i < rc.issued; ++i)
            if (i >= 0) frtc::mbar_wait(&sy.full[i % R.stages], (i / R.stages) & 1, kWaitNs);
        if (convs > 0) frtc::mbar_wait(&sy.wbar, static_cast<uint32_t>((convs - 1) & 1), kWaitNs);
    }
    else if (warp == 1 && lane == 0)
    {
        frtc::mma_commit(&sy.done);
        frtc::mbar_wait(&sy.done, 0, kWaitNs);
    }
    frtc::tc_fence_before();
    __syncthreads();
    if (warp == 1)
    {
        frtc::tc_fence_after();
        frtc::tmem_dealloc(tmem, U.tmemCols);
    }
}

__global__ void __launch_bounds__(192) k_wgrad(const __grid_constant__ CUtensorMap mapX0,
                                               const __grid_constant__ CUtensorMap mapX1,
                                               const __grid_constant__ CUtensorMap mapDY, const WgradArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ SyncState sy;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cin = a.c0 + a.c1;
    constexpr uint32_t xBytes = kWgradXPlanes * kPlaneBytes;  // 46080 = 45 KiB
    const uint32_t dyPlane = kTileW * kTileH * 16;            // 2048
    const uint32_t dyBytes = static_cast<uint32_t>(a.cout / 8) * dyPlane;
    const uint32_t stageBytes = xBytes + 8 * dyPlane;         // room for cout = 64
    const int t0 = blockIdx.y * a.tapsPerGroup;
    const int nt = min(a.tapsPerGroup, 9 - t0);
    const uint32_t allocCols = tmem_cols(a.tapsPerGroup * a.cout);

    // Planes cin/8 .. 15 of every X stage are constant: plane cin/8 holds 1.0 in
    // channel 0 (its accumulator row is the bias gradient), the rest are zero.
    for (int s = 0; s < kWgradStages; ++s)
    {
        uint32_t* p = reinterpret_cast<uint32_t*>(smem + s * stageBytes + (cin / 8) * kPlaneBytes);
        const int words = (kWgradXPlanes - cin / 8) * kPlaneBytes / 4;
        for (int i = threadIdx.x; i < words; i += blockDim.x)
            p[i] = (i < kPlaneBytes / 4 && (i & 3) == 0) ? 0x3F80u : 0u;
    }
    frtc::fence_proxy_async_smem();
    if (threadIdx.x == 0)
    {
        for (int s = 0; s < kMaxStages; ++s)
        {
            frtc::mbar_init(&sy.full[s], 1);
            frtc::mbar_init(&sy.empty[s], 1);
        }
        frtc::mbar_init(&sy.done, 1);
        sy.abort = 0;
        frtc::fence_mbar_init();
    }
    if (warp == 1) frtc::tmem_alloc(&sy.tmem, allocCols);
    frtc::tc_fence_before();
    __syncthreads();
    frtc::tc_fence_after();
    const uint32_t tmem = sy.tmem;
    volatile int* abortp = &sy.abort;
    const int ntiles = blockIdx.x < a.numTiles ? (a.numTiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (warp == 0)
    {
        if (lane == 0)
        {
            const uint32_t loadBytes = static_cast<uint32_t>(cin / 8) * kPlaneBytes + dyBytes;
            int issued = 0;
            for (int tile = blockIdx.x; tile < a.numTiles; tile += gridDim.x, ++issued)
            {
                const int s = issued % kWgradStages;
                const uint32_t ph = (issued / kWgradStages) & 1;
                if (issued >= kWgradStages && !wait_or_abort(&sy.empty[s], ph ^ 1, abortp, a.status)) break;
                int b, tx, ty;
                decode_tile(tile, a.tilesX, a.tilesY, b, tx, ty);
                unsigned char* dst = smem + s * stageBytes;
                frtc::mbar_expect_tx(&sy.full[s], loadBytes);
                frtc::tma_load_3d(dst, &mapX0, 8 * (tx * kTileW - 1), ty * kTileH - 1, b * (a.c0 / 8), &sy.full[s]);
                if (a.c1)
                    frtc::tma_load_3d(dst + (a.c0 / 8) * kPlaneBytes, &mapX1, 8 * (tx * kTileW - 1), ty * kTileH - 1,
                                      b * (a.c1 / 8), &sy.full[s]);
                frtc::tma_load_3d(dst + xBytes, &mapDY, 8 * tx * kTileW, ty * kTileH, b * (a.cout / 8), &sy.full[s]);
            }
            for (int i = issued - kWgradStages; i < issued; ++i)
                if (i >= 0) frtc::mbar_wait(&sy.full[i % kWgradStages], (i / kWgradStages) & 1, kWaitNs);
        }
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            const uint32_t idesc = frtc::idesc_bf16_f32(128, a.cout, 1, 1);
            int it = 0;
            for (int tile = blockIdx.x; tile < a.numTiles; tile += gridDim.x, ++it)
            {
                const int s = it % kWgradStages;
                if (!wait_or_abort(&sy.full[s], (it / kWgradStages) & 1, abortp, a.status)) break;
                frtc::tc_fence_after();
                const uint32_t xb = frtc::smem_u32(smem + s * stageBytes);
                const uint32_t yb = xb + xBytes;
                constexpr uint64_t aHi = frtc::smem_desc_hi(kRowBytes, kPlaneBytes);
                const uint64_t bHi = frtc::smem_desc_hi(128u, dyPlane);
                for (int tt = 0; tt < nt; ++tt)
                {
                    const int t = t0 + tt;
                    const uint32_t d = tmem + static_cast<uint32_t>(tt * a.cout);
                    const uint32_t aTap = xb + static_cast<uint32_t>(((t / 3) * kHaloW + (t % 3)) * 16);
#pragma unroll
                    for (int j = 0; j < kTileH / 2; ++j)
                    {
                        // A: rows = input channels (MN-major), K = 16 pixels = halo rows 2j+dy, 2j+1+dy.
                        const uint64_t ad = aHi | ((aTap + static_cast<uint32_t>(2 * j * kRowBytes)) >> 4);
                        // B: rows = output channels (MN-major), K = the same 16 output pixels.
                        const uint64_t bd = bHi | ((yb + static_cast<uint32_t>(2 * j) * 128u) >> 4);
                        frtc::mma_bf16(d, ad, bd, idesc, (it | j) != 0);
                    }
                }
                frtc::mma_commit(&sy.empty[s]);
            }
            frtc::mma_commit(&sy.done);
            frtc::mbar_wait(&sy.done, 0, kWaitNs);
        }
    }
    else
    {
        const int q = warp & 3;
        const int row = q * 32 + lane;  // input channel (row cin: bias)
        int ok = 1;
        if (lane == 0) ok = wait_or_abort(&sy.done, 0, abortp, a.status);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        frtc::tc_fence_after();
        const size_t base =
            ((static_cast<size_t>(blockIdx.y) * gridDim.x + blockIdx.x) * a.tapsPerGroup) * (cin + 1);
        for (int tt = 0; tt < nt; ++tt)
            for (int g = 0; g < a.cout / 16; ++g)
            {
                float v[16];
                frtc::tmem_ld16(tmem + (static_cast<uint32_t>(q * 32) << 16) +
                                    static_cast<uint32_t>(tt * a.cout + g * 16),
                                v);
                if (row <= cin)
                {
                    float* dst = a.partial + ((base + static_cast<size_t>(tt) * (cin + 1) + row) * a.cout + g * 16);
#pragma unroll
                    for (int i = 0; i < 16; ++i) dst[i] = (ok && ntiles > 0) ? v[i] : 0.f;
                }
            }
    }
    frtc::tc_fence_before();
    __syncthreads();
    if (warp == 1)
    {
        frtc::tc_fence_after();
        frtc::tmem_dealloc(tmem, allocCols);
    }
}

}  // namespace

// Opt-in limit for the dynamic shared memory of both kernels: the 227 KiB
// per-block maximum minus room for their static shared memory.
constexpr int kMaxDynSmem = 220 * 1024;

uint32_t conv_smem_bytes(int cin, int cout, int stages, bool paired, int mb)
{
    const uint32_t wbytes = paired ? 5u * 2u * 8u * cout * 2u : 9u * cin * cout * 2u;
    const uint32_t w = (wbytes + 1023u) & ~1023u;
    const uint32_t plane = static_cast<uint32_t>(kHaloW * (kTileH * mb + 2) * 16);
    const uint32_t stage = (static_cast<uint32_t>(cin / 8) * plane + 1023u) & ~1023u;
    return w + stage * stages;
}

uint32_t wgrad_smem_bytes(int /*cout*/)
{
    return kWgradStages * (kWgradXPlanes * kPlaneBytes + 8 * kTileW * kTileH * 16);
}

void launch_conv3x3(const CUtensorMap& map0, const CUtensorMap& map1, const ConvArgs& a, int grid, uint32_t smem,
                    cudaStream_t st, bool programmatic)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
        attr = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(192);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = programmatic ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k_conv3x3, map0, map1, a);
}

void unet_attributes()
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_unet_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
        attr = true;
    }
}

int unet_fwd_ctas_per_sm(uint32_t smem)
{
    unet_attributes();
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_unet_fwd, 192, smem) != cudaSuccess) return 0;
    return nb;
}

cudaError_t launch_unet_fwd(const UnetArgs& u, int grid, uint32_t smem, cudaStream_t st)
{
    unet_attributes();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(192);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_unet_fwd, u);
}

void launch_wgrad(const CUtensorMap& mapX0, const CUtensorMap& mapX1, const CUtensorMap& mapDY, const WgradArgs& a,
                  int gridX, int gridY, uint32_t smem, cudaStream_t st)
{
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
        attr = true;
    }
    k_wgrad<<<dim3(gridX, gridY), 192, smem, st>>>(mapX0, mapX1, mapDY, a);
}

}  // namespace fra
