// C ABI of include/forkerrenderer.h: render context, scene upload, the frame's
// pass sequence (Render::Render, src/render.cpp:40-58) and read-back in the
// reference's buffer layouts.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fr_aonet.h"
#include "fr_aonet_internal.h"
#include "fr_context_internal.h"
#include "fr_hostmath.h"
#include "fr_kernels.cuh"
#include "fr_sample_tables.h"
#include "fr_scene_internal.h"
#include "forkerrenderer.h"

namespace
{

int fail(fr_ctx* c, int code, const std::string& m)
{
    if (c) c->err = m;
    return code;
}

int cuda_check(fr_ctx* c, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return FR_OK;
    if (e == cudaErrorMemoryAllocation)
        return fail(c, FR_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(c, FR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define FR_CUDA(call)                                         \
    do                                                        \
    {                                                         \
        int _rc = cuda_check(ctx, (call), #call);             \
        if (_rc != FR_OK) return _rc;                         \
    } while (0)

template <typename T>
int upload(fr_ctx* ctx, T*& dst, const void* src, size_t bytes)
{
    void* p = nullptr;
    FR_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
    ctx->sceneBufs.push_back(FrDevBuf{p, bytes});
    if (bytes) FR_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    dst = reinterpret_cast<T*>(p);
    return FR_OK;
}

void free_scene(fr_ctx* ctx)
{
    for (auto& b : ctx->sceneBufs) cudaFree(b.p);
    ctx->sceneBufs.clear();
    ctx->hasScene = false;
}

// The kernel nodes of captured graph g that take the frame constants (fr_ctx::fcNodes).
bool collect_fc_nodes(fr_ctx* ctx, cudaGraph_t g)
{
    ctx->fcNodes.clear();
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return false;
    std::vector<cudaGraphNode_t> nodes(n);
    if (n && cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return false;
    for (cudaGraphNode_t node : nodes)
    {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(node, &t) != cudaSuccess) return false;
        if (t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams p;
        if (cudaGraphKernelNodeGetParams(node, &p) != cudaSuccess) return false;
        int index = 0, nargs = 0;
        if (!frk::frame_const_param(p.func, index, nargs)) continue;
        if (!p.kernelParams || nargs > 16) return false;
        ctx->fcNodes.push_back(fr_ctx::FcNode{node, p, index, nargs});
    }
    return true;
}

void drop_graph(fr_ctx* ctx)
{
    if (ctx->graphExec) cudaGraphExecDestroy(ctx->graphExec);
    ctx->graphExec = nullptr;
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->graph = nullptr;
    ctx->fcNodes.clear();
}

void free_frame(fr_ctx* ctx)
{
    drop_graph(ctx);  // its kernels address these buffers
    ctx->lastKeyValid = false;
    for (void* p : ctx->frameAllocs) cudaFree(p);
    ctx->frameAllocs.clear();
    ctx->W = ctx->H = ctx->SW = ctx->SH = 0;
    ctx->aoFeat = nullptr;
    ctx->aoFeatCap = 0;
    ctx->probePart = nullptr;
    ctx->probePlain = nullptr;
    ctx->probePartCap = 0;
    ctx->ssaoTblGlobal = nullptr;
}

template <typename T>
int falloc(fr_ctx* ctx, T*& dst, size_t count)
{
    void* p = nullptr;
    FR_CUDA(cudaMalloc(&p, sizeof(T) * (count ? count : 1)));
    ctx->frameAllocs.push_back(p);
    dst = reinterpret_cast<T*>(p);
    return FR_OK;
}

#define FR_TRY(x)                \
    do                           \
    {                            \
        int _rc = (x);           \
        if (_rc != FR_OK) return _rc; \
    } while (0)

int tiles_of(int w, int h) { return ((w + frk::kTile - 1) / frk::kTile) * ((h + frk::kTile - 1) / frk::kTile); }

int ensure_frame(fr_ctx* ctx, int W, int H, int SW, int SH)
{
    if (W == ctx->W && H == ctx->H && SW == ctx->SW && SH == ctx->SH) return FR_OK;
    // pixel and texel indices are 32-bit in the kernels
    if (W < 1 || H < 1 || SW < 0 || SH < 0 || (long long)W * H > (1ll << 30) || (long long)SW * SH > (1ll << 30))
        return fail(ctx, FR_ERR_INVALID, "the working frame and the shadow map must each hold at most 2^30 pixels");
    free_frame(ctx);
    const size_t P = (size_t)W * H, SP = (size_t)SW * SH;
    const int V = ctx->S.numVerts, N = ctx->S.numNormals, T = ctx->S.numTris;
    FR_TRY(falloc(ctx, ctx->vo.scr, V));
    FR_TRY(falloc(ctx, ctx->vo.pw, V));
    FR_TRY(falloc(ctx, ctx->vo.lw, V));
    FR_TRY(falloc(ctx, ctx->vo.tw, V));
    FR_TRY(falloc(ctx, ctx->vo.npre, N));
    FR_TRY(falloc(ctx, ctx->scrL, V));
    // The shadow and camera passes each have their own visibility keys, triangle
    // lists and tile bins: in deferred frames they run at the same time.
    ctx->keysCap = P;
    FR_TRY(falloc(ctx, ctx->keys, P));
    FR_TRY(falloc(ctx, ctx->keysShadow, SP > 0 ? SP : 1));
    FR_TRY(falloc(ctx, ctx->counters, 8));
    auto scratch = [&](frk::RasterScratch& rs, unsigned long long* keys, int tiles, int* counters) -> int {
        const long long binCap =
            ctx->cfg.bin_capacity > 0 ? ctx->cfg.bin_capacity : (long long)tiles * 16 + (1 << 22);
        rs = frk::RasterScratch{};
        rs.keys = keys;
        rs.counters = counters;
        rs.triCap = T > 0 ? T : 1;
        rs.binCap = binCap;
        FR_TRY(falloc(ctx, rs.mediumTris, rs.triCap));
        FR_TRY(falloc(ctx, rs.mediumIdx, rs.triCap));
        FR_TRY(falloc(ctx, rs.largeTris, rs.triCap));
        FR_TRY(falloc(ctx, rs.largeIdx, rs.triCap));
        FR_TRY(falloc(ctx, rs.largeAux, rs.triCap));
        FR_TRY(falloc(ctx, rs.tileCount, tiles));
        FR_TRY(falloc(ctx, rs.tileStart, tiles + 1));
        FR_TRY(falloc(ctx, rs.tileFill, tiles));
        FR_TRY(falloc(ctx, rs.binTri, (size_t)binCap));
        return FR_OK;
    };
    FR_TRY(scratch(ctx->rsShadow, ctx->keysShadow, tiles_of(SW, SH) > 0 ? tiles_of(SW, SH) : 1, ctx->counters));
    // the shadow map's fused resolve reads each winning triangle's record (one load round trip)
    FR_TRY(falloc(ctx, ctx->rsShadow.triRec, 2 * (size_t)ctx->rsShadow.triCap));
    FR_TRY(scratch(ctx->rsCam, ctx->keys, tiles_of(W, H), ctx->counters + 4));
    FR_TRY(falloc(ctx, ctx->gb.a, P));
    FR_TRY(falloc(ctx, ctx->gb.b, P));
    FR_TRY(falloc(ctx, ctx->gb.c, P));
    FR_TRY(falloc(ctx, ctx->gb.depth, P));
    FR_TRY(falloc(ctx, ctx->gb.ao, P));
    FR_TRY(falloc(ctx, ctx->shadow, SP));
    FR_TRY(falloc(ctx, ctx->frame8, P));
    FR_TRY(falloc(ctx, ctx->ssaa, P));
    FR_TRY(falloc(ctx, ctx->blurTmp, P));
    FR_TRY(falloc(ctx, ctx->ssaoBg16, 16));
    if (ctx->cfg.keep_float_frame) FR_TRY(falloc(ctx, ctx->frameF, 3 * P));
    else ctx->frameF = nullptr;
    FR_CUDA(cudaMemsetAsync(ctx->counters, 0, sizeof(int) * 8, ctx->stream));
    FR_CUDA(cudaMemsetAsync(ctx->shadow, 0, sizeof(float) * SP, ctx->stream));
    // frames may run on a caller's stream and on the second stream: the cleared
    // buffers are ready before either sees them
    FR_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->W = W, ctx->H = H, ctx->SW = SW, ctx->SH = SH;
    return FR_OK;
}

// Status of the last frame's raster passes (bin / list overflow).
int check_status(fr_ctx* ctx)
{
    if (!ctx->statusPending) return FR_OK;
    FR_CUDA(cudaEventSynchronize(ctx->ev[6]));
    ctx->statusPending = false;
    int bits = ctx->hostCounters[3] | ctx->hostCounters[7];
    if (bits & frk::kStatusBinOverflow)
        return fail(ctx, FR_ERR_BIN_OVERFLOW, "tile-bin capacity exceeded: raise fr_config.bin_capacity");
    if (bits & frk::kStatusListOverflow) return fail(ctx, FR_ERR_BIN_OVERFLOW, "triangle list overflow");
    if (ctx->cfg.ao_mode == FR_AO_LEARNED && ctx->aonet && fra_take_status(ctx->aonet))
        return fail(ctx, FR_ERR_TIMEOUT, "learned AO: a bounded device wait of the network gave up");
    return FR_OK;
}

void fill_frame_const(fr_ctx* ctx, const fr_frame_matrices& m)
{
    frctx_frame_const(ctx, m, ctx->fc);
}

}  // namespace

// A zero G-buffer texel shades to black when the eye and the light are finite.
void frctx_refresh_background(frd::FrameConst& F)
{
    bool fin = true;
    for (int i = 0; i < 3; ++i)
        fin = fin && std::isfinite(F.eye[i]) && std::isfinite(F.lightPos[i]) && std::isfinite(F.lightColor[i]);
    F.bgBlack = fin ? 1 : 0;
}

// Frame constants of matrices `m` under the context's scene and configuration.
void frctx_frame_const(fr_ctx* ctx, const fr_frame_matrices& m, frd::FrameConst& F)
{
    std::memcpy(F.V, m.view, 64);
    std::memcpy(F.P, m.projection, 64);
    std::memcpy(F.VP, m.view_projection, 64);
    std::memcpy(F.L, m.light_space, 64);
    std::memcpy(F.VPort, m.viewport, 64);
    std::memcpy(F.SVPort, m.shadow_viewport, 64);
    std::memcpy(F.eye, ctx->info.eye, 12);
    std::memcpy(F.lightPos, ctx->info.light_pos, 12);
    std::memcpy(F.lightColor, ctx->info.light_color, 12);
    F.W = m.width, F.H = m.height, F.SW = m.shadow_width, F.SH = m.shadow_height;
    F.shadowOn = ctx->info.shadow_on;
    F.deferred = ctx->info.deferred;
    F.ssaoOn = ctx->info.ssao_on;
    F.shadowMode = ctx->cfg.shadow_mode;
    F.pcfN = ctx->cfg.pcf_samples;
    F.blockerN = ctx->cfg.blocker_samples;
    F.ssaoN = ctx->cfg.ssao_samples;
    F.ssaoRadius = ctx->cfg.ssao_radius;
    F.ssaoBias = ctx->cfg.ssao_bias;
    F.ssaoRange = ctx->cfg.ssao_range;
    frctx_refresh_background(F);
    const float* vm = m.viewport;
    F.vportSimple = vm[1] == 0.f && vm[2] == 0.f && vm[4] == 0.f && vm[6] == 0.f && vm[8] == 0.f && vm[9] == 0.f;
}

namespace
{

cudaStream_t stream_of(fr_ctx* ctx, const fr_frame_params* p)
{
    return (p && p->stream) ? reinterpret_cast<cudaStream_t>(p->stream) : ctx->stream;
}

// Matrices, per-model light matrices, buffers: everything a pass needs.
int begin_frame(fr_ctx* ctx, const fr_frame_params* params)
{
    if (!ctx->hasScene) return fail(ctx, FR_ERR_INVALID, "no scene uploaded");
    const fr_frame_matrices& m = (params && params->matrices) ? *params->matrices : ctx->defaultMats;
    ctx->mats = m;
    fill_frame_const(ctx, m);
    if (params && params->eye)
    {
        std::memcpy(ctx->fc.eye, params->eye, 12);
        frctx_refresh_background(ctx->fc);
    }
    cudaStream_t st = stream_of(ctx, params);
    if (!ctx->lsValid || std::memcmp(ctx->lsUsed, m.light_space, 64) != 0)
    {
        fr::M4 L;
        std::memcpy(L.m, m.light_space, 64);
        for (auto& md : ctx->hostModels)
        {
            fr::M4 M;
            std::memcpy(M.m, md.M, 64);
            fr::M4 LM = fr::mul(L, M);
            std::memcpy(md.LM, LM.m, 64);
        }
        FR_CUDA(cudaMemcpyAsync(ctx->dModels, ctx->hostModels.data(), sizeof(frd::DevModel) * ctx->hostModels.size(),
                                cudaMemcpyHostToDevice, st));
        FR_CUDA(cudaStreamSynchronize(st));  // host staging vector is reused
        std::memcpy(ctx->lsUsed, m.light_space, 64);
        ctx->lsValid = true;
    }
    FR_TRY(ensure_frame(ctx, m.width, m.height, m.shadow_width, m.shadow_height));
    return FR_OK;
}

int do_shadow(fr_ctx* ctx, cudaStream_t st)
{
    if (!ctx->info.shadow_on) return FR_OK;
    frk::launch_transform_light(ctx->S, ctx->fc, ctx->scrL, st);
    frk::RasterParams rp{ctx->SW, ctx->SH, ctx->cfg.small_tri_area, ctx->cfg.medium_tri_area};
    frk::launch_raster(ctx->S, ctx->scrL, rp, ctx->rsShadow, st, ctx->launches, true, ctx->shadow);
    ctx->launches += 1;
    FR_CUDA(cudaGetLastError());
    return FR_OK;
}

int do_camera(fr_ctx* ctx, cudaStream_t st, bool forwardPass)
{
    frk::launch_transform_camera(ctx->S, ctx->fc, ctx->vo, st);
    frk::RasterParams rp{ctx->W, ctx->H, ctx->cfg.small_tri_area, ctx->cfg.medium_tri_area};
    frk::launch_raster(ctx->S, ctx->vo.scr, rp, ctx->rsCam, st, ctx->launches);
    if (forwardPass)
        frk::launch_forward_shade(ctx->S, ctx->fc, ctx->vo, ctx->keys, ctx->shadow, ctx->gb.depth, ctx->frame8,
                                  ctx->frameF, st, ctx->counters, ctx->hostCountersDev);
    else
        frk::launch_resolve_gbuffer(ctx->S, ctx->fc, ctx->vo, ctx->keys, ctx->gb, st);
    ctx->launches += 2;
    FR_CUDA(cudaGetLastError());
    return FR_OK;
}

// Timing events: inside a stream capture they become external event-record
// nodes, so the replayed graph records them as the direct launches do.
cudaError_t record_event(fr_ctx* ctx, cudaEvent_t ev, cudaStream_t st)
{
    // without pass timings only the frame's first and last events are recorded
    if (!ctx->cfg.pass_timings && ev != ctx->ev[0] && ev != ctx->ev[6]) return cudaSuccess;
    return ctx->capturing ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal) : cudaEventRecord(ev, st);
}

// Buffers of the learned-AO path (network input, probe partials and decision).
int ensure_ao(fr_ctx* ctx, cudaStream_t st)
{
    const size_t P = (size_t)ctx->W * ctx->H;
    if (ctx->aoFeatCap < P)
    {
        FR_TRY(falloc(ctx, ctx->aoFeat, P));
        ctx->aoFeatCap = P;
    }
    const size_t nb = 2 * (size_t)frk::ao_probe_blocks(ctx->W, ctx->H) + 2;
    if (ctx->probePartCap < nb)
    {
        FR_TRY(falloc(ctx, ctx->probePart, nb));
        FR_TRY(falloc(ctx, ctx->probePlain, (size_t)(ctx->W / 8) * (ctx->H / 8) + 1));
        FR_TRY(falloc(ctx, ctx->aoGate, 1));
        FR_TRY(falloc(ctx, ctx->probeMean, 1));
        FR_TRY(falloc(ctx, ctx->probeDone, 1));
        FR_CUDA(cudaMemsetAsync(ctx->aoGate, 0, sizeof(int), st));
        FR_CUDA(cudaMemsetAsync(ctx->probeMean, 0, sizeof(float), st));
        FR_CUDA(cudaMemsetAsync(ctx->probeDone, 0, sizeof(unsigned), st));
        ctx->probePartCap = nb;
    }
    if (!ctx->ssaoTblGlobal)
    {
        // the table depends on the sample count and radius only: built once per frame size
        FR_TRY(falloc(ctx, ctx->ssaoTblGlobal, 16 * (size_t)(2 * ctx->cfg.ssao_samples + 2)));
        frk::launch_ssao_table_global(ctx->fc, ctx->ssaoTable, ctx->ssaoTblGlobal, st);
        FR_CUDA(cudaGetLastError());
    }
    return FR_OK;
}

int do_ssao(fr_ctx* ctx, cudaStream_t st, cudaEvent_t mid = nullptr)
{
    if (!ctx->info.ssao_on || !ctx->info.deferred)
    {
        if (mid) FR_CUDA(record_event(ctx, mid, st));
        return FR_OK;
    }
    if (ctx->cfg.ao_mode == FR_AO_LEARNED)
    {
        // Network AO, then the 1-in-64 probe; plain SSAO + blur run only when the
        // probe sets the gate (the gated kernels return at once otherwise).
        if (!ctx->aonet) return fail(ctx, FR_ERR_INVALID, "ao_mode is FR_AO_LEARNED but no network is attached");
        if ((ctx->W % fra::kLevelAlign) || (ctx->H % fra::kLevelAlign))
            return fail(ctx, FR_ERR_UNSUPPORTED, "learned AO needs W, H multiples of 32");
        FR_TRY(ensure_ao(ctx, st));
        // background pixels take the plain SSAO's per-noise-cell value (written by the
        // head; computed by one extra CTA of the input kernel)
        frk::launch_ao_features_blocks(ctx->fc, ctx->gb, ctx->aoFeat, st, ctx->aoInputTable, ctx->cfg.ao_input_samples,
                                       ctx->ssaoTable, ctx->ssaoBg16);
        // the probe's plain values need the G-buffer only: they run on stream3 beside
        // the network and join before the comparison
        FR_CUDA(cudaEventRecord(ctx->probeForkEv, st));
        FR_CUDA(cudaStreamWaitEvent(ctx->stream3, ctx->probeForkEv, 0));
        frk::launch_ao_probe_plain(ctx->fc, ctx->gb, ctx->ssaoTblGlobal, ctx->probePlain, ctx->stream3);
        FR_CUDA(cudaEventRecord(ctx->probeJoinEv, ctx->stream3));
        int rc = fra_forward_blocks(ctx->aonet, reinterpret_cast<const uint16_t*>(ctx->aoFeat), 1, ctx->H, ctx->W,
                                    ctx->gb.ao, st, &ctx->launches, ctx->gb.depth, ctx->ssaoBg16);
        ctx->launches += 1;
        if (rc != FR_OK)
        {
            cudaStreamWaitEvent(st, ctx->probeJoinEv, 0);  // a capture must not end with stream3 forked
            return fail(ctx, rc, std::string("network forward: ") + fr_aonet_last_error(ctx->aonet));
        }
        FR_CUDA(cudaStreamWaitEvent(st, ctx->probeJoinEv, 0));
        frk::launch_ao_probe_compare(ctx->fc, ctx->gb.ao, ctx->probePlain, ctx->cfg.ao_probe_threshold, ctx->probePart,
                                     ctx->probeDone, ctx->aoGate, ctx->probeMean, st);
        ctx->launches += 2;
        if (mid) FR_CUDA(record_event(ctx, mid, st));
        frk::launch_ssao(ctx->fc, ctx->gb, ctx->ssaoTable, ctx->ssaoBg16, st, ctx->aoGate, false);
        if (frk::launch_blur(ctx->cfg.blur_mode, ctx->W, ctx->H, ctx->gb.ao, ctx->blurTmp, st, ctx->launches,
                             ctx->aoGate, ctx->cfg.blur_warmup) != FR_OK)
            return fail(ctx, FR_ERR_UNSUPPORTED, "frame lines too long for the in-place blur");
        ctx->launches += 1;
        FR_CUDA(cudaGetLastError());
        return FR_OK;
    }
    frk::launch_ssao(ctx->fc, ctx->gb, ctx->ssaoTable, ctx->ssaoBg16, st);
    ctx->launches += 2;
    if (mid) FR_CUDA(record_event(ctx, mid, st));
    if (frk::launch_blur(ctx->cfg.blur_mode, ctx->W, ctx->H, ctx->gb.ao, ctx->blurTmp, st, ctx->launches, nullptr,
                         ctx->cfg.blur_warmup) != FR_OK)
        return fail(ctx, FR_ERR_UNSUPPORTED, "frame lines too long for the in-place blur");
    FR_CUDA(cudaGetLastError());
    return FR_OK;
}

int do_lighting(fr_ctx* ctx, cudaStream_t st)
{
    frk::launch_lighting(ctx->S, ctx->fc, ctx->gb, ctx->shadow, ctx->frame8, ctx->frameF, st, ctx->counters,
                         ctx->hostCountersDev);
    ctx->launches += 1;
    FR_CUDA(cudaGetLastError());
    return FR_OK;
}

int do_ssaa(fr_ctx* ctx, cudaStream_t st)
{
    if (!ctx->info.ssaa_on) return FR_OK;
    frk::launch_ssaa(ctx->W, ctx->H, ctx->info.ssaa_kernel, ctx->frame8, ctx->ssaa, st);
    ctx->launches += 1;
    FR_CUDA(cudaGetLastError());
    return FR_OK;
}

int set_tables(fr_ctx* ctx)
{
    const fr_config& c = ctx->cfg;
    if (c.pcf_samples < 1 || c.pcf_samples > 256 || c.blocker_samples < 1 || c.blocker_samples > 256)
        return fail(ctx, FR_ERR_INVALID, "pcf / blocker samples must be in [1, 256]");
    // the SSAO kernel holds its 16-cell sample table in shared memory (48 B a sample)
    if (c.ssao_samples < 1 || c.ssao_samples > 256)
        return fail(ctx, FR_ERR_INVALID, "ssao samples must be in [1, 256]");
    // a warp's 32 small boxes are flattened into one int-indexed pixel list, and a
    // medium triangle's box is walked by one warp
    if (c.small_tri_area < 0 || c.small_tri_area > 65536 || c.medium_tri_area < 0 || c.medium_tri_area > (1 << 20))
        return fail(ctx, FR_ERR_INVALID, "small_tri_area must be in [0, 65536], medium_tri_area in [0, 2^20]");
    std::vector<float> blk(2 * c.blocker_samples), pcf(2 * c.pcf_samples);
    fr_make_disk_table(FR_TABLE_SEED_BLOCKER, c.blocker_samples, blk.data());
    fr_make_disk_table(FR_TABLE_SEED_PCF, c.pcf_samples, pcf.data());
    // RandomVectorInUnitDisk().xy * PCSS_BLOCKER_SEARCH_FILTER_SIZE (shadow.cpp:75-76):
    // float * double, rounded back to float.
    for (float& v : blk) v = (float)((double)v * 0.005);
    frk::set_shadow_tables(blk.data(), c.blocker_samples, pcf.data(), c.pcf_samples, ctx->stream);
    std::vector<float> ssao(3 * 16 * c.ssao_samples);
    fr_make_ssao_table(c.ssao_samples, ssao.data());
    FR_CUDA(cudaMalloc(&ctx->ssaoTable, sizeof(float) * ssao.size()));
    FR_CUDA(cudaMemcpyAsync(ctx->ssaoTable, ssao.data(), sizeof(float) * ssao.size(), cudaMemcpyHostToDevice,
                            ctx->stream));
    if (c.ao_input_samples < -1 || c.ao_input_samples > 64)
        return fail(ctx, FR_ERR_INVALID, "ao input samples must be -1 (depth residual) or in [0, 64]");
    if (c.texture_wrap < 0 || c.texture_wrap > 3) return fail(ctx, FR_ERR_INVALID, "texture_wrap must be in [0, 3]");
    if (c.texture_filter < 0 || c.texture_filter > 1)
        return fail(ctx, FR_ERR_INVALID, "texture_filter must be 0 (Nearest) or 1 (Linear)");
    if (c.ao_input_samples > 0)
    {
        std::vector<float> k(3 * 16 * c.ao_input_samples);
        fr_make_ssao_table(c.ao_input_samples, k.data());
        FR_CUDA(cudaMalloc(&ctx->aoInputTable, sizeof(float) * k.size()));
        FR_CUDA(cudaMemcpyAsync(ctx->aoInputTable, k.data(), sizeof(float) * k.size(), cudaMemcpyHostToDevice,
                                ctx->stream));
    }
    FR_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->ssaoTableN = c.ssao_samples;
    return FR_OK;
}

}  // namespace

extern "C" {

void fr_config_defaults(fr_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->shadow_mode = FR_SHADOW_PCSS;
    c->shadow_size = 0;
    c->pcf_samples = 64;
    c->blocker_samples = 32;
    c->ssao_samples = 32;
    c->ssao_radius = 0.075f;
    c->ssao_bias = 0.0005f;
    c->ssao_range = 0.01f;
    c->blur_mode = FR_BLUR_REFERENCE;
    c->ao_mode = FR_AO_SSAO;
    c->keep_float_frame = 0;
    c->small_tri_area = 512;  // 128 -> 512: 10 us less on the 409,602-triangle 1280x800 deferred frame
    c->medium_tri_area = 8192;
    c->bin_capacity = 0;
    c->device = 0;
    c->ao_probe_threshold = 0.02f;
    c->ao_input_samples = 0;
    c->texture_wrap = 0;
    c->texture_filter = 0;
    c->concurrent_passes = 1;
    c->blur_warmup = 0;
    c->pass_timings = 1;
}

fr_ctx* fr_create(const fr_config* cfg, char* err, size_t errlen)
{
    auto bail = [&](const std::string& m) -> fr_ctx* {
        if (err && errlen) std::snprintf(err, errlen, "%s", m.c_str());
        return nullptr;
    };
    fr_ctx* ctx = new fr_ctx();
    if (cfg) ctx->cfg = *cfg;
    else fr_config_defaults(&ctx->cfg);
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
    {
        delete ctx;
        return bail(std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    if (ctx->cfg.device < 0 || ctx->cfg.device >= n)
    {
        delete ctx;
        return bail("bad device ordinal");
    }
    cudaSetDevice(ctx->cfg.device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete ctx;
        return bail("cudaStreamCreate failed");
    }
    // the camera chain of concurrent deferred frames: its blocks are scheduled ahead
    // of the shadow pass's, which fills the SMs it leaves idle
    int leastPri = 0, greatestPri = 0;
    cudaDeviceGetStreamPriorityRange(&leastPri, &greatestPri);
    // the learned-AO probe's plain values: at the lowest priority, they fill the SMs
    // the network's small levels leave idle
    if (cudaStreamCreateWithPriority(&ctx->stream2, cudaStreamNonBlocking, greatestPri) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->stream3, cudaStreamNonBlocking, leastPri) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->forkEv, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->joinEv, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->probeForkEv, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->probeJoinEv, cudaEventDisableTiming) != cudaSuccess)
    {
        fr_destroy(ctx);
        return bail("cudaStreamCreate / cudaEventCreate failed");
    }
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    // the frame's status words: written by the frame's shading kernel (launch_lighting /
    // launch_forward_shade), read by the host after the frame's last event
    if (cudaHostAlloc(reinterpret_cast<void**>(&ctx->hostCounters), sizeof(int) * 8, cudaHostAllocMapped) !=
            cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->hostCountersDev), ctx->hostCounters, 0) != cudaSuccess)
    {
        cudaGetLastError();
        fr_destroy(ctx);
        return bail("cudaHostAlloc (mapped status words) failed");
    }
    std::memset(ctx->hostCounters, 0, sizeof(int) * 8);
    if (set_tables(ctx) != FR_OK)
    {
        std::string m = ctx->err;
        fr_destroy(ctx);
        return bail(m);
    }
    return ctx;
}

void fr_destroy(fr_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->cfg.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
    if (ctx->stream3) cudaStreamSynchronize(ctx->stream3);
    drop_graph(ctx);
    free_frame(ctx);
    free_scene(ctx);
    frout_free(ctx);
    if (ctx->rgbBuf) cudaFree(ctx->rgbBuf);
    if (ctx->ssaoTable) cudaFree(ctx->ssaoTable);
    if (ctx->aoInputTable) cudaFree(ctx->aoInputTable);
    if (ctx->hostCounters) cudaFreeHost(ctx->hostCounters);
    for (auto& ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->forkEv) cudaEventDestroy(ctx->forkEv);
    if (ctx->joinEv) cudaEventDestroy(ctx->joinEv);
    if (ctx->probeForkEv) cudaEventDestroy(ctx->probeForkEv);
    if (ctx->probeJoinEv) cudaEventDestroy(ctx->probeJoinEv);
    if (ctx->stream3) cudaStreamDestroy(ctx->stream3);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* fr_last_error(const fr_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fr_upload_scene(fr_ctx* ctx, const fr_scene* s)
{
    if (!ctx || !s) return fail(ctx, FR_ERR_INVALID, "null argument");
    cudaSetDevice(ctx->cfg.device);
    FR_CUDA(cudaStreamSynchronize(ctx->stream));
    free_frame(ctx);
    free_scene(ctx);
    const fr_scene_info& I = s->info;
    const int V = (int)I.num_vertices, N = (int)I.num_normals, Nt = (int)I.num_uvs, T = (int)I.num_triangles;
    std::vector<float4> pos(V), tan(V), nrm(N);
    std::vector<float2> uv(Nt);
    for (int i = 0; i < V; ++i)
    {
        pos[i] = make_float4(s->positions[3 * i], s->positions[3 * i + 1], s->positions[3 * i + 2], 0.f);
        tan[i] = make_float4(s->tangents[3 * i], s->tangents[3 * i + 1], s->tangents[3 * i + 2], 0.f);
    }
    for (int i = 0; i < N; ++i)
        nrm[i] = make_float4(s->normals[3 * i], s->normals[3 * i + 1], s->normals[3 * i + 2], 0.f);
    for (int i = 0; i < Nt; ++i) uv[i] = make_float2(s->uvs[2 * i], s->uvs[2 * i + 1]);
    std::vector<int4> triV(T), triT(T), triN(T);
    for (int t = 0; t < T; ++t)
    {
        const fr_mesh_view& me = s->meshes[s->tri_mesh[t]];
        triV[t] = make_int4(s->tri_v[3 * t], s->tri_v[3 * t + 1], s->tri_v[3 * t + 2], s->tri_mesh[t]);
        triT[t] = make_int4(s->tri_vt[3 * t], s->tri_vt[3 * t + 1], s->tri_vt[3 * t + 2], me.material);
        triN[t] = make_int4(s->tri_vn[3 * t], s->tri_vn[3 * t + 1], s->tri_vn[3 * t + 2], me.model);
    }
    std::vector<int> vmodel(V), nmodel(N);
    ctx->hostModels.assign(s->models.size(), frd::DevModel{});
    for (size_t m = 0; m < s->models.size(); ++m)
    {
        const fr_model_view& mv = s->models[m];
        for (int64_t i = 0; i < mv.num_vertices; ++i) vmodel[mv.first_vertex + i] = (int)m;
        for (int64_t i = 0; i < mv.num_normals; ++i) nmodel[mv.first_normal + i] = (int)m;
        frd::DevModel& d = ctx->hostModels[m];
        std::memcpy(d.M, mv.model_matrix, 64);
        fr::M4 M;
        std::memcpy(M.m, mv.model_matrix, 64);
        fr::make_normal_matrix(M, d.N3);
        d.has_tangents = mv.has_tangents;
        d.support_pbr = mv.support_pbr;
    }
    std::vector<frd::DevMaterial> mats(s->materials.size());
    for (size_t i = 0; i < mats.size(); ++i)
    {
        const fr_material_view& a = s->materials[i];
        frd::DevMaterial& b = mats[i];
        std::memcpy(b.ka, a.ka, 12), std::memcpy(b.kd, a.kd, 12), std::memcpy(b.ks, a.ks, 12);
        std::memcpy(b.ke, a.ke, 12), std::memcpy(b.pbr_albedo, a.pbr_albedo, 12);
        b.roughness = a.roughness, b.metalness = a.metalness;
        b.map_kd = a.map_kd, b.map_ks = a.map_ks, b.map_ke = a.map_ke, b.map_bump = a.map_bump;
        b.map_ao = a.map_ao, b.map_pr = a.map_pr, b.map_pm = a.map_pm;
    }
    std::vector<frd::DevTexture> texs(s->textures.size());
    size_t poolBytes = 0;
    for (size_t i = 0; i < texs.size(); ++i)
    {
        const fr_host_texture& t = s->textures[i];
        texs[i].w = t.width, texs[i].h = t.height, texs[i].bpp = t.bpp;
        texs[i].wf = (float)(t.width - 0.001);
        texs[i].hf = (float)(t.height - 0.001);
        texs[i].off = poolBytes;
        size_t b = (size_t)t.width * t.height * (t.bpp == 1 ? 1 : 4);
        poolBytes += (b + 255) & ~(size_t)255;
    }
    std::vector<unsigned char> pool(poolBytes ? poolBytes : 16, 0);
    for (size_t i = 0; i < texs.size(); ++i)
    {
        const fr_host_texture& t = s->textures[i];
        unsigned char* dst = pool.data() + texs[i].off;
        size_t n = (size_t)t.width * t.height;
        if (t.bpp == 1) std::memcpy(dst, t.data.data(), n);
        else
        {
            uint32_t* d32 = reinterpret_cast<uint32_t*>(dst);
            for (size_t k = 0; k < n; ++k)
            {
                const uint8_t* px = t.data.data() + k * t.bpp;  // B, G, R[, A]
                d32[k] = (uint32_t)px[2] | ((uint32_t)px[1] << 8) | ((uint32_t)px[0] << 16);
            }
        }
    }
    frd::DevScene& S = ctx->S;
    S = frd::DevScene{};
    S.numTris = T, S.numVerts = V, S.numNormals = N, S.numModels = (int)s->models.size();
    S.texWrap = ctx->cfg.texture_wrap;
    S.texLinear = ctx->cfg.texture_filter == 1;
    FR_TRY(upload(ctx, S.pos, pos.data(), sizeof(float4) * pos.size()));
    FR_TRY(upload(ctx, S.tan, tan.data(), sizeof(float4) * tan.size()));
    FR_TRY(upload(ctx, S.nrm, nrm.data(), sizeof(float4) * nrm.size()));
    FR_TRY(upload(ctx, S.uv, uv.data(), sizeof(float2) * uv.size()));
    FR_TRY(upload(ctx, S.triV, triV.data(), sizeof(int4) * triV.size()));
    FR_TRY(upload(ctx, S.triT, triT.data(), sizeof(int4) * triT.size()));
    FR_TRY(upload(ctx, S.triN, triN.data(), sizeof(int4) * triN.size()));
    FR_TRY(upload(ctx, S.vmodel, vmodel.data(), sizeof(int) * vmodel.size()));
    FR_TRY(upload(ctx, S.nmodel, nmodel.data(), sizeof(int) * nmodel.size()));
    FR_TRY(upload(ctx, ctx->dModels, ctx->hostModels.data(), sizeof(frd::DevModel) * ctx->hostModels.size()));
    S.models = ctx->dModels;
    FR_TRY(upload(ctx, S.materials, mats.data(), sizeof(frd::DevMaterial) * mats.size()));
    FR_TRY(upload(ctx, S.textures, texs.data(), sizeof(frd::DevTexture) * texs.size()));
    FR_TRY(upload(ctx, S.texels, pool.data(), pool.size()));
    {
        void* g8 = nullptr;
        FR_CUDA(cudaMalloc(&g8, sizeof(float) * 256));
        ctx->sceneBufs.push_back(FrDevBuf{g8, sizeof(float) * 256});
        frk::launch_gamma8_table(static_cast<float*>(g8), ctx->stream);
        FR_CUDA(cudaGetLastError());
        S.gamma8 = static_cast<const float*>(g8);
    }
    FR_CUDA(cudaStreamSynchronize(ctx->stream));  // host staging vectors go out of scope
    // generateTangents (model.cpp:430-476) of the models the loader leaves to the device
    std::vector<unsigned char> pending(s->models.size(), 0);
    bool anyPending = false;
    for (size_t m = 0; m < s->models.size() && m < s->tangent_pending.size(); ++m)
        if (s->tangent_pending[m]) pending[m] = 1, anyPending = true;
    if (anyPending)
    {
        std::vector<int> faces;
        for (int t = 0; t < T; ++t)
            if (pending[s->meshes[s->tri_mesh[t]].model]) faces.push_back(t);
        const int rc = fr_generate_tangents(ctx, faces, pending);
        if (rc != FR_OK) return fail(ctx, rc, "tangent generation on the device failed");
    }
    ctx->info = I;
    fr_scene_frame_matrices(s, ctx->cfg.shadow_size, &ctx->defaultMats);
    ctx->lsValid = false;
    ctx->hasScene = true;
    return FR_OK;
}

int fr_shadow_pass(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    FR_TRY(begin_frame(ctx, p));
    return do_shadow(ctx, stream_of(ctx, p));
}

int fr_forward_pass(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    FR_TRY(begin_frame(ctx, p));
    return do_camera(ctx, stream_of(ctx, p), true);
}

int fr_geometry_pass(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    FR_TRY(begin_frame(ctx, p));
    return do_camera(ctx, stream_of(ctx, p), false);
}

int fr_ssao_pass(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    FR_TRY(begin_frame(ctx, p));
    return do_ssao(ctx, stream_of(ctx, p));
}

int fr_lighting_pass(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    FR_TRY(begin_frame(ctx, p));
    FR_TRY(do_ssao(ctx, stream_of(ctx, p)));
    return do_lighting(ctx, stream_of(ctx, p));
}

int fr_ssaa_pass(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    FR_TRY(begin_frame(ctx, p));
    return do_ssaa(ctx, stream_of(ctx, p));
}

namespace
{

// The launches of one frame on `st` (captured into the frame graph, or run directly).
// Concurrent deferred frames fork the camera chain (geometry, SSAO, blur) onto the
// context's high-priority second stream while the shadow pass runs on `st`: the
// shadow map is read only by lighting, so the two chains join before it. They write
// disjoint buffers (separate visibility keys, bins and counters), so the results
// are those of the sequential order.
int record_frame(fr_ctx* ctx, cudaStream_t st)
{
    ctx->launches = 0;
    ctx->concurrent = ctx->info.deferred && ctx->cfg.concurrent_passes;
    // events: 0 start | shadow | 1 | geometry / forward | 2 | ssao | 3 | blur | 4 | 7 join | lighting | 5 | ssaa | 6
    // (concurrent: shadow runs 0 -> 1 while geometry runs 0 -> 2)
    FR_CUDA(record_event(ctx, ctx->ev[0], st));
    if (ctx->concurrent)
    {
        cudaStream_t cam = ctx->stream2;
        FR_CUDA(cudaEventRecord(ctx->forkEv, st));
        FR_CUDA(cudaStreamWaitEvent(cam, ctx->forkEv, 0));
        FR_TRY(do_camera(ctx, cam, false));
        FR_CUDA(record_event(ctx, ctx->ev[2], cam));
        FR_TRY(do_ssao(ctx, cam, ctx->ev[3]));
        FR_CUDA(record_event(ctx, ctx->ev[4], cam));
        FR_CUDA(cudaEventRecord(ctx->joinEv, cam));
        FR_TRY(do_shadow(ctx, st));
        FR_CUDA(record_event(ctx, ctx->ev[1], st));
        FR_CUDA(cudaStreamWaitEvent(st, ctx->joinEv, 0));
        FR_CUDA(record_event(ctx, ctx->ev[7], st));
        FR_TRY(do_lighting(ctx, st));
        FR_CUDA(record_event(ctx, ctx->ev[5], st));
    }
    else
    {
        FR_TRY(do_shadow(ctx, st));
        FR_CUDA(record_event(ctx, ctx->ev[1], st));
        if (ctx->info.deferred)
        {
            FR_TRY(do_camera(ctx, st, false));
            FR_CUDA(record_event(ctx, ctx->ev[2], st));
            FR_TRY(do_ssao(ctx, st, ctx->ev[3]));
            FR_CUDA(record_event(ctx, ctx->ev[4], st));
            FR_CUDA(record_event(ctx, ctx->ev[7], st));
            FR_TRY(do_lighting(ctx, st));
            FR_CUDA(record_event(ctx, ctx->ev[5], st));
        }
        else
        {
            FR_TRY(do_camera(ctx, st, true));
            for (int i : {2, 3, 4, 7, 5}) FR_CUDA(record_event(ctx, ctx->ev[i], st));
        }
    }
    FR_TRY(do_ssaa(ctx, st));
    FR_CUDA(record_event(ctx, ctx->ev[6], st));
    return FR_OK;
}

}  // namespace

int fr_render_frame(fr_ctx* ctx, const fr_frame_params* p)
{
    if (!ctx) return FR_ERR_INVALID;
    cudaSetDevice(ctx->cfg.device);
    FR_TRY(check_status(ctx));
    FR_TRY(begin_frame(ctx, p));
    cudaStream_t st = stream_of(ctx, p);
    if (ctx->cfg.frame_graph)
    {
        // The key leaves out the camera (view, projection, their product, the eye):
        // a graph captured for another camera is replayed with its kernel nodes'
        // frame constants replaced (cudaGraphExecKernelNodeSetParams).
        fr_ctx::GraphKey key;
        std::memset(&key, 0, sizeof key);
        key.fc = ctx->fc;
        std::memset(key.fc.V, 0, sizeof key.fc.V);
        std::memset(key.fc.P, 0, sizeof key.fc.P);
        std::memset(key.fc.VP, 0, sizeof key.fc.VP);
        std::memset(key.fc.eye, 0, sizeof key.fc.eye);
        key.stream = st;
        key.net = ctx->aonet;
        key.W = ctx->W, key.H = ctx->H, key.SW = ctx->SW, key.SH = ctx->SH;
        if (ctx->graphExec && std::memcmp(&key, &ctx->graphKey, sizeof key) == 0)
        {
            bool ok = true;
            if (std::memcmp(&ctx->fc, &ctx->graphFc, sizeof ctx->fc) != 0)
            {
                for (const fr_ctx::FcNode& n : ctx->fcNodes)
                {
                    void* args[16];
                    for (int a = 0; a < n.nargs; ++a) args[a] = n.params.kernelParams[a];
                    args[n.index] = &ctx->fc;
                    cudaKernelNodeParams p = n.params;
                    p.kernelParams = args;
                    p.extra = nullptr;
                    if (cudaGraphExecKernelNodeSetParams(ctx->graphExec, n.node, &p) != cudaSuccess)
                    {
                        ok = false;
                        break;
                    }
                }
                if (ok) ctx->graphFc = ctx->fc;
            }
            if (ok)
            {
                FR_CUDA(cudaGraphLaunch(ctx->graphExec, st));
                ctx->launches = ctx->graphLaunches;
                ctx->statusPending = true;
                return FR_OK;
            }
            cudaGetLastError();
            drop_graph(ctx);  // the update failed: capture again
        }
        // Capture on the second consecutive frame with the same key: the first
        // runs directly and performs every allocation and one-time setup.
        const bool repeat = ctx->lastKeyValid && std::memcmp(&key, &ctx->lastKey, sizeof key) == 0;
        ctx->lastKey = key;
        ctx->lastKeyValid = true;
        if (repeat)
        {
            drop_graph(ctx);
            cudaGraph_t g = nullptr;
            FR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            ctx->capturing = true;
            const int rc = record_frame(ctx, st);
            ctx->capturing = false;
            const cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (rc == FR_OK && ce == cudaSuccess && g && collect_fc_nodes(ctx, g) &&
                cudaGraphInstantiate(&ctx->graphExec, g, cudaGraphInstantiateFlagUseNodePriority) == cudaSuccess)
            {
                ctx->graph = g;
                ctx->graphFc = ctx->fc;
                ctx->graphKey = key;
                ctx->graphLaunches = ctx->launches;
                FR_CUDA(cudaGraphLaunch(ctx->graphExec, st));
                ctx->statusPending = true;
                return FR_OK;
            }
            if (g) cudaGraphDestroy(g);
            ctx->graphExec = nullptr;
            ctx->fcNodes.clear();
            cudaGetLastError();  // capture failed: run the frame directly
        }
    }
    FR_TRY(record_frame(ctx, st));
    ctx->statusPending = true;
    return FR_OK;
}

int fr_last_timings(fr_ctx* ctx, float* ms, int32_t n)
{
    if (!ctx || !ms) return FR_ERR_INVALID;
    FR_CUDA(cudaEventSynchronize(ctx->ev[6]));
    float t[7] = {0, 0, 0, 0, 0, 0, 0};
    // concurrent frames: geometry starts with the shadow pass, lighting at the join
    const int from[7] = {0, ctx->concurrent ? 0 : 1, 2, 3, 7, 5, 0};
    const int to[7] = {1, 2, 3, 4, 5, 6, 6};
    for (int i = ctx->cfg.pass_timings ? 0 : 6; i < 7; ++i)
        FR_CUDA(cudaEventElapsedTime(&t[i], ctx->ev[from[i]], ctx->ev[to[i]]));
    for (int i = 0; i < n && i < 7; ++i) ms[i] = t[i];
    return check_status(ctx);
}

int32_t fr_last_launch_count(const fr_ctx* ctx) { return ctx ? ctx->launches : 0; }

int64_t fr_scene_tangents(fr_ctx* ctx, float* dst, size_t bytes)
{
    if (!ctx) return FR_ERR_INVALID;
    if (!ctx->hasScene) return fail(ctx, FR_ERR_INVALID, "no scene uploaded");
    const size_t V = (size_t)ctx->S.numVerts, need = 12 * V;
    if (!dst) return (int64_t)need;
    if (bytes < need) return fail(ctx, FR_ERR_INVALID, "destination too small");
    if (V == 0) return FR_OK;
    cudaSetDevice(ctx->cfg.device);
    FR_CUDA(cudaMemcpy2DAsync(dst, 12, ctx->S.tan, sizeof(float4), 12, V, cudaMemcpyDeviceToHost, ctx->stream));
    FR_CUDA(cudaStreamSynchronize(ctx->stream));
    return FR_OK;
}

int64_t fr_download(fr_ctx* ctx, int32_t id, void* dst, size_t bytes)
{
    if (!ctx) return FR_ERR_INVALID;
    if (ctx->W == 0) return fail(ctx, FR_ERR_INVALID, "no frame rendered");
    const size_t P = (size_t)ctx->W * ctx->H;
    const int k = ctx->info.ssaa_on ? ctx->info.ssaa_kernel : 1;
    size_t need = 0;
    switch (id)
    {
        case FR_BUF_DEPTH: case FR_BUF_GB_TYPE: case FR_BUF_AO: case FR_BUF_TRIANGLE_ID: need = 4 * P; break;
        case FR_BUF_SHADOW: need = 4 * (size_t)ctx->SW * ctx->SH; break;
        case FR_BUF_GB_NORMAL: case FR_BUF_GB_POSITION: case FR_BUF_GB_LIGHTNDC: case FR_BUF_GB_ALBEDO:
        case FR_BUF_GB_EMISSIVE: case FR_BUF_GB_PARAM: case FR_BUF_FRAME_F32: need = 12 * P; break;
        case FR_BUF_FRAME_U8: need = 3 * P; break;
        case FR_BUF_SSAA_U8: need = 3 * (size_t)(ctx->W / k) * (ctx->H / k); break;
        default: return fail(ctx, FR_ERR_INVALID, "unknown buffer id");
    }
    if (!dst) return (int64_t)need;
    if (bytes < need) return fail(ctx, FR_ERR_INVALID, "destination too small");
    cudaSetDevice(ctx->cfg.device);
    cudaStream_t st = ctx->stream;
    if (id == FR_BUF_FRAME_U8 || id == FR_BUF_SSAA_U8)
    {
        // pinned host memory the device can address: the packing kernel writes it
        // directly, queued behind the frame's last event, and one wait covers both
        cudaPointerAttributes pa{};
        const cudaError_t ae = cudaPointerGetAttributes(&pa, dst);
        if (ae != cudaSuccess) cudaGetLastError();  // this call's own error: take the copy below
        if (ae == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer && pa.device == ctx->cfg.device)
        {
            const size_t n = id == FR_BUF_FRAME_U8 ? P : (size_t)(ctx->W / k) * (ctx->H / k);
            if (ctx->statusPending) FR_CUDA(cudaStreamWaitEvent(st, ctx->ev[6], 0));
            frk::launch_pack_rgb(id == FR_BUF_FRAME_U8 ? ctx->frame8 : ctx->ssaa,
                                 static_cast<uint8_t*>(pa.devicePointer), (int)n, st);
            FR_CUDA(cudaGetLastError());
            FR_CUDA(cudaStreamSynchronize(st));
            return check_status(ctx);
        }
    }
    FR_CUDA(cudaStreamSynchronize(st));
    {
        int rc = check_status(ctx);
        if (rc != FR_OK) return rc;
    }
    void* tmp = nullptr;
    auto d2h = [&](const void* src, size_t n) -> int {
        FR_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, st));
        FR_CUDA(cudaStreamSynchronize(st));
        return FR_OK;
    };
    int rc = FR_OK;
    switch (id)
    {
        case FR_BUF_DEPTH: rc = d2h(ctx->gb.depth, need); break;
        case FR_BUF_AO: rc = d2h(ctx->gb.ao, need); break;
        case FR_BUF_SHADOW: rc = d2h(ctx->shadow, need); break;
        case FR_BUF_FRAME_F32:
            if (!ctx->frameF) return fail(ctx, FR_ERR_INVALID, "FRAME_F32 needs fr_config.keep_float_frame");
            rc = d2h(ctx->frameF, need);
            break;
        case FR_BUF_TRIANGLE_ID:
            FR_CUDA(cudaMalloc(&tmp, need));
            frk::launch_triangle_ids(ctx->keys, (int)P, (int*)tmp, st);
            rc = d2h(tmp, need);
            break;
        case FR_BUF_FRAME_U8:
        case FR_BUF_SSAA_U8:
        {
            // packed to R, G, B on the device, then one copy into dst (pinned,
            // device-addressable destinations took the direct path above)
            const size_t n = id == FR_BUF_FRAME_U8 ? P : (size_t)(ctx->W / k) * (ctx->H / k);
            if (ctx->rgbCap < 3 * n)
            {
                if (ctx->rgbBuf) cudaFree(ctx->rgbBuf);
                ctx->rgbBuf = nullptr, ctx->rgbCap = 0;
                FR_CUDA(cudaMalloc(&ctx->rgbBuf, 3 * n));
                ctx->rgbCap = 3 * n;
            }
            frk::launch_pack_rgb(id == FR_BUF_FRAME_U8 ? ctx->frame8 : ctx->ssaa, ctx->rgbBuf, (int)n, st);
            rc = d2h(ctx->rgbBuf, need);
            break;
        }
        default:
        {
            int which = id == FR_BUF_GB_NORMAL ? 0 : id == FR_BUF_GB_POSITION ? 1 : id == FR_BUF_GB_LIGHTNDC ? 2
                      : id == FR_BUF_GB_ALBEDO ? 3 : id == FR_BUF_GB_EMISSIVE ? 4 : id == FR_BUF_GB_PARAM ? 5 : 6;
            FR_CUDA(cudaMalloc(&tmp, need));
            frk::launch_unpack_gbuffer(ctx->S, ctx->gb, ctx->W, ctx->H, which, (float*)tmp, st);
            rc = d2h(tmp, need);
        }
    }
    if (tmp) cudaFree(tmp);
    if (rc != FR_OK) return rc;
    return FR_OK;
}

}  // extern "C"

// ---- learned AO (include/fr_aonet.h) ------------------------------------------------

extern "C" {

int fr_set_ao_net(fr_ctx* ctx, fr_aonet* net)
{
    if (!ctx) return FR_ERR_INVALID;
    if (ctx->graphExec) cudaGraphExecDestroy(ctx->graphExec);
    ctx->graphExec = nullptr;
    ctx->lastKeyValid = false;
    if (net && fra_device(net) != ctx->cfg.device)
        return fail(ctx, FR_ERR_INVALID, "network and context are on different devices");
    ctx->aonet = net;
    return FR_OK;
}

int fr_ao_features(fr_ctx* ctx, uint16_t* dst, void* stream)
{
    if (!ctx || !dst) return FR_ERR_INVALID;
    if (ctx->W == 0) return fail(ctx, FR_ERR_INVALID, "no geometry pass yet");
    cudaSetDevice(ctx->cfg.device);
    cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->stream;
    frk::launch_ao_features(ctx->fc, ctx->gb, reinterpret_cast<uint4*>(dst), st, ctx->aoInputTable,
                           ctx->cfg.ao_input_samples);
    FR_CUDA(cudaGetLastError());
    return FR_OK;
}

int fr_ao_probe_result(fr_ctx* ctx, float* mean_sq_diff, int32_t* fell_back)
{
    if (!ctx) return FR_ERR_INVALID;
    if (!ctx->aoGate) return fail(ctx, FR_ERR_INVALID, "no learned-AO frame yet");
    cudaSetDevice(ctx->cfg.device);
    FR_CUDA(cudaStreamSynchronize(ctx->stream));
    float m = 0.f;
    int g = 0;
    FR_CUDA(cudaMemcpy(&m, ctx->probeMean, sizeof(float), cudaMemcpyDeviceToHost));
    FR_CUDA(cudaMemcpy(&g, ctx->aoGate, sizeof(int), cudaMemcpyDeviceToHost));
    if (mean_sq_diff) *mean_sq_diff = m;
    if (fell_back) *fell_back = g;
    return FR_OK;
}

}  // extern "C"

// ---- accessors for the learned-AO trainer (fr_context_internal.h) -------------------

float* frctx_ao(fr_ctx* ctx) { return ctx->gb.ao; }
const float* frctx_depth(fr_ctx* ctx) { return ctx->gb.depth; }
cudaStream_t frctx_stream(fr_ctx* ctx) { return ctx->stream; }
void frctx_size(const fr_ctx* ctx, int* W, int* H)
{
    *W = ctx->W;
    *H = ctx->H;
}
