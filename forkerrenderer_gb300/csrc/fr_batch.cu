// Batched multi-view rendering (include/fr_batch.h): many camera views of
// uneven sizes plus per-light shadow maps in one CUDA graph, with the fine
// raster and the lighting as persistent launches over (view, tile) queues.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fr_aonet.h"
#include "fr_aonet_internal.h"
#include "fr_batch.h"
#include "fr_context_internal.h"
#include "fr_hostmath.h"
#include "fr_kernels.cuh"

namespace
{

constexpr int kBranches = 8;  // parallel graph branches of the per-view stages

struct Alloc
{
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T* get(size_t count)
    {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, sizeof(T) * (count ? count : 1));
        if (e != cudaSuccess)
        {
            err = e;
            return nullptr;
        }
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~Alloc()
    {
        for (void* p : ptrs) cudaFree(p);
    }
};

int tiles_of(int w, int h, int t) { return ((w + t - 1) / t) * ((h + t - 1) / t); }

// Raster scratch of one view or shadow map (as fr_context allocates it per pass).
bool alloc_raster(Alloc& A, frk::RasterScratch& rs, int W, int H, int T, long long binCapCfg)
{
    const int tiles = tiles_of(W, H, frk::kTile);
    rs = {};
    rs.keys = A.get<unsigned long long>((size_t)W * H);
    rs.triCap = T > 0 ? T : 1;
    rs.binCap = binCapCfg > 0 ? binCapCfg : (long long)tiles * 16 + (1 << 22);
    rs.mediumTris = A.get<frx::RTri>(rs.triCap);
    rs.mediumIdx = A.get<int>(rs.triCap);
    rs.largeTris = A.get<frx::RTri>(rs.triCap);
    rs.largeIdx = A.get<int>(rs.triCap);
    rs.largeAux = A.get<float4>(rs.triCap);
    rs.counters = A.get<int>(4);
    rs.tileCount = A.get<int>(tiles);
    rs.tileStart = A.get<int>(tiles + 1);
    rs.tileFill = A.get<int>(tiles);
    rs.binTri = A.get<int>((size_t)rs.binCap);
    return A.err == cudaSuccess;
}

}  // namespace

struct fr_batch
{
    fr_ctx* ctx = nullptr;
    std::string err;
    Alloc mem;
    int nViews = 0, nLights = 0;
    std::vector<fr_view_desc> viewDesc;
    std::vector<fr_light_desc> lightDesc;

    struct View
    {
        frd::FrameConst F;
        frd::VertexOut vo;
        frk::RasterScratch rs;
        frd::GBuffer gb;
        unsigned* frame8;
        float* blurTmp;
        float* bg16;
        uint4* aoFeat;  // learned AO: network input (2x2-block layout)
        float* probePart;
        float* probePlain;
        unsigned* probeDone;
        int* gate;
        float* probeMean;
        int aoMode;
    };
    struct Light
    {
        frd::FrameConst F;  // shadow pass (L, SVPort, SW, SH) and shadow lookups
        frd::DevScene S;    // the scene with this light's per-model light matrices
        int4* scrL;
        frk::RasterScratch rs;
        float* shadow;
    };
    std::vector<View> views;
    std::vector<Light> lights;
    frd::DevScene viewScene{};  // models' light matrices from light 0 (the G-buffer's light NDC)

    frk::ViewRaster* dRaster = nullptr;
    int* dRasterStart = nullptr;
    int rasterItems = 0;
    frk::ViewShade* dShade = nullptr;
    int* dShadeStart = nullptr;
    int shadeItems = 0;
    frk::BatchLight* dLights = nullptr;
    int* dQueues = nullptr;
    float4* ssaoTblGlobal = nullptr;

    fr_batch_tuning tuning{16, 64, 2};
    cudaStream_t br[kBranches] = {};
    cudaEvent_t forkEv = nullptr, joinEv[kBranches] = {};
    cudaEvent_t tev[5] = {};
    cudaGraphExec_t exec = nullptr;
    int numSMs = 152;
};

namespace
{

int bfail(fr_batch* b, int code, const std::string& m)
{
    if (b) b->err = m;
    return code;
}

#define B_CUDA(b, x)                                                                                           \
    do                                                                                                         \
    {                                                                                                          \
        cudaError_t e_ = (x);                                                                                  \
        if (e_ != cudaSuccess) return bfail((b), FR_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

fr::M4 light_space(const fr_batch* b, const fr_light_desc& L)
{
    const fr_scene_info& I = b->ctx->info;
    if (L.type == FR_LIGHT_POINT)
    {
        // the reference's shadow frustum (render.cpp:73-78)
        const float ratio = (float)I.width / I.height;
        fr::M4 lview = fr::make_look_at(fr::V3{L.position[0], L.position[1], L.position[2]}, fr::V3{0.f, 0.f, 0.f});
        fr::M4 lproj = fr::make_ortho(-3.f * ratio, 3.f * ratio, -3.f, 3.f, 0.1f, 20.f);
        return fr::mul(lproj, lview);
    }
    const float e = L.extent > 0.f ? L.extent : 6.f;
    const float d = 2.f * e + 10.f;
    const fr::V3 eye{-L.direction[0] * d, -L.direction[1] * d, -L.direction[2] * d};
    fr::M4 lview = fr::make_look_at(eye, fr::V3{0.f, 0.f, 0.f});
    fr::M4 lproj = fr::make_ortho(-e, e, -e, e, 0.1f, 2.f * d);
    return fr::mul(lproj, lview);
}

void models_for(fr_batch* b, const fr::M4& L, std::vector<frd::DevModel>& out)
{
    out = b->ctx->hostModels;
    for (auto& md : out)
    {
        fr::M4 M;
        std::memcpy(M.m, md.M, 64);
        fr::M4 LM = fr::mul(L, M);
        std::memcpy(md.LM, LM.m, 64);
    }
}

// The work of one render, recorded on ctx->stream (captured into the graph).
int record(fr_batch* b)
{
    fr_ctx* ctx = b->ctx;
    cudaStream_t st = ctx->stream;
    const frk::RasterParams base{0, 0, ctx->cfg.small_tri_area, ctx->cfg.medium_tri_area};
    int launches = 0;
    auto rec = [&](cudaEvent_t e, cudaStream_t s) { return cudaEventRecordWithFlags(e, s, cudaEventRecordExternal); };
    B_CUDA(b, rec(b->tev[0], st));
    // 1. transforms, setup and binning of every shadow map and view (parallel branches)
    B_CUDA(b, cudaEventRecord(b->forkEv, st));
    for (int i = 0; i < kBranches; ++i) B_CUDA(b, cudaStreamWaitEvent(b->br[i], b->forkEv, 0));
    int next = 0;
    for (auto& L : b->lights)
    {
        cudaStream_t s = b->br[next++ % kBranches];
        frk::launch_transform_light(L.S, L.F, L.scrL, s);
        frk::RasterParams rp = base;
        rp.W = L.F.SW, rp.H = L.F.SH;
        frk::launch_raster(L.S, L.scrL, rp, L.rs, s, launches, false);
    }
    for (auto& V : b->views)
    {
        cudaStream_t s = b->br[next++ % kBranches];
        frk::launch_transform_camera(b->viewScene, V.F, V.vo, s);
        frk::RasterParams rp = base;
        rp.W = V.F.W, rp.H = V.F.H;
        frk::launch_raster(b->viewScene, V.vo.scr, rp, V.rs, s, launches, false);
    }
    for (int i = 0; i < kBranches; ++i)
    {
        B_CUDA(b, cudaEventRecord(b->joinEv[i], b->br[i]));
        B_CUDA(b, cudaStreamWaitEvent(st, b->joinEv[i], 0));
    }
    B_CUDA(b, rec(b->tev[1], st));
    // 2. the fine raster of every shadow map and view: one persistent launch
    frk::launch_tile_raster_views(b->dRaster, b->dRasterStart, b->nLights + b->nViews, b->rasterItems, b->dQueues,
                                  b->tuning.bin_batch, b->numSMs * b->tuning.ctas_per_sm, st);
    B_CUDA(b, rec(b->tev[2], st));
    // 3. resolves and ambient occlusion (learned views share the network: one branch)
    B_CUDA(b, cudaEventRecord(b->forkEv, st));
    for (int i = 0; i < kBranches; ++i) B_CUDA(b, cudaStreamWaitEvent(b->br[i], b->forkEv, 0));
    next = 0;
    for (auto& L : b->lights)
        frk::launch_resolve_shadow(L.S, L.scrL, L.rs.keys, L.F.SW, L.F.SH, L.shadow, b->br[next++ % kBranches]);
    for (auto& V : b->views)
    {
        const bool learned = V.aoMode == FR_AO_LEARNED;
        cudaStream_t s = learned ? b->br[0] : b->br[1 + (next++ % (kBranches - 1))];
        frk::launch_resolve_gbuffer(b->viewScene, V.F, V.vo, V.rs.keys, V.gb, s);
        if (!V.F.ssaoOn) continue;
        if (learned)
        {
            frk::launch_ao_features_blocks(V.F, V.gb, V.aoFeat, s, ctx->aoInputTable, ctx->cfg.ao_input_samples,
                                           ctx->ssaoTable, V.bg16);
            int rc = fra_forward_blocks(ctx->aonet, reinterpret_cast<const uint16_t*>(V.aoFeat), 1, V.F.H, V.F.W,
                                        V.gb.ao, s, &launches, V.gb.depth, V.bg16, false);
            ++launches;
            if (rc != FR_OK) return bfail(b, rc, std::string("network forward: ") + fr_aonet_last_error(ctx->aonet));
            frk::launch_ao_probe_plain(V.F, V.gb, b->ssaoTblGlobal, V.probePlain, s);
            frk::launch_ao_probe_compare(V.F, V.gb.ao, V.probePlain, ctx->cfg.ao_probe_threshold, V.probePart,
                                         V.probeDone, V.gate, V.probeMean, s);
            frk::launch_ssao(V.F, V.gb, ctx->ssaoTable, V.bg16, s, V.gate, false);
            if (frk::launch_blur(ctx->cfg.blur_mode, V.F.W, V.F.H, V.gb.ao, V.blurTmp, s, launches, V.gate,
                                 ctx->cfg.blur_warmup) != FR_OK)
                return bfail(b, FR_ERR_UNSUPPORTED, "view lines too long for the in-place blur");
        }
        else
        {
            frk::launch_ssao(V.F, V.gb, ctx->ssaoTable, V.bg16, s);
            if (frk::launch_blur(ctx->cfg.blur_mode, V.F.W, V.F.H, V.gb.ao, V.blurTmp, s, launches, nullptr,
                                 ctx->cfg.blur_warmup) != FR_OK)
                return bfail(b, FR_ERR_UNSUPPORTED, "view lines too long for the in-place blur");
        }
    }
    for (int i = 0; i < kBranches; ++i)
    {
        B_CUDA(b, cudaEventRecord(b->joinEv[i], b->br[i]));
        B_CUDA(b, cudaStreamWaitEvent(st, b->joinEv[i], 0));
    }
    B_CUDA(b, rec(b->tev[3], st));
    // 4. deferred lighting of every view with every light: one persistent launch
    frk::launch_lighting_views(b->viewScene, b->dShade, b->dShadeStart, b->nViews, b->shadeItems, b->dLights,
                               b->nLights, b->dQueues + 1, b->tuning.light_tile, b->numSMs * b->tuning.ctas_per_sm, st);
    B_CUDA(b, rec(b->tev[4], st));
    B_CUDA(b, cudaGetLastError());
    return FR_OK;
}

// Item tables of the lighting queue for tile edge T.
int build_shade_queue(fr_batch* b)
{
    std::vector<int> start(b->nViews + 1, 0);
    for (int v = 0; v < b->nViews; ++v)
        start[v + 1] = start[v] + tiles_of(b->views[v].F.W, b->views[v].F.H, b->tuning.light_tile);
    b->shadeItems = start[b->nViews];
    B_CUDA(b, cudaMemcpy(b->dShadeStart, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    return FR_OK;
}

int capture(fr_batch* b)
{
    fr_ctx* ctx = b->ctx;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    int rc = build_shade_queue(b);
    if (rc != FR_OK) return rc;
    cudaStream_t st = ctx->stream;
    cudaGraph_t g = nullptr;
    B_CUDA(b, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = record(b);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (rc != FR_OK || ce != cudaSuccess || !g)
    {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc != FR_OK ? rc : bfail(b, FR_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    }
    cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return bfail(b, FR_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    return FR_OK;
}

bool valid_tuning(const fr_batch_tuning& t)
{
    return (t.light_tile == 8 || t.light_tile == 16 || t.light_tile == 32) &&
           (t.bin_batch == 64 || t.bin_batch == 256 || t.bin_batch == 1024) &&
           (t.ctas_per_sm == 1 || t.ctas_per_sm == 2 || t.ctas_per_sm == 4);
}

}  // namespace

extern "C" {

fr_batch* fr_batch_create(fr_ctx* ctx, const fr_view_desc* views, int32_t n_views, const fr_light_desc* lights,
                          int32_t n_lights, char* err, size_t errlen)
{
    auto bail = [&](const std::string& m) -> fr_batch* {
        if (err && errlen) std::snprintf(err, errlen, "%s", m.c_str());
        return nullptr;
    };
    if (!ctx || !views || n_views < 1 || !lights || n_lights < 1 || n_lights > frk::kMaxBatchLights)
        return bail("need a context, 1+ views and 1..4 lights");
    if (!ctx->hasScene) return bail("no scene uploaded");
    if (!ctx->info.deferred) return bail("batched views render the deferred path");
    cudaSetDevice(ctx->cfg.device);
    fr_batch* b = new fr_batch();
    b->ctx = ctx;
    b->nViews = n_views, b->nLights = n_lights;
    b->viewDesc.assign(views, views + n_views);
    b->lightDesc.assign(lights, lights + n_lights);
    int dev = ctx->cfg.device;
    cudaDeviceGetAttribute(&b->numSMs, cudaDevAttrMultiProcessorCount, dev);
    Alloc& A = b->mem;
    const int T = ctx->S.numTris, V = ctx->S.numVerts, N = ctx->S.numNormals;
    bool anyLearned = false;

    // lights: per-light scene copy (its per-model light matrices), raster scratch, shadow map
    std::vector<frd::DevModel> hm;
    for (int k = 0; k < n_lights; ++k)
    {
        const fr_light_desc& LD = lights[k];
        if (LD.shadow_size < 16 || LD.shadow_size > 16384) return fr_batch_destroy(b), bail("bad shadow_size");
        fr_batch::Light L{};
        const fr::M4 LS = light_space(b, LD);
        models_for(b, LS, hm);
        frd::DevModel* dm = A.get<frd::DevModel>(hm.size());
        if (!dm) return fr_batch_destroy(b), bail("out of device memory");
        cudaMemcpy(dm, hm.data(), sizeof(frd::DevModel) * hm.size(), cudaMemcpyHostToDevice);
        L.S = ctx->S;
        L.S.models = dm;
        if (k == 0)
        {
            b->viewScene = ctx->S;
            b->viewScene.models = dm;
        }
        fr_frame_matrices m = ctx->defaultMats;
        std::memcpy(m.light_space, LS.m, 64);
        fr::M4 svp = fr::make_viewport(LD.shadow_size, LD.shadow_size);
        std::memcpy(m.shadow_viewport, svp.m, 64);
        m.shadow_width = m.shadow_height = LD.shadow_size;
        frctx_frame_const(ctx, m, L.F);
        std::memcpy(L.F.lightPos, LD.position, 12);
        std::memcpy(L.F.lightColor, LD.color, 12);
        L.scrL = A.get<int4>(V);
        L.shadow = A.get<float>((size_t)LD.shadow_size * LD.shadow_size);
        if (!alloc_raster(A, L.rs, LD.shadow_size, LD.shadow_size, T, ctx->cfg.bin_capacity))
            return fr_batch_destroy(b), bail("out of device memory");
        b->lights.push_back(L);
    }
    // views
    for (int v = 0; v < n_views; ++v)
    {
        const fr_view_desc& VD = views[v];
        const int W = VD.matrices.width, H = VD.matrices.height;
        if (W < 1 || H < 1 || W > 8192 || H > 8192) return fr_batch_destroy(b), bail("bad view size");
        fr_batch::View X{};
        fr_frame_matrices m = VD.matrices;
        std::memcpy(m.light_space, b->lights[0].F.L, 64);  // light 0's NDC in the G-buffer
        m.shadow_width = b->lights[0].F.SW, m.shadow_height = b->lights[0].F.SH;
        std::memcpy(m.shadow_viewport, b->lights[0].F.SVPort, 64);
        frctx_frame_const(ctx, m, X.F);
        std::memcpy(X.F.eye, VD.eye, 12);
        std::memcpy(X.F.lightPos, lights[0].position, 12);
        std::memcpy(X.F.lightColor, lights[0].color, 12);
        X.aoMode = VD.ao_mode;
        if (X.aoMode == FR_AO_LEARNED)
        {
            anyLearned = true;
            if (W % fra::kLevelAlign || H % fra::kLevelAlign)
                return fr_batch_destroy(b), bail("learned-AO views need W, H multiples of 32");
        }
        const size_t P = (size_t)W * H;
        X.vo.scr = A.get<int4>(V);
        X.vo.pw = A.get<float4>(V);
        X.vo.lw = A.get<float4>(V);
        X.vo.tw = A.get<float4>(V);
        X.vo.npre = A.get<float4>(N);
        X.gb.a = A.get<float4>(P);
        X.gb.b = A.get<float4>(P);
        X.gb.c = A.get<uint4>(P);
        X.gb.depth = A.get<float>(P);
        X.gb.ao = A.get<float>(P);
        X.frame8 = A.get<unsigned>(P);
        X.blurTmp = A.get<float>(P);
        X.bg16 = A.get<float>(16);
        if (X.aoMode == FR_AO_LEARNED)
        {
            X.aoFeat = A.get<uint4>(P / 2 + 1);
            X.probePart = A.get<float>(2 * (size_t)frk::ao_probe_blocks(W, H) + 2);
            X.probePlain = A.get<float>((size_t)(W / 8) * (H / 8) + 1);
            X.probeDone = A.get<unsigned>(1);
            X.gate = A.get<int>(1);
            X.probeMean = A.get<float>(1);
        }
        if (!alloc_raster(A, X.rs, W, H, T, ctx->cfg.bin_capacity) || A.err != cudaSuccess)
            return fr_batch_destroy(b), bail("out of device memory");
        if (X.aoMode == FR_AO_LEARNED)
        {
            cudaMemset(X.probeDone, 0, sizeof(unsigned));
            cudaMemset(X.gate, 0, sizeof(int));
        }
        b->views.push_back(X);
    }
    if (anyLearned && !ctx->aonet) return fr_batch_destroy(b), bail("learned-AO views need fr_set_ao_net");
    if (anyLearned)
    {
        long long maxPix = 0;
        int mW = 0, mH = 0;
        for (auto& X : b->views)
            if (X.aoMode == FR_AO_LEARNED && (long long)X.F.W * X.F.H > maxPix)
                maxPix = (long long)X.F.W * X.F.H, mW = X.F.W, mH = X.F.H;
        if (fra_reserve(ctx->aonet, 1, mH, mW) != FR_OK)
            return fr_batch_destroy(b), bail(std::string("network buffers: ") + fr_aonet_last_error(ctx->aonet));
        b->ssaoTblGlobal = A.get<float4>(16 * (size_t)(2 * ctx->cfg.ssao_samples + 2));
        frk::launch_ssao_table_global(b->views[0].F, ctx->ssaoTable, b->ssaoTblGlobal, ctx->stream);
    }
    // queue tables: shadow maps first, then views
    std::vector<frk::ViewRaster> vr;
    std::vector<int> rstart(1, 0);
    for (auto& L : b->lights)
    {
        vr.push_back(frk::ViewRaster{{L.F.SW, L.F.SH, ctx->cfg.small_tri_area, ctx->cfg.medium_tri_area}, L.rs});
        rstart.push_back(rstart.back() + tiles_of(L.F.SW, L.F.SH, frk::kTile));
    }
    for (auto& X : b->views)
    {
        vr.push_back(frk::ViewRaster{{X.F.W, X.F.H, ctx->cfg.small_tri_area, ctx->cfg.medium_tri_area}, X.rs});
        rstart.push_back(rstart.back() + tiles_of(X.F.W, X.F.H, frk::kTile));
    }
    b->rasterItems = rstart.back();
    rstart.pop_back();
    std::vector<frk::ViewShade> vs;
    for (auto& X : b->views) vs.push_back(frk::ViewShade{X.F, X.gb, X.frame8, lights[0].type == FR_LIGHT_POINT ? 0 : -1});
    std::vector<frk::BatchLight> bl;
    for (int k = 0; k < n_lights; ++k)
    {
        frk::BatchLight x{};
        x.S = b->lights[k].F;
        x.shadow = b->lights[k].shadow;
        std::memcpy(x.pos, lights[k].position, 12);
        float d[3] = {lights[k].direction[0], lights[k].direction[1], lights[k].direction[2]};
        float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int i = 0; i < 3; ++i) x.dir[i] = len > 0.f ? d[i] / len : 0.f;
        std::memcpy(x.color, lights[k].color, 12);
        x.type = lights[k].type;
        bl.push_back(x);
    }
    b->dRaster = A.get<frk::ViewRaster>(vr.size());
    b->dRasterStart = A.get<int>(rstart.size());
    b->dShade = A.get<frk::ViewShade>(vs.size());
    b->dShadeStart = A.get<int>(n_views + 1);
    b->dLights = A.get<frk::BatchLight>(bl.size());
    b->dQueues = A.get<int>(2);
    if (A.err != cudaSuccess) return fr_batch_destroy(b), bail("out of device memory");
    cudaMemcpy(b->dRaster, vr.data(), sizeof(frk::ViewRaster) * vr.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(b->dRasterStart, rstart.data(), sizeof(int) * rstart.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(b->dShade, vs.data(), sizeof(frk::ViewShade) * vs.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(b->dLights, bl.data(), sizeof(frk::BatchLight) * bl.size(), cudaMemcpyHostToDevice);
    for (int i = 0; i < kBranches; ++i)
    {
        cudaStreamCreateWithFlags(&b->br[i], cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&b->joinEv[i], cudaEventDisableTiming);
    }
    cudaEventCreateWithFlags(&b->forkEv, cudaEventDisableTiming);
    for (auto& e : b->tev) cudaEventCreate(&e);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return fr_batch_destroy(b), bail("batch setup failed");
    return b;
}

void fr_batch_destroy(fr_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->ctx->cfg.device);
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (int i = 0; i < kBranches; ++i)
    {
        if (b->br[i]) cudaStreamDestroy(b->br[i]);
        if (b->joinEv[i]) cudaEventDestroy(b->joinEv[i]);
    }
    if (b->forkEv) cudaEventDestroy(b->forkEv);
    for (auto& e : b->tev)
        if (e) cudaEventDestroy(e);
    delete b;
}

const char* fr_batch_last_error(const fr_batch* b) { return b ? b->err.c_str() : "null batch"; }

int fr_batch_set_tuning(fr_batch* b, const fr_batch_tuning* t)
{
    if (!b || !t || !valid_tuning(*t)) return bfail(b, FR_ERR_INVALID, "tuning: light_tile {8,16,32}, bin_batch "
                                                                       "{64,256,1024}, ctas_per_sm {1,2,4}");
    if (std::memcmp(t, &b->tuning, sizeof *t) != 0)
    {
        b->tuning = *t;
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    return FR_OK;
}

int fr_batch_get_tuning(const fr_batch* b, fr_batch_tuning* t)
{
    if (!b || !t) return FR_ERR_INVALID;
    *t = b->tuning;
    return FR_OK;
}

int fr_batch_render(fr_batch* b)
{
    if (!b) return FR_ERR_INVALID;
    cudaSetDevice(b->ctx->cfg.device);
    if (!b->exec)
    {
        int rc = capture(b);
        if (rc != FR_OK) return rc;
    }
    B_CUDA(b, cudaGraphLaunch(b->exec, b->ctx->stream));
    return FR_OK;
}

int fr_batch_timings(fr_batch* b, float* ms, int32_t n)
{
    if (!b || !ms) return FR_ERR_INVALID;
    B_CUDA(b, cudaEventSynchronize(b->tev[4]));
    float t[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&t[i], b->tev[i], b->tev[i + 1]);
    cudaEventElapsedTime(&t[4], b->tev[0], b->tev[4]);
    for (int i = 0; i < n && i < 5; ++i) ms[i] = t[i];
    // raster status (bin / list overflow) of every shadow map and view
    for (auto& L : b->lights)
    {
        int c[4];
        B_CUDA(b, cudaMemcpy(c, L.rs.counters, sizeof c, cudaMemcpyDeviceToHost));
        if (c[3]) return bfail(b, FR_ERR_BIN_OVERFLOW, "shadow map tile-bin capacity exceeded");
    }
    for (auto& X : b->views)
    {
        int c[4];
        B_CUDA(b, cudaMemcpy(c, X.rs.counters, sizeof c, cudaMemcpyDeviceToHost));
        if (c[3]) return bfail(b, FR_ERR_BIN_OVERFLOW, "view tile-bin capacity exceeded");
    }
    return FR_OK;
}

int fr_batch_autotune(fr_batch* b, int32_t reps, fr_batch_tuning* best, float* best_ms)
{
    if (!b || reps < 1) return FR_ERR_INVALID;
    const int tiles[3] = {8, 16, 32}, caps[3] = {64, 256, 1024}, ctas[3] = {1, 2, 4};
    fr_batch_tuning bt = b->tuning;
    float bms = FLT_MAX;
    for (int a : tiles)
        for (int c : caps)
            for (int k : ctas)
            {
                fr_batch_tuning t{a, c, k};
                int rc = fr_batch_set_tuning(b, &t);
                if (rc != FR_OK) return rc;
                std::vector<float> v;
                for (int r = 0; r < reps + 1; ++r)
                {
                    rc = fr_batch_render(b);
                    if (rc != FR_OK) return rc;
                    float ms[5];
                    rc = fr_batch_timings(b, ms, 5);
                    if (rc != FR_OK) return rc;
                    if (r > 0) v.push_back(ms[4]);
                }
                std::sort(v.begin(), v.end());
                const float med = v[v.size() / 2];
                if (med < bms) bms = med, bt = t;
            }
    int rc = fr_batch_set_tuning(b, &bt);
    if (best) *best = bt;
    if (best_ms) *best_ms = bms;
    return rc;
}

int fr_batch_work(const fr_batch* b, int64_t* triangles, int64_t* pixels, int64_t* shadow_texels)
{
    if (!b) return FR_ERR_INVALID;
    int64_t px = 0, sx = 0;
    for (auto& X : b->views) px += (int64_t)X.F.W * X.F.H;
    for (auto& L : b->lights) sx += (int64_t)L.F.SW * L.F.SH;
    if (triangles) *triangles = (int64_t)b->ctx->S.numTris * (b->nViews + b->nLights);
    if (pixels) *pixels = px;
    if (shadow_texels) *shadow_texels = sx;
    return FR_OK;
}

int64_t fr_batch_download(fr_batch* b, int32_t view, int32_t id, void* dst, size_t bytes)
{
    if (!b) return FR_ERR_INVALID;
    cudaSetDevice(b->ctx->cfg.device);
    const void* src = nullptr;
    size_t need = 0;
    unsigned* rgba = nullptr;
    if (view < 0)
    {
        const int k = -1 - view;
        if (k >= b->nLights || id != FR_BUF_SHADOW) return bfail(b, FR_ERR_INVALID, "bad light buffer");
        src = b->lights[k].shadow;
        need = sizeof(float) * b->lights[k].F.SW * b->lights[k].F.SH;
    }
    else
    {
        if (view >= b->nViews) return bfail(b, FR_ERR_INVALID, "bad view");
        const auto& X = b->views[view];
        const size_t P = (size_t)X.F.W * X.F.H;
        if (id == FR_BUF_DEPTH) src = X.gb.depth, need = 4 * P;
        else if (id == FR_BUF_AO) src = X.gb.ao, need = 4 * P;
        else if (id == FR_BUF_FRAME_U8) rgba = X.frame8, need = 3 * P;
        else return bfail(b, FR_ERR_INVALID, "batch views hold FR_BUF_FRAME_U8, FR_BUF_DEPTH and FR_BUF_AO");
    }
    if (!dst) return (int64_t)need;
    if (bytes < need) return bfail(b, FR_ERR_INVALID, "destination too small");
    B_CUDA(b, cudaStreamSynchronize(b->ctx->stream));
    if (src)
    {
        B_CUDA(b, cudaMemcpy(dst, src, need, cudaMemcpyDeviceToHost));
        return FR_OK;
    }
    // packed r | g << 8 | b << 16 -> RGB8
    std::vector<unsigned> tmp(need / 3);
    B_CUDA(b, cudaMemcpy(tmp.data(), rgba, sizeof(unsigned) * tmp.size(), cudaMemcpyDeviceToHost));
    unsigned char* o = static_cast<unsigned char*>(dst);
    for (size_t i = 0; i < tmp.size(); ++i)
    {
        o[3 * i] = tmp[i] & 0xff;
        o[3 * i + 1] = (tmp[i] >> 8) & 0xff;
        o[3 * i + 2] = (tmp[i] >> 16) & 0xff;
    }
    return FR_OK;
}

}  // extern "C"
