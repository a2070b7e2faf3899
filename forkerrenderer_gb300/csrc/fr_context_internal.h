// The render context (fr_ctx) and accessors, for library code outside
// fr_context.cu (the learned-AO trainer, batched multi-view rendering).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fr_aonet.h"
#include "fr_kernels.cuh"
#include "forkerrenderer.h"

struct FrDevBuf
{
    void* p = nullptr;
    size_t bytes = 0;
};

struct FrOutputState;  // TGA output buffers (fr_output.cu)

struct fr_ctx
{
    fr_config cfg{};
    cudaStream_t stream = nullptr;
    // deferred frames: the shadow pass runs on stream2, forked from the frame's
    // stream and joined back before lighting (the camera chain runs meanwhile)
    cudaStream_t stream2 = nullptr;
    cudaEvent_t forkEv = nullptr, joinEv = nullptr;
    // learned AO: the probe's plain SSAO runs on stream3 beside the network
    cudaStream_t stream3 = nullptr;
    cudaEvent_t probeForkEv = nullptr, probeJoinEv = nullptr;
    bool concurrent = false;  // the last frame ran the shadow and camera chains side by side
    std::string err;
    std::vector<FrDevBuf> sceneBufs;

    bool hasScene = false;
    fr_scene_info info{};
    fr_frame_matrices defaultMats{};
    std::vector<frd::DevModel> hostModels;
    float lsUsed[16];
    bool lsValid = false;
    frd::DevScene S{};
    frd::DevModel* dModels = nullptr;

    // frame buffers
    int W = 0, H = 0, SW = 0, SH = 0;
    frd::VertexOut vo{};
    int4* scrL = nullptr;
    frk::RasterScratch rsCam{}, rsShadow{};
    unsigned long long* keys = nullptr;       // camera pass visibility keys (W * H)
    unsigned long long* keysShadow = nullptr; // shadow pass visibility keys (SW * SH)
    size_t keysCap = 0;
    frd::GBuffer gb{};
    float* shadow = nullptr;
    unsigned* frame8 = nullptr;
    float* frameF = nullptr;
    unsigned* ssaa = nullptr;
    float* blurTmp = nullptr;
    float* ssaoTable = nullptr;
    float* ssaoBg16 = nullptr;  // AO of background pixels per noise cell
    int ssaoTableN = 0;
    int* counters = nullptr;  // 8 ints: shadow pass [0..3], camera pass [4..7]
    int* hostCounters = nullptr;     // mapped pinned host memory: the last frame's status words
    int* hostCountersDev = nullptr;  // its device address
    std::vector<void*> frameAllocs;

    frd::FrameConst fc{};
    fr_frame_matrices mats{};
    bool shadowDone = false, geometryDone = false, lightingDone = false, ssaaDone = false;

    cudaEvent_t ev[8] = {};
    int launches = 0;
    bool statusPending = false;

    // learned AO
    fr_aonet* aonet = nullptr;
    uint4* aoFeat = nullptr;   // network input, one 8-channel BF16 vector per pixel
    size_t aoFeatCap = 0;
    float* probePart = nullptr;
    float* probePlain = nullptr;  // the probe pixels' plain SSAO, NaN where uncovered
    size_t probePartCap = 0;
    int* aoGate = nullptr;     // 1 = run plain SSAO + blur this frame
    float* probeMean = nullptr;
    unsigned* probeDone = nullptr;  // block counter of the probe's last-block decision
    float4* ssaoTblGlobal = nullptr;
    float* aoInputTable = nullptr;  // K-sample SSAO table of the learned AO's input (cfg.ao_input_samples)

    // frame graph (fr_config.frame_graph): the frame's launches captured once and
    // replayed while the frame constants, stream, network and buffers are unchanged
    struct GraphKey
    {
        frd::FrameConst fc;
        cudaStream_t stream;
        fr_aonet* net;
        int W, H, SW, SH;
    };
    cudaGraphExec_t graphExec = nullptr;
    cudaGraph_t graph = nullptr;  // the captured graph, kept for its nodes' handles
    // kernel nodes that take the frame constants by value: a new camera updates them in place
    struct FcNode
    {
        cudaGraphNode_t node;
        cudaKernelNodeParams params;  // as captured (its argument pointers live in `graph`)
        int index, nargs;
    };
    std::vector<FcNode> fcNodes;
    bool capturing = false;
    GraphKey graphKey{};
    frd::FrameConst graphFc{};  // the frame constants the graph's kernel nodes hold
    GraphKey lastKey{};
    bool lastKeyValid = false;
    int graphLaunches = 0;
    FrOutputState* output = nullptr;
    uint8_t* rgbBuf = nullptr;  // fr_download's packed R, G, B bytes of the 8-bit images
    size_t rgbCap = 0;
};



void frctx_frame_const(fr_ctx* ctx, const fr_frame_matrices& m, frd::FrameConst& F);
void frctx_refresh_background(frd::FrameConst& F);
float* frctx_ao(fr_ctx* ctx);           // AO plane of the last SSAO pass, W * H floats
const float* frctx_depth(fr_ctx* ctx);  // depth buffer, FLT_MAX where no triangle
cudaStream_t frctx_stream(fr_ctx* ctx);
void frout_free(fr_ctx* ctx);  // releases ctx->output
void frctx_size(const fr_ctx* ctx, int* W, int* H);
// Model::generateTangents on the device into ctx->S.tan for the models flagged in
// pendingModels; faces = their triangles in draw order (fr_tangents.cu).
int fr_generate_tangents(fr_ctx* ctx, const std::vector<int>& faces, const std::vector<unsigned char>& pendingModels);
