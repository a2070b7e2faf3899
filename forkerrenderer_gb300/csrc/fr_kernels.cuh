// Launch interface of the frame kernels (fr_kernels.cu), used by fr_context.cu.
#pragma once

#include <cuda_runtime.h>

#include "fr_device.cuh"

namespace frk
{

constexpr int kTile = 16;  // screen tile edge for the binned raster path

// Scratch of one rasterisation (camera or shadow) pass.
struct RasterScratch
{
    unsigned long long* keys;  // [W*H] visibility keys
    frx::RTri* mediumTris;     // [cap] triangles drawn one warp each
    int* mediumIdx;
    frx::RTri* largeTris;      // [cap] triangles drawn through tile bins
    int* largeIdx;
    float4* largeAux;          // [cap] the large triangles' per-vertex .w screen data
    int4* triRec;              // [2 * triangles] resolve records (tri_record), or null
    int* counters;             // [0] medium count, [1] large count, [2] bin pairs, [3] status bits
    int* tileCount;            // [tiles]
    int* tileStart;            // [tiles + 1]
    int* tileFill;             // [tiles]
    int* binTri;               // [binCap]
    int triCap;                // capacity of the medium / large lists
    long long binCap;          // capacity of binTri
};

enum StatusBits : int
{
    kStatusListOverflow = 1,
    kStatusBinOverflow = 2
};

struct RasterParams
{
    int W, H;              // raster target size
    int smallArea;         // bbox area drawn by one thread
    int mediumArea;        // bbox area drawn by one warp (larger: tile bins)
};

// ---- batched multi-view rendering (fr_batch.h) -------------------------------------------

// One entry of the persistent fine-raster queue: a camera view or a shadow map.
struct ViewRaster
{
    RasterParams rp;
    RasterScratch rs;
};

// A light of a batch. Its shadow lookups use S's matrices and parameters
// (L = light space, SW / SH, shadowMode, pcfN, blockerN).
struct BatchLight
{
    frd::FrameConst S;
    const float* shadow;
    float pos[3];     // point light position
    float dir[3];     // directional light: direction the light travels (unit)
    float color[3];
    int type;         // 0 point, 1 directional
};

// A camera view of a batch in the persistent lighting queue.
struct ViewShade
{
    frd::FrameConst F;    // the view's matrices, size, eye, shadowOn
    frd::GBuffer gb;
    unsigned* frame8;
    int ndcLight;         // light whose light-space NDC the G-buffer holds (interpolated per
                          // vertex as the reference does), or -1: projected per pixel
};

// Vertex stages.
void launch_transform_camera(const frd::DevScene& S, const frd::FrameConst& F, frd::VertexOut vo,
                             cudaStream_t st);
void launch_transform_light(const frd::DevScene& S, const frd::FrameConst& F, int4* scrL, cudaStream_t st);

// Visibility raster: clears keys, classifies and draws every triangle.
// scr: per-vertex (sx, sy, depth bits, *) screen data of this pass.
// shadowOut (a shadow pass): the fine raster also writes the shadow map (the
// resolve of launch_resolve_shadow fused in).
void launch_raster(const frd::DevScene& S, const int4* scr, const RasterParams& rp, RasterScratch& rs,
                   cudaStream_t st, int& launches, bool tileRaster = true, float* shadowOut = nullptr);

// Persistent fine raster over the (entry, tile) items of many views: entry e owns
// items itemStart[e] .. itemStart[e+1]-1; queue: a zeroed counter. cap: triangles
// staged in shared memory per batch (64, 256 or 1024).
void launch_tile_raster_views(const ViewRaster* vr, const int* itemStart, int nEntries, int total, int* queue,
                              int cap, int grid, cudaStream_t st);

// Persistent deferred lighting over the (view, T x T tile) items of many views
// with up to kMaxBatchLights lights (PBR sums the lights' direct terms; Blinn-Phong
// materials use light 0). T: 8, 16 or 32.
constexpr int kMaxBatchLights = 4;
void launch_lighting_views(const frd::DevScene& S, const ViewShade* views, const int* itemStart, int nViews, int total,
                           const BatchLight* lights, int nLights, int* queue, int T, int grid, cudaStream_t st);

// Resolves.
void launch_resolve_shadow(const frd::DevScene& S, const int4* scrL, const unsigned long long* keys, int SW,
                           int SH, float* shadow, cudaStream_t st);
void launch_resolve_gbuffer(const frd::DevScene& S, const frd::FrameConst& F, frd::VertexOut vo,
                            const unsigned long long* keys, frd::GBuffer gb, cudaStream_t st);
// counters / statusOut (optional): block 0 copies the 8 raster counters to statusOut
// (host memory the device can address) as the frame's status.
void launch_forward_shade(const frd::DevScene& S, const frd::FrameConst& F, frd::VertexOut vo,
                          const unsigned long long* keys, const float* shadow, float* depth,
                          unsigned* frame8, float* frameF, cudaStream_t st, const int* counters = nullptr,
                          int* statusOut = nullptr);

// SSAO + blur. table: 16 * N * 3 floats (fr_make_ssao_table). withBackground:
// false when bg16 already holds this frame's background values.
void launch_ssao(const frd::FrameConst& F, frd::GBuffer gb, const float* table, float* bg16, cudaStream_t st,
                 const int* gate = nullptr, bool withBackground = true);
// For a kernel node of a captured frame: whether `func` takes the frame constants
// by value, at which argument position, and how many arguments it has.
bool frame_const_param(const void* func, int& index, int& nargs);
// DevScene::gamma8: 256 floats pow(b / 255, 2.2) computed with the device's powf.
void launch_gamma8_table(float* out, cudaStream_t st);
// gate (device int, optional): the kernels do nothing when *gate == 0. warm: warm-up
// steps of the parallel in-place blur (0 = its default; every value gives the same bits).
// Returns FR_OK, or FR_ERR_UNSUPPORTED when a line of the in-place blur is too long
// for one CTA's shared memory (rows beyond 56,319 or columns beyond 28,159 pixels).
int launch_blur(int mode, int W, int H, float* ao, float* tmp, cudaStream_t st, int& launches,
                const int* gate = nullptr, int warm = 0);

// Learned AO: network input from the G-buffer (fr_aonet.h layout, or already in
// the network's 2x2-block layout), the SSAO sample table in global memory, and
// the 1-in-64 plain-SSAO probe: one warp per probe pixel; the last block sets
// *gate = 1 when the network's AO differs by more than `threshold` (mean squared).
// part: 2 * ao_probe_blocks floats; done: a zeroed counter (left zeroed).
// The 16 per-noise-cell SSAO values of background pixels (k_ssao_background), ungated.
void launch_ssao_background(const frd::FrameConst& F, const float* depth, const float* table, float* bg16,
                            cudaStream_t st);
// inputTable / K: K-sample SSAO table for channel 3 (K = 0: the normal's z instead).
void launch_ao_features(const frd::FrameConst& F, frd::GBuffer gb, uint4* out, cudaStream_t st,
                        const float* inputTable, int K);
// With bg16 the same launch also writes the 16 background values of the frame's
// SSAO (launch_ssao_background's, from frameTable).
void launch_ao_features_blocks(const frd::FrameConst& F, frd::GBuffer gb, uint4* out, cudaStream_t st,
                               const float* inputTable, int K, const float* frameTable = nullptr,
                               float* bg16 = nullptr);
void launch_ssao_table_global(const frd::FrameConst& F, const float* table, float4* out, cudaStream_t st);
int ao_probe_blocks(int W, int H);
// The probe in two launches: the plain values of the probe pixels (they read the
// G-buffer only: plain holds (W/8)(H/8) floats, NaN where uncovered), then the
// comparison with the network's AO and the decision.
void launch_ao_probe_plain(const frd::FrameConst& F, frd::GBuffer gb, const float4* tbl, float* plain,
                           cudaStream_t st);
void launch_ao_probe_compare(const frd::FrameConst& F, const float* ao, const float* plain, float threshold,
                             float* part, unsigned* done, int* gate, float* mean, cudaStream_t st);

void launch_lighting(const frd::DevScene& S, const frd::FrameConst& F, frd::GBuffer gb, const float* shadow,
                     unsigned* frame8, float* frameF, cudaStream_t st, const int* counters = nullptr,
                     int* statusOut = nullptr);

void launch_ssaa(int W, int H, int k, const unsigned* frame8, unsigned* out, cudaStream_t st);

// Download helpers (reference AoS layouts).
void launch_unpack_gbuffer(const frd::DevScene& S, frd::GBuffer gb, int W, int H, int which, float* out,
                           cudaStream_t st);
// n pixels of R | G << 8 | B << 16 to packed R, G, B bytes.
void launch_pack_rgb(const unsigned* in, uint8_t* out, int n, cudaStream_t st);
void launch_triangle_ids(const unsigned long long* keys, int n, int* out, cudaStream_t st);

void set_shadow_tables(const float* blocker_xy_scaled, int nb, const float* pcf_xy, int np, cudaStream_t st);

}  // namespace frk
