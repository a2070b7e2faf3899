// fr_train_ao: trains the learned-AO U-Net on AO this renderer produces, and
// evaluates it through the frame's learned-AO path (network + probe) against
// the labels, next to plain SSAO.
//
// Labels: plain SSAO at cfg.label_samples samples + the render config's blur,
// rendered from random cameras on a hemisphere around the scene centre. The
// training set stays resident in HBM: per view 8 bytes of network input (four
// BF16 channels) and 4 bytes of label per pixel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fr_aonet.h"
#include "fr_aonet_internal.h"
#include "fr_context_internal.h"

namespace
{

constexpr int kMaxBatch = 32;

struct CropJobs
{
    int view[kMaxBatch];
    int x0[kMaxBatch];
    int y0[kMaxBatch];
};

// Keeps channels 0..3 of the 8-channel network input of one view.
__global__ void k_compact(const uint4* __restrict__ src, uint2* __restrict__ dst, long long n)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_uint2(src[i].x, src[i].y);
}

// Batch of crops: input [B][1][crop][crop][8] (channels 4..7 zero) and labels [B][crop][crop].
__global__ void k_crop(const uint2* __restrict__ feat, const float* __restrict__ labels, CropJobs jobs, int B,
                       int crop, int W, int H, uint4* __restrict__ in, float* __restrict__ lab)
{
    const long long n = static_cast<long long>(B) * crop * crop;
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = static_cast<int>(i % crop);
    const long long r = i / crop;
    const int y = static_cast<int>(r % crop);
    const int b = static_cast<int>(r / crop);
    const long long src = static_cast<long long>(jobs.view[b]) * W * H + static_cast<long long>(jobs.y0[b] + y) * W +
                          (jobs.x0[b] + x);
    const uint2 f = feat[src];
    in[i] = make_uint4(f.x, f.y, 0u, 0u);
    lab[i] = labels[src];
}

// Label -1 where no triangle covers the pixel: outside the training loss.
__global__ void k_mask_background(float* __restrict__ label, const float* __restrict__ depth, long long n)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && !(depth[i] < FLT_MAX)) label[i] = -1.f;
}

// sse learned all, sse learned covered, sse plain all, sse plain covered, covered, max |learned|, max |plain|,
// sse of AO = 1 (no occlusion) covered
constexpr int kErrSums = 8;

__global__ void k_err(const float* __restrict__ label, const float* __restrict__ plain, const float* __restrict__ learned,
                      const float* __restrict__ depth, int n, float* __restrict__ part)
{
    __shared__ float red[kErrSums][8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float v[kErrSums] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < n)
    {
        const float dl = learned[i] - label[i], dp = plain[i] - label[i];
        const bool cov = depth[i] < FLT_MAX;
        v[0] = dl * dl;
        v[2] = dp * dp;
        if (cov)
        {
            v[1] = v[0];
            v[3] = v[2];
            v[4] = 1.f;
            v[5] = fabsf(dl);
            v[6] = fabsf(dp);
            v[7] = (1.f - label[i]) * (1.f - label[i]);
        }
    }
    for (int k = 0; k < kErrSums; ++k)
    {
        float x = v[k];
        for (int o = 16; o > 0; o >>= 1)
        {
            const float y = __shfl_down_sync(0xffffffffu, x, o);
            x = (k == 5 || k == 6) ? fmaxf(x, y) : x + y;
        }
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < kErrSums)
    {
        const int k = threadIdx.x;
        float x = red[k][0];
        for (int w = 1; w < 8; ++w) x = (k == 5 || k == 6) ? fmaxf(x, red[k][w]) : x + red[k][w];
        part[static_cast<size_t>(blockIdx.x) * kErrSums + k] = x;
    }
}

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double unit(uint64_t& s) { return static_cast<double>(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

// A camera on the hemisphere around the origin: distance uniform in [rmin, rmax],
// direction uniform in area over the cap cos(polar) in [cmin, cmax].
void sample_eye(uint64_t& s, const fr_ao_train_config& c, float eye[3])
{
    const double r = c.radius_min + (c.radius_max - c.radius_min) * unit(s);
    const double ct = c.cos_min + (c.cos_max - c.cos_min) * unit(s);
    const double st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
    const double ph = 6.283185307179586 * unit(s);
    eye[0] = static_cast<float>(r * st * std::cos(ph));
    eye[1] = static_cast<float>(r * ct);
    eye[2] = static_cast<float>(r * st * std::sin(ph));
}

struct Ctx
{
    fr_ctx* c = nullptr;
    ~Ctx()
    {
        if (c) fr_destroy(c);
    }
};

struct DevMem
{
    void* p = nullptr;
    ~DevMem()
    {
        if (p) cudaFree(p);
    }
};

}  // namespace

extern "C" {

void fr_ao_train_defaults(fr_ao_train_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->train_views = 2000;
    c->eval_views = 200;
    c->steps = 3000;
    c->batch = 16;
    c->crop = 256;
    c->lr = 1e-3f;
    c->label_samples = 256;
    c->radius_min = 4.f;
    c->radius_max = 8.f;
    c->cos_min = 0.25f;
    c->cos_max = 0.95f;
    c->seed = 1;
    c->log_every = 100;
    c->lr_final = 0.f;
}

int fr_train_ao(const fr_scene* scene, fr_aonet* net, const fr_config* render_cfg, const fr_ao_train_config* cfgp,
                fr_ao_train_report* rep, float* losses, char* err, size_t errlen)
{
    auto fail = [&](int code, const std::string& m) {
        if (err && errlen) std::snprintf(err, errlen, "%s", m.c_str());
        return code;
    };
    if (!scene || !net || !render_cfg || !cfgp || !rep) return fail(FR_ERR_INVALID, "null argument");
    const fr_ao_train_config C = *cfgp;
    if (C.batch < 1 || C.batch > kMaxBatch || C.crop < 32 || (C.crop % 32) || C.train_views < 1 || C.steps < 0 ||
        C.eval_views < 0 || C.label_samples < 1 || C.first_step < 0 || C.schedule_steps < 0)
        return fail(FR_ERR_INVALID, "bad training configuration");
    std::memset(rep, 0, sizeof *rep);
    const int dev = render_cfg->device;
    if (fra_device(net) != dev) return fail(FR_ERR_INVALID, "network and render config are on different devices");
    cudaSetDevice(dev);

    char cerr[512];
    fr_config cl = *render_cfg, cp = *render_cfg, cn = *render_cfg;
    cl.ssao_samples = C.label_samples;
    cl.ao_mode = FR_AO_SSAO;
    cp.ao_mode = FR_AO_SSAO;
    cn.ao_mode = FR_AO_LEARNED;
    cn.ao_probe_threshold = FLT_MAX;  // statistics only: never fall back during evaluation
    Ctx label, plain, learned;
    if (!(label.c = fr_create(&cl, cerr, sizeof cerr))) return fail(FR_ERR_CUDA, cerr);
    if (!(plain.c = fr_create(&cp, cerr, sizeof cerr))) return fail(FR_ERR_CUDA, cerr);
    if (!(learned.c = fr_create(&cn, cerr, sizeof cerr))) return fail(FR_ERR_CUDA, cerr);
    for (fr_ctx* c : {label.c, plain.c, learned.c})
        if (fr_upload_scene(c, scene) != FR_OK) return fail(FR_ERR_CUDA, fr_last_error(c));
    fr_set_ao_net(learned.c, net);

    const float target[3] = {0.f, 0.f, 0.f};
    fr_frame_matrices m;
    {
        float eye[3] = {0.f, 5.f, 5.f};
        fr_scene_view_matrices(scene, eye, target, 0, &m);
    }
    const int W = m.width, H = m.height;
    rep->width = W, rep->height = H;
    if (W < C.crop || H < C.crop || (W % 32) || (H % 32))
        return fail(FR_ERR_INVALID, "view smaller than the crop, or not a multiple of 32");
    const long long HW = static_cast<long long>(W) * H;
    cudaStream_t st = frctx_stream(label.c);

    DevMem feat, labels, tmp, bIn, bLab, errPart;
    if (cudaMalloc(&feat.p, sizeof(uint2) * HW * C.train_views) != cudaSuccess ||
        cudaMalloc(&labels.p, sizeof(float) * HW * C.train_views) != cudaSuccess ||
        cudaMalloc(&tmp.p, sizeof(uint4) * HW) != cudaSuccess ||
        cudaMalloc(&bIn.p, sizeof(uint4) * C.batch * C.crop * C.crop) != cudaSuccess ||
        cudaMalloc(&bLab.p, sizeof(float) * C.batch * C.crop * C.crop) != cudaSuccess ||
        cudaMalloc(&errPart.p, sizeof(float) * kErrSums * ((HW + 255) / 256)) != cudaSuccess)
        return fail(FR_ERR_OOM, "training set allocation failed");

    // ---- labels ----
    auto t0 = std::chrono::steady_clock::now();
    uint64_t vs = C.seed * 0x9E3779B97F4A7C15ull + 17;
    for (int v = 0; v < C.train_views; ++v)
    {
        float eye[3];
        sample_eye(vs, C, eye);
        fr_scene_view_matrices(scene, eye, target, 0, &m);
        fr_frame_params p{&m, nullptr};
        if (fr_geometry_pass(label.c, &p) != FR_OK || fr_ssao_pass(label.c, &p) != FR_OK)
            return fail(FR_ERR_CUDA, fr_last_error(label.c));
        fr_ao_features(label.c, static_cast<uint16_t*>(tmp.p), st);
        k_compact<<<static_cast<int>((HW + 255) / 256), 256, 0, st>>>(
            static_cast<const uint4*>(tmp.p), static_cast<uint2*>(feat.p) + HW * v, HW);
        cudaMemcpyAsync(static_cast<float*>(labels.p) + HW * v, frctx_ao(label.c), sizeof(float) * HW,
                        cudaMemcpyDeviceToDevice, st);
        k_mask_background<<<static_cast<int>((HW + 255) / 256), 256, 0, st>>>(static_cast<float*>(labels.p) + HW * v,
                                                                             frctx_depth(label.c), HW);
    }
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return fail(FR_ERR_CUDA, "label rendering failed");
    auto t1 = std::chrono::steady_clock::now();
    rep->label_seconds = std::chrono::duration<float>(t1 - t0).count();

    // ---- training ----
    // steps first_step .. first_step + steps - 1 of a run whose schedule has
    // schedule_steps steps; the crop stream draws 3 numbers per crop, so a resumed
    // run skips the draws of the steps already taken
    uint64_t cs = C.seed * 0xD1B54A32D192ED03ull + 5;
    for (long long k = 0; k < 3ll * C.batch * C.first_step; ++k) splitmix(cs);
    const int schedule = C.schedule_steps > 0 ? C.schedule_steps : C.first_step + C.steps;
    int logged = 0;
    for (int step = C.first_step; step < C.first_step + C.steps; ++step)
    {
        CropJobs jobs{};
        for (int b = 0; b < C.batch; ++b)
        {
            jobs.view[b] = static_cast<int>(splitmix(cs) % static_cast<uint64_t>(C.train_views));
            jobs.x0[b] = static_cast<int>(splitmix(cs) % static_cast<uint64_t>(W - C.crop + 1));
            jobs.y0[b] = static_cast<int>(splitmix(cs) % static_cast<uint64_t>(H - C.crop + 1));
        }
        const long long n = static_cast<long long>(C.batch) * C.crop * C.crop;
        k_crop<<<static_cast<int>((n + 255) / 256), 256, 0, st>>>(static_cast<const uint2*>(feat.p),
                                                                 static_cast<const float*>(labels.p), jobs, C.batch,
                                                                 C.crop, W, H, static_cast<uint4*>(bIn.p),
                                                                 static_cast<float*>(bLab.p));
        const bool log = (C.log_every > 0 && step % C.log_every == 0) || step == C.first_step + C.steps - 1;
        float loss = 0.f;
        int rc = fr_aonet_backward(net, static_cast<const uint16_t*>(bIn.p), static_cast<const float*>(bLab.p),
                                   C.batch, C.crop, C.crop, log ? &loss : nullptr, st);
        if (rc != FR_OK) return fail(rc, fr_aonet_last_error(net));
        float lr = C.lr;
        if (C.lr_final > 0.f && schedule > 1)
            lr = static_cast<float>(C.lr_final + 0.5 * (C.lr - C.lr_final) *
                                                     (1.0 + std::cos(3.141592653589793 * step / (schedule - 1))));
        rc = fr_aonet_adam_step(net, lr, 0.9f, 0.999f, 1e-8f, st);
        if (rc != FR_OK) return fail(rc, fr_aonet_last_error(net));
        if (log)
        {
            if (logged == 0) rep->first_loss = loss;
            rep->final_loss = loss;
            if (losses) losses[logged] = loss;
            ++logged;
        }
        rep->steps_done = step + 1 - C.first_step;
    }
    if (fr_aonet_check(net, st) != FR_OK) return fail(FR_ERR_CUDA, fr_aonet_last_error(net));
    auto t2 = std::chrono::steady_clock::now();
    rep->train_seconds = std::chrono::duration<float>(t2 - t1).count();

    // ---- evaluation through the frame path ----
    uint64_t es = C.seed * 0xA24BAED4963EE407ull + 99;
    double sse[4] = {0, 0, 0, 0}, cov = 0, mxl = 0, mxp = 0, probeSum = 0, probeMax = 0, sseNone = 0;
    const int nb = static_cast<int>((HW + 255) / 256);
    std::vector<float> part(static_cast<size_t>(nb) * kErrSums);
    for (int v = 0; v < C.eval_views; ++v)
    {
        float eye[3];
        sample_eye(es, C, eye);
        fr_scene_view_matrices(scene, eye, target, 0, &m);
        fr_frame_params p{&m, nullptr};
        for (fr_ctx* c : {label.c, plain.c, learned.c})
            if (fr_geometry_pass(c, &p) != FR_OK || fr_ssao_pass(c, &p) != FR_OK)
                return fail(FR_ERR_CUDA, fr_last_error(c));
        float pm = 0.f;
        int fb = 0;
        if (fr_ao_probe_result(learned.c, &pm, &fb) != FR_OK) return fail(FR_ERR_CUDA, fr_last_error(learned.c));
        cudaDeviceSynchronize();
        k_err<<<nb, 256, 0, st>>>(frctx_ao(label.c), frctx_ao(plain.c), frctx_ao(learned.c), frctx_depth(label.c),
                                  static_cast<int>(HW), static_cast<float*>(errPart.p));
        if (cudaMemcpyAsync(part.data(), errPart.p, sizeof(float) * part.size(), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return fail(FR_ERR_CUDA, "evaluation failed");
        for (int b = 0; b < nb; ++b)
        {
            const float* q = &part[static_cast<size_t>(b) * kErrSums];
            for (int k = 0; k < 4; ++k) sse[k] += q[k];
            cov += q[4];
            mxl = std::max(mxl, static_cast<double>(q[5]));
            mxp = std::max(mxp, static_cast<double>(q[6]));
            sseNone += q[7];
        }
        probeSum += pm;
        probeMax = std::max(probeMax, static_cast<double>(pm));
    }
    auto t3 = std::chrono::steady_clock::now();
    rep->eval_seconds = std::chrono::duration<float>(t3 - t2).count();
    if (C.eval_views > 0)
    {
        const double all = static_cast<double>(HW) * C.eval_views;
        rep->eval_rmse = static_cast<float>(std::sqrt(sse[0] / all));
        rep->eval_rmse_covered = static_cast<float>(std::sqrt(sse[1] / std::max(cov, 1.0)));
        rep->plain_rmse = static_cast<float>(std::sqrt(sse[2] / all));
        rep->plain_rmse_covered = static_cast<float>(std::sqrt(sse[3] / std::max(cov, 1.0)));
        rep->eval_max_err = static_cast<float>(mxl);
        rep->plain_max_err = static_cast<float>(mxp);
        rep->probe_mean_avg = static_cast<float>(probeSum / C.eval_views);
        rep->probe_mean_max = static_cast<float>(probeMax);
        rep->none_rmse_covered = static_cast<float>(std::sqrt(sseNone / std::max(cov, 1.0)));
    }
    fr_set_ao_net(learned.c, nullptr);
    return FR_OK;
}

}  // extern "C"
