/* fr_aonet.h — learned ambient occlusion: a small U-Net that maps view-space
 * depth and normals to the AO buffer that the renderer's SSAO pass + blur
 * produce (Render::DoSSAO, src/render.cpp:214-289, and
 * Buffer1f::TwoPassGaussianBlurDenoised, src/buffer.cpp:59-98).
 *
 * The reference has no learned AO; these entry points have no counterpart
 * there. They are the "fr_train_ao / fr_set_ao_weights" half of the C ABI.
 *
 * Network (all convolutions 3x3, zero padding, ReLU; BF16 weights and
 * activations, FP32 accumulation on the tensor cores). Level 0 works on 2x2
 * pixel blocks: the 4-channel input is rearranged space-to-depth into 16
 * channels at H/2 x W/2 and the 1x1 head emits each block's four sub-pixel AO
 * values. Levels are 4x apart: 4x4 average pooling down, bilinear x4
 * upsampling (half-pixel centres) up. The receptive field (about +-150 pixels)
 * covers the SSAO kernel's screen footprint.
 *   level 0 (H/2 x W/2):    e0a 16->16, e0b 16->16 (skip s0), pool
 *   level 1 (H/8 x W/8):    e1a 16->32, e1b 32->32 (skip s1), pool
 *   level 2 (H/32 x W/32):  b0 32->64, b1 64->64, upsample
 *   level 1:                d1a [up 64 | s1 32]->32, d1b 32->32, upsample
 *   level 0:                d0a [up 32 | s0 16]->16, d0b 16->16, 1x1 16->4, sigmoid
 * Parameter order (FP32): for each of the 10 3x3 layers W[cout][cin][3][3]
 * then b[cout]; then the head's w[4][16] and b[4] (output k = sub-pixel
 * (k / 2, k % 2) of the block).
 *
 * Input tensor ("chunk-planar" BF16): [B][1][H][W][8], channels 0..3 =
 * view-space depth / 8 (positive, 0 for background), view-space normal x, y,
 * and channel 3 = the normal's z (fr_config.ao_input_samples = 0), the depth
 * channel's BF16 rounding residual times 256 (ao_input_samples = -1: depth to
 * about 16 mantissa bits, from view depth and normal alone) or a K-sample
 * SSAO of the pixel without blur (ao_input_samples = K); channels 4..7 zero;
 * all zero for background pixels. H and W must be multiples of 32.
 */
#ifndef FR_AONET_H
#define FR_AONET_H

#include <stddef.h>
#include <stdint.h>

#include "forkerrenderer.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fr_aonet fr_aonet;

#define FR_AONET_NUM_PARAMS 120196
#define FR_AONET_MAX_PIXELS (16 * 256 * 256 * 4) /* B*H*W capacity of one call */

/* Creates a network on `device` with He-normal weights drawn from `seed`. */
fr_aonet* fr_aonet_create(int32_t device, uint64_t seed, char* err, size_t errlen);
void fr_aonet_destroy(fr_aonet* net);
const char* fr_aonet_last_error(const fr_aonet* net);
int64_t fr_aonet_num_params(void);

/* 1: the renderer runs the network's forward for a frame as one cooperative
 * launch of a persistent kernel (every layer, grid barriers between them);
 * 0 (default): one launch per layer, each a programmatic dependent of the one
 * before. Both give identical results; at 1280x800 the single launch is the
 * slower (one CTA per SM leaves each layer's epilogue without the overlap that
 * several CTAs per SM give). */
int fr_aonet_set_fused(fr_aonet* net, int32_t fused);

/* FP32 master parameters, in the order above. */
int fr_aonet_get_params(fr_aonet* net, float* dst, int64_t count);
int fr_aonet_set_params(fr_aonet* net, const float* src, int64_t count);

/* AO = net(in). in: device BF16 [B][1][H][W][8]; ao: device FP32 [B][H][W]. */
int fr_aonet_forward(fr_aonet* net, const uint16_t* in, int32_t B, int32_t H, int32_t W, float* ao, void* stream);

/* Mean squared error against `label` (device FP32 [B][H][W]; pixels whose label
 * is negative are left out of the loss, the mean still divides by B*H*W) and the gradient
 * of every parameter (readable with fr_aonet_get_grads). `loss` (host) may be
 * NULL; when given, the call waits for the stream. */
int fr_aonet_backward(fr_aonet* net, const uint16_t* in, const float* label, int32_t B, int32_t H, int32_t W,
                      float* loss, void* stream);
int fr_aonet_get_grads(fr_aonet* net, float* dst, int64_t count);

/* One Adam update (PyTorch's formulation, bias-corrected) from the last gradient. */
int fr_aonet_adam_step(fr_aonet* net, float lr, float beta1, float beta2, float eps, void* stream);

/* Forward + backward + Adam. */
int fr_aonet_train_step(fr_aonet* net, const uint16_t* in, const float* label, int32_t B, int32_t H, int32_t W,
                        float lr, float* loss, void* stream);

/* The whole training state: parameters, Adam's first and second moments (count =
 * fr_aonet_num_params() floats each; NULL = not wanted) and Adam's step count.
 * With fr_ao_train_config.first_step this resumes a run exactly: N steps, a
 * checkpoint, a set_state and M more steps give the same floats as N + M steps. */
int fr_aonet_get_state(fr_aonet* net, float* params, float* adam_m, float* adam_v, int64_t count,
                       int64_t* adam_step);
int fr_aonet_set_state(fr_aonet* net, const float* params, const float* adam_m, const float* adam_v, int64_t count,
                       int64_t adam_step);

/* Waits for `stream` and reports a kernel status (a timed-out pipeline wait or
 * grid barrier) as FR_ERR_TIMEOUT, clearing it. */
int fr_aonet_check(fr_aonet* net, void* stream);

/* Longest wait of a CTA at a grid barrier of the fused forward (fr_aonet_set_fused)
 * before the launch gives up, in nanoseconds (0 = the default, 2 s). A wait that
 * runs out sets the network's status: the kernel returns, its TMEM freed, and the
 * next fr_aonet_check (or the renderer's next synchronising call) reports
 * FR_ERR_TIMEOUT; the network stays usable. */
int fr_aonet_set_wait_limit(fr_aonet* net, uint64_t ns);

/* For tests of that bounded wait: CTA `cta` of the fused forward leaves after the
 * first stage without arriving at its grid barrier, so the others wait until the
 * limit (-1 = off, the default). Nothing runs out of bounds: the absent CTA's
 * stage is complete and the others stop at the barrier. */
int fr_aonet_test_absent_cta(fr_aonet* net, int32_t cta);

/* Number of kernels the last forward / train step launched. */
int32_t fr_aonet_last_launch_count(const fr_aonet* net);

/* ---- renderer integration ---------------------------------------------------- */

/* The network `fr_render_frame` uses when fr_config.ao_mode == FR_AO_LEARNED
 * (NULL detaches). The context does not own it. */
int fr_set_ao_net(fr_ctx* ctx, fr_aonet* net);

/* The network's input for the last geometry pass, written to `dst` (device BF16
 * [1][1][H][W][8]), channel 3 as the context's ao_input_samples says. */
int fr_ao_features(fr_ctx* ctx, uint16_t* dst, void* stream);

/* Probe of the learned AO: the mean squared difference between the network's AO
 * and plain SSAO (fr_config.ssao_samples, no blur) on one pixel in 64, and
 * whether the last frame fell back to plain SSAO + blur because that mean
 * exceeded fr_config.ao_probe_threshold. Waits for the frame. */
int fr_ao_probe_result(fr_ctx* ctx, float* mean_sq_diff, int32_t* fell_back);

/* ---- training (fr_train_ao) ------------------------------------------------------ */

typedef struct fr_ao_train_config
{
    int32_t train_views;     /* random camera views rendered for training (2000)            */
    int32_t eval_views;      /* held-out views for evaluation (200)                          */
    int32_t steps;           /* Adam steps                                                   */
    int32_t batch;           /* crops per step (16)                                          */
    int32_t crop;            /* crop edge in pixels, a multiple of 32 (256)                  */
    float lr;                /* Adam learning rate (1e-3)                                    */
    int32_t label_samples;   /* SSAO samples of the labels (256)                             */
    float radius_min;        /* camera distance from the scene centre (4)                    */
    float radius_max;        /* (8)                                                          */
    float cos_min, cos_max;  /* range of the camera direction's vertical cosine (0.25, 0.95) */
    uint64_t seed;           /* views, crops                                                 */
    int32_t log_every;       /* loss read-back interval in steps (0 = end only)              */
    float lr_final;          /* learning rate at the last step: cosine decay from lr; 0 = lr */
    int32_t first_step;      /* resume: index of the first step run (0 = from the start); the
                                crop stream and the learning-rate schedule continue from it,
                                with the network's state restored by fr_aonet_set_state       */
    int32_t schedule_steps;  /* length of the cosine schedule (0 = first_step + steps)        */
} fr_ao_train_config;

typedef struct fr_ao_train_report
{
    int32_t steps_done;
    float first_loss, final_loss;    /* mean squared error of the first / last logged batch   */
    float eval_rmse;                 /* learned AO vs label, all pixels of the eval views      */
    float eval_rmse_covered;         /* learned AO vs label, pixels covered by geometry        */
    float eval_max_err;              /* max |learned - label| (covered pixels)                 */
    float plain_rmse;                /* plain SSAO (render config's samples + blur) vs label   */
    float plain_rmse_covered;
    float plain_max_err;
    float probe_mean_avg, probe_mean_max;  /* the probe statistic over the eval views          */
    float label_seconds, train_seconds, eval_seconds;
    int32_t width, height;           /* view size (the scene's)                                */
    float none_rmse_covered;         /* AO = 1 (no ambient occlusion) vs label, covered pixels */
} fr_ao_train_report;

void fr_ao_train_defaults(fr_ao_train_config* cfg);

/* Trains `net` on AO this renderer produces: views of `scene` from cameras on a
 * hemisphere around the scene centre, labelled with plain SSAO at
 * cfg->label_samples samples followed by render_cfg's blur; random crops, Adam.
 * Pixels no triangle covers are left out of the loss (lighting never reads their AO).
 * Then evaluates on cfg->eval_views further views against the same labels, next
 * to plain SSAO with render_cfg's sample count. render_cfg gives the SSAO
 * radius / bias / range / blur and the device. `losses` (host, optional) receives
 * the logged losses (cfg->steps / cfg->log_every + 1 floats). */
int fr_train_ao(const fr_scene* scene, fr_aonet* net, const fr_config* render_cfg, const fr_ao_train_config* cfg,
                fr_ao_train_report* report, float* losses, char* err, size_t errlen);

/* Frame matrices of the scene seen from `eye` looking at `target` (the scene's
 * camera otherwise: perspective fov 45, near 0.01, far 20, render.cpp:73-78). */
int fr_scene_view_matrices(const fr_scene* scene, const float eye[3], const float target[3], int32_t shadow_size,
                           fr_frame_matrices* out);

#ifdef __cplusplus
}
#endif

#endif /* FR_AONET_H */
