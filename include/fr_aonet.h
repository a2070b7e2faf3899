/* fr_aonet.h — learned ambient occlusion: a small U-Net that maps view-space
 * depth and normals to the AO buffer that the renderer's SSAO pass + blur
 * produce (Render::DoSSAO, src/render.cpp:214-289, and
 * Buffer1f::TwoPassGaussianBlurDenoised, src/buffer.cpp:59-98).
 *
 * The reference has no learned AO; these entry points have no counterpart
 * there. They are the "fr_train_ao / fr_set_ao_weights" half of the C ABI.
 *
 * Network (all convolutions 3x3, zero padding, ReLU; BF16 weights and
 * activations, FP32 accumulation on the tensor cores):
 *   level 0 (H x W):      e0a 4->16, e0b 16->16 (skip s0), 2x2 average pool
 *   level 1 (H/2 x W/2):  e1a 16->32, e1b 32->32 (skip s1), 2x2 average pool
 *   level 2 (H/4 x W/4):  b0 32->64, b1 64->64, bilinear x2 upsample
 *   level 1:              d1a [up 64 | s1 32]->32, d1b 32->32, bilinear x2 upsample
 *   level 0:              d0a [up 32 | s0 16]->16, d0b 16->16, 1x1 16->1, sigmoid
 * Parameter order (FP32): for each of the 10 3x3 layers W[cout][cin][3][3]
 * then b[cout]; then the head's w[16] and b[1].
 *
 * Input tensor ("chunk-planar" BF16): [B][1][H][W][8], channels 0..3 =
 * view-space depth / 8 (positive, 0 for background), view-space normal xyz;
 * channels 4..7 zero. H and W must be multiples of 4.
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

#define FR_AONET_NUM_PARAMS 118417
#define FR_AONET_MAX_PIXELS (16 * 256 * 256 * 4) /* B*H*W capacity of one call */

/* Creates a network on `device` with He-normal weights drawn from `seed`. */
fr_aonet* fr_aonet_create(int32_t device, uint64_t seed, char* err, size_t errlen);
void fr_aonet_destroy(fr_aonet* net);
const char* fr_aonet_last_error(const fr_aonet* net);
int64_t fr_aonet_num_params(void);

/* FP32 master parameters, in the order above. */
int fr_aonet_get_params(fr_aonet* net, float* dst, int64_t count);
int fr_aonet_set_params(fr_aonet* net, const float* src, int64_t count);

/* AO = net(in). in: device BF16 [B][1][H][W][8]; ao: device FP32 [B][H][W]. */
int fr_aonet_forward(fr_aonet* net, const uint16_t* in, int32_t B, int32_t H, int32_t W, float* ao, void* stream);

/* Mean squared error against `label` (device FP32 [B][H][W]) and the gradient
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

/* Waits for `stream` and reports a kernel status (a timed-out pipeline wait) as FR_ERR_CUDA. */
int fr_aonet_check(fr_aonet* net, void* stream);

/* Number of kernels the last forward / train step launched. */
int32_t fr_aonet_last_launch_count(const fr_aonet* net);

/* ---- renderer integration ---------------------------------------------------- */

/* The network `fr_render_frame` uses when fr_config.ao_mode == FR_AO_LEARNED
 * (NULL detaches). The context does not own it. */
int fr_set_ao_net(fr_ctx* ctx, fr_aonet* net);

/* The network's input for the last geometry pass, written to `dst` (device BF16
 * [1][1][H][W][8]). */
int fr_ao_features(fr_ctx* ctx, uint16_t* dst, void* stream);

/* Probe of the learned AO: the mean squared difference between the network's AO
 * and plain SSAO (fr_config.ssao_samples, no blur) on one pixel in 64, and
 * whether the last frame fell back to plain SSAO + blur because that mean
 * exceeded fr_config.ao_probe_threshold. Waits for the frame. */
int fr_ao_probe_result(fr_ctx* ctx, float* mean_sq_diff, int32_t* fell_back);

/* Frame matrices of the scene seen from `eye` looking at `target` (the scene's
 * camera otherwise: perspective fov 45, near 0.01, far 20, render.cpp:73-78). */
int fr_scene_view_matrices(const fr_scene* scene, const float eye[3], const float target[3], int32_t shadow_size,
                           fr_frame_matrices* out);

#ifdef __cplusplus
}
#endif

#endif /* FR_AONET_H */
