/*
 * CPU oracle of the per-frame pipeline (TEST INFRASTRUCTURE ONLY).
 *
 * A plain C++ restatement of the reference renderer's frame, statement by
 * statement in the reference's own order and float/double types, used only by
 * tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the
 * checker of the GB300 path. Nothing in the product links or calls it.
 *
 * Parity of this oracle is pinned against the reference itself: the reference
 * sources are compiled from where they lie by oracle/Makefile.ref together with
 * oracle/ref_harness.cpp, and tests/golden/ holds its outputs on seeded scenes
 * (tests/golden/make_golden.py); tests/test_oracle_golden.py checks this
 * oracle against them bit for bit.
 */
#ifndef FR_ORACLE_H
#define FR_ORACLE_H

#include <stdint.h>

#include "forkerrenderer.h"
#include "fr_batch.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fr_oracle_config
{
    int32_t shadow_mode;     /* 0 hard, 1 PCF, 2 PCSS                            */
    int32_t shadow_size;     /* 0 = screen sized (reference), else S x S          */
    int32_t pcf_samples, blocker_samples, ssao_samples;
    float ssao_radius, ssao_bias, ssao_range;
    int32_t blur_mode;       /* 0 reference in-place, 1 separable, 2 none          */
    int32_t threads;         /* worker threads (>= 1)                              */
    int32_t texture_wrap;    /* Texture::WrapMode: 0 NoWrap, 1 Repeat, 2 Mirrored, 3 Clamp */
    int32_t texture_filter;  /* Texture::FilterMode: 0 Nearest, 1 Linear (bilinear)  */
} fr_oracle_config;

/* Output buffers, caller allocated (NULL = not wanted). Sizes: W x H working
 * resolution, Sw x Sh shadow map, w x h SSAA output; layouts as the reference's
 * Buffer1f / Buffer3f (x + y * width). */
typedef struct fr_oracle_out
{
    float* depth;        /* W*H                                                  */
    float* shadow;       /* Sw*Sh                                                */
    float* gb_normal;    /* W*H*3 (deferred only)                               */
    float* gb_position;
    float* gb_lightndc;
    float* gb_albedo;
    float* gb_emissive;
    float* gb_param;
    float* gb_type;      /* W*H                                                  */
    float* ao;           /* W*H                                                  */
    float* frame;        /* W*H*3 float                                          */
    uint8_t* frame8;     /* W*H*3 GenerateImage() bytes                          */
    uint8_t* ssaa8;      /* (W/k)*(H/k)*3                                        */
    double seconds;      /* wall time of the frame (set by the oracle)           */
} fr_oracle_out;

/* The frame matrices restated from geometry.cpp:60-179 / render.cpp. */
int fr_oracle_matrices(const fr_scene_view* scene, int32_t shadow_size, fr_frame_matrices* out);

/* One frame. mats NULL = fr_oracle_matrices(scene, cfg->shadow_size). */
int fr_oracle_render(const fr_scene_view* scene, const fr_oracle_config* cfg,
                     const fr_frame_matrices* mats, fr_oracle_out* out);

/* One view of the batched renderer (include/fr_batch.h), which has no reference
 * counterpart: the camera `view` (its shadow fields unused) seen from `eye`,
 * deferred, lit by 1..4 point or directional lights each with its own
 * shadow_size^2 shadow map (written to shadows[k] when non-NULL). */
int fr_oracle_render_lights(const fr_scene_view* scene, const fr_oracle_config* cfg,
                            const fr_frame_matrices* view, const float eye[3], const fr_light_desc* lights,
                            int32_t n_lights, fr_oracle_out* out, float* const* shadows);

/* TGA output (oracle/fr_oracle_tga.cpp): the reference's float -> uint8 image
 * conversions and its TGA writer. */
uint8_t fr_oracle_u8(float v);
void fr_oracle_image_1f(const float* v, int64_t n, uint8_t* out);  /* Buffer1f::GenerateImage */
void fr_oracle_image_3f(const float* v, int64_t n, uint8_t* out);  /* Buffer3f::GenerateImage (B, G, R) */
int64_t fr_oracle_tga_max_bytes(int64_t width, int64_t height, int32_t bytespp);
/* File bytes into out (cap >= fr_oracle_tga_max_bytes); returns the size, -1 on bad arguments. */
int64_t fr_oracle_tga_encode(const uint8_t* px, int32_t width, int32_t height, int32_t bytespp, int32_t rle,
                             int32_t vflip, uint8_t* out, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
