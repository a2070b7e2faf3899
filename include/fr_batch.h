/* fr_batch.h — many views of one scene rendered together: camera views of
 * uneven sizes plus per-light shadow maps, replayed as one CUDA graph.
 *
 * No counterpart in the reference, which renders one camera with one point
 * light (Render::Render, src/render.cpp:40-58); every view runs the same passes
 * and arithmetic as fr_render_frame. Stages of a batch:
 *   1. per light: light transform + triangle setup and tile binning of its shadow map,
 *      per view: camera transform + setup and binning           (parallel graph branches)
 *   2. one persistent launch over the (view-or-shadow-map, 16x16 tile) queue:
 *      the fine raster of every view and shadow map
 *   3. per light: shadow-map resolve; per view: G-buffer resolve and ambient
 *      occlusion (plain SSAO + blur, or the learned network with its probe)
 *   4. one persistent launch over the (view, T x T tile) queue: deferred lighting
 *      with all of the batch's lights (PBR sums the lights' direct terms before
 *      ambient, emission and tone mapping; Blinn-Phong materials use light 0).
 * With one view at the scene's camera and one light equal to the scene's point
 * light the frame is bit-identical to fr_render_frame's.
 */
#ifndef FR_BATCH_H
#define FR_BATCH_H

#include <stddef.h>
#include <stdint.h>

#include "forkerrenderer.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fr_view_desc
{
    fr_frame_matrices matrices; /* camera matrices and size (the shadow fields are unused) */
    float eye[3];               /* camera position (the lighting's view vector)           */
    int32_t ao_mode;            /* FR_AO_SSAO or FR_AO_LEARNED (needs fr_set_ao_net)      */
} fr_view_desc;

enum fr_light_type { FR_LIGHT_POINT = 0, FR_LIGHT_DIRECTIONAL = 1 };

typedef struct fr_light_desc
{
    int32_t type;         /* fr_light_type                                                         */
    float position[3];    /* point light: position; its shadow map uses the reference's frustum
                             (ortho +-3*aspect x +-3, near 0.1, far 20, looking at the origin)    */
    float direction[3];   /* directional light: the direction the light travels; shadow map ortho
                             +-extent x +-extent around the origin                               */
    float color[3];
    float extent;         /* directional: half size of the shadow frustum (world units)          */
    int32_t shadow_size;  /* S x S shadow map                                                    */
} fr_light_desc;

typedef struct fr_batch_tuning
{
    int32_t light_tile;   /* lighting work-item tile edge: 8, 16 or 32                            */
    int32_t bin_batch;    /* triangles the fine raster stages per shared-memory batch: 64, 256, 1024 */
    int32_t ctas_per_sm;  /* CTAs per SM of both persistent launches: 1, 2 or 4                   */
} fr_batch_tuning;

typedef struct fr_batch fr_batch;

/* The context's scene and configuration (shadow mode, sample counts, SSAO
 * parameters, blur) apply to every view. At most 4 lights. */
fr_batch* fr_batch_create(fr_ctx* ctx, const fr_view_desc* views, int32_t n_views, const fr_light_desc* lights,
                          int32_t n_lights, char* err, size_t errlen);
void fr_batch_destroy(fr_batch* batch);
const char* fr_batch_last_error(const fr_batch* batch);

int fr_batch_set_tuning(fr_batch* batch, const fr_batch_tuning* tuning);
int fr_batch_get_tuning(const fr_batch* batch, fr_batch_tuning* tuning);

/* Renders every view: one CUDA graph launch on the context's stream (captured on
 * the first call and after a tuning change). */
int fr_batch_render(fr_batch* batch);

/* Device milliseconds of the last render: [transforms + setup + binning,
 * persistent fine raster, resolves + ambient occlusion, persistent lighting,
 * total]. Waits for the batch. */
int fr_batch_timings(fr_batch* batch, float* ms, int32_t n);

/* Sweeps light_tile {8,16,32} x bin_batch {64,256,1024} x ctas_per_sm {1,2,4},
 * keeps the fastest (median of `reps` renders each). */
int fr_batch_autotune(fr_batch* batch, int32_t reps, fr_batch_tuning* best, float* best_ms);

/* Work of one render: triangles set up (scene triangles x (views + lights))
 * and pixels shaded (the views' pixels). */
int fr_batch_work(const fr_batch* batch, int64_t* triangles, int64_t* pixels, int64_t* shadow_texels);

/* Reads one buffer of view `view` (FR_BUF_FRAME_U8, FR_BUF_DEPTH, FR_BUF_AO) or,
 * with view = -1 - k, light k's shadow map (FR_BUF_SHADOW). Same layouts and
 * return convention as fr_download. */
int64_t fr_batch_download(fr_batch* batch, int32_t view, int32_t buffer_id, void* dst, size_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* FR_BATCH_H */
