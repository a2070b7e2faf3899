/*
 * ForkerRenderer-GB300: C ABI of the per-frame rasterisation pipeline.
 *
 * The reference renderer has no plugin or FFI; its seam is the C++ namespace
 * Render:: (src/render.h:22-37) over the static ForkerGL:: state
 * (src/forkergl.h:41-55), reached from main() as
 *     Scene scene(file);  Render::Preconfigure(scene);  Render::Render(scene);
 * (src/main.cpp:33-40) and read back by Output:: (src/output.cpp:12-86).
 * This header is that seam as a C ABI: plain pointers and sizes, status codes,
 * no C++ or torch types. Each entry point names the reference code it replaces.
 *
 * Conventions: functions return FR_OK (0) or a negative FR_ERR_* code; the
 * message of the last failure of a context is fr_last_error(ctx). A context owns
 * its device memory; callers own host buffers. A context is not thread-safe;
 * separate contexts are independent. Every call is asynchronous on the context's
 * stream unless it copies to host memory (fr_download / fr_*_timings), which
 * synchronises that stream.
 */
#ifndef FORKERRENDERER_H
#define FORKERRENDERER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define FR_OK 0
#define FR_ERR_INVALID -1      /* bad argument or call order                      */
#define FR_ERR_IO -2           /* scene / model / texture file unreadable          */
#define FR_ERR_PARSE -3        /* malformed .scene / .obj / .mtl / .tga            */
#define FR_ERR_CUDA -4         /* CUDA runtime failure (message has the detail)    */
#define FR_ERR_OOM -5          /* device allocation failed                          */
#define FR_ERR_BIN_OVERFLOW -6 /* tile-bin capacity exceeded; raise bin_capacity    */
#define FR_ERR_TIMEOUT -7      /* a bounded device wait gave up                     */
#define FR_ERR_UNSUPPORTED -8  /* option outside what this build implements         */

/* ---- scene (host side) ------------------------------------------------------ */
typedef struct fr_scene fr_scene;

/* Parses a .scene file and every .obj/.mtl/.tga it names, exactly as the
 * reference loader does (Scene::Scene src/scene.cpp:19-196, Model::Load
 * src/model.cpp:16-73 with loadObjectFile :143-255, loadMaterials :258-408,
 * generateTangents :430-476, normalizePositionVertices :107-138,
 * TGAImage::ReadTgaFile src/tgaimage.cpp:43-105). Relative model paths are
 * resolved against the directory of the .scene file. Returns NULL on failure
 * and, if err is non-NULL, writes a message into err[0..errlen). */
fr_scene* fr_scene_load(const char* scene_path, char* err, size_t errlen);
void fr_scene_free(fr_scene* scene);

typedef struct fr_scene_info
{
    int32_t width, height;   /* "screen" (scene.cpp:77-81), default 1280 x 800   */
    int32_t deferred;        /* "mode deferred" (scene.cpp:58-76)                 */
    int32_t ssaa_on, ssaa_kernel; /* "ssaa on|off k" (scene.cpp:82-87)           */
    int32_t ssao_on;         /* "ssao on|off"                                       */
    int32_t shadow_on;       /* "shadow on|off" (Shadow::SetShadowStatus)          */
    int32_t perspective;     /* "camera persp|ortho"                                */
    float eye[3], target[3]; /* camera look-from / look-at                          */
    float light_pos[3], light_color[3]; /* "light point x y z r g b"              */
    int32_t num_models, num_meshes, num_materials, num_textures;
    int64_t num_vertices, num_uvs, num_normals, num_triangles;
} fr_scene_info;

int fr_scene_get_info(const fr_scene* scene, fr_scene_info* out);

/* Read-only view of the flattened scene (valid while the scene lives).
 * Triangles are in the reference's draw order: scene model order, then mesh
 * name order within a model (std::map, src/model.h:44), then face order; the
 * position of a triangle in this order is its global index, the tie-break of
 * the depth test. Index arrays hold GLOBAL indices into the vertex arrays. */
typedef struct fr_model_view
{
    float model_matrix[16]; /* MakeModelMatrix (geometry.cpp:92-108), row major */
    float position[3], rotate_y, scale;
    int32_t has_tangents;   /* generateTangent flag of the "model" line          */
    int32_t support_pbr;    /* Model::SupportPBR (model.cpp:52-68)               */
    int32_t first_mesh, num_meshes;
    int64_t first_vertex, num_vertices, first_normal, num_normals;
} fr_model_view;

typedef struct fr_mesh_view
{
    int32_t model, material;
    int64_t first_triangle, num_triangles;
} fr_mesh_view;

/* Material + PBRMaterial (the headers under src/materials) merged; texture slots are indices
 * into the texture table or -1 (no map). */
typedef struct fr_material_view
{
    float ka[3], kd[3], ks[3], ke[3];
    float pbr_albedo[3];           /* PBRMaterial::albedo, default 1, set by Kd */
    float roughness, metalness;    /* Pr / Pm                                    */
    int32_t map_kd, map_ks, map_ke, map_bump, map_ao, map_pr, map_pm;
} fr_material_view;

/* Texture bytes as TGAImage holds them after both vertical flips: row-major
 * x + y * width, bytes_per_pixel in {1, 3, 4}, channel order B, G, R, A. */
typedef struct fr_texture_view
{
    int32_t width, height, bytes_per_pixel;
    const uint8_t* data;
} fr_texture_view;

typedef struct fr_scene_view
{
    fr_scene_info info;
    const fr_model_view* models;
    const fr_mesh_view* meshes;
    const fr_material_view* materials;
    const fr_texture_view* textures;
    const float* positions; /* 3 * num_vertices, model space                       */
    const float* uvs;       /* 2 * num_uvs                                          */
    const float* normals;   /* 3 * num_normals, as read (not normalised)            */
    const float* tangents;  /* 3 * num_vertices (unit, (1,0,0) if none); 0 where the
                               model has no tangents                                */
    const int32_t* tri_v;   /* 3 * num_triangles                                    */
    const int32_t* tri_vt;
    const int32_t* tri_vn;
    const int32_t* tri_mesh; /* num_triangles                                        */
} fr_scene_view;

int fr_scene_get_view(const fr_scene* scene, fr_scene_view* out);

/* The inverse of fr_scene_get_view: a scene built from caller-owned arrays laid
 * out as fr_scene_view describes them (the arrays are copied; info's counts give
 * their lengths). This is how a host that already holds the reference's Scene
 * (src/scene.h:61-71, with its Model / Mesh / Material / Texture objects,
 * model.h:15-70, mesh.h:16-64) hands it over without a file: every index is
 * checked against the counts. tangents: one unit vector per vertex as
 * Model::generateTangents left them (model.cpp:430-476), or NULL to have them
 * generated from the faces for the models whose has_tangents is set. Returns
 * NULL on failure with a message in err[0..errlen). */
fr_scene* fr_scene_from_view(const fr_scene_view* view, char* err, size_t errlen);

/* ---- frame matrices (host side, reference operation order) ------------------ */
typedef struct fr_frame_matrices
{
    float view[16], projection[16], view_projection[16]; /* camera            */
    float light_space[16];  /* Ortho(+-3*aspect, +-3, 0.1, 20) * LookAt(light -> 0)
                               (render.cpp:73-78)                                */
    float viewport[16];     /* SetViewportMatrix(0,0,W',H') (forkergl.cpp:89-102) */
    float shadow_viewport[16];
    int32_t width, height;  /* working (SSAA-scaled) size, render.cpp:21-31       */
    int32_t shadow_width, shadow_height;
} fr_frame_matrices;

/* Computes every matrix of one frame with the reference's float operation order
 * (MakeLookAtMatrix / MakePerspectiveMatrix / MakeOrthographicMatrix,
 * geometry.cpp:110-179; fov 45, near 0.01, far 20, render.cpp:9-14,106-114).
 * shadow_size 0 = screen-sized shadow map rasterised with the screen viewport,
 * as the reference does (render.cpp:68); S > 0 = S x S map with its own viewport. */
int fr_scene_frame_matrices(const fr_scene* scene, int32_t shadow_size, fr_frame_matrices* out);

/* ---- render context --------------------------------------------------------- */
enum fr_shadow_mode { FR_SHADOW_HARD = 0, FR_SHADOW_PCF = 1, FR_SHADOW_PCSS = 2 };
enum fr_blur_mode
{
    FR_BLUR_REFERENCE = 0, /* in-place two-pass Gaussian, sequential per row / column,
                              bit-exact with Buffer1f::TwoPassGaussianBlurDenoised
                              (buffer.cpp:59-98)                                       */
    FR_BLUR_SEPARABLE = 1, /* ping-pong separable Gaussian (parallel; not in-place)  */
    FR_BLUR_NONE = 2
};
enum fr_ao_mode { FR_AO_SSAO = 0, FR_AO_LEARNED = 1 };

typedef struct fr_config
{
    int32_t shadow_mode;      /* fr_shadow_mode; reference default PCSS (shadow.h:16) */
    int32_t shadow_size;      /* 0 = screen sized (reference), else S x S              */
    int32_t pcf_samples;      /* PCF_NUM_SAMPLES, reference 64 (shadow.h:20)            */
    int32_t blocker_samples;  /* PCSS_BLOCKER_SEARCH_NUM_SAMPLES, reference 32          */
    int32_t ssao_samples;     /* reference 32 (render.cpp:219); 1..256                  */
    float ssao_radius;        /* reference 0.075 (render.cpp:222)                       */
    float ssao_bias;          /* reference 0.0005 (render.cpp:258)                      */
    float ssao_range;         /* range check, reference 0.01 (render.cpp:224)           */
    int32_t blur_mode;        /* fr_blur_mode                                            */
    int32_t ao_mode;          /* fr_ao_mode                                              */
    int32_t keep_float_frame; /* also keep FrameBuffer as float RGB (download/tests)    */
    int32_t small_tri_area;   /* raster: bbox area (px, 0..65536) up to which a triangle's
                                 pixels are dealt to the lanes of its setup warp        */
    int32_t medium_tri_area;  /* raster: bbox area (px, 0..2^20) up to which a triangle is
                                 drawn by one warp; larger ones go through 16x16 tile
                                 bins                                                   */
    int64_t bin_capacity;     /* max (triangle, tile) pairs per pass; 0 = automatic    */
    int32_t device;           /* CUDA device ordinal                                    */
    float ao_probe_threshold; /* learned AO: mean squared difference to plain SSAO on the
                                 1-in-64 probe above which the frame falls back to plain
                                 SSAO + blur (fr_aonet.h)                               */
    int32_t frame_graph;      /* 1: fr_render_frame captures the frame's launches into a CUDA
                                 graph and replays it while the frame constants, stream and
                                 buffers are unchanged (the first such frame runs directly) */
    int32_t ao_input_samples; /* learned AO input: 0 = view depth + view normal (x, y, z);
                                 -1 = view depth, normal x, y and the depth channel's BF16
                                 rounding residual x 256 (depth to ~16 mantissa bits);
                                 K > 0 = view depth, normal x, y and a K-sample SSAO of the
                                 pixel (no blur) that the network denoises (fr_aonet.h)   */
    int32_t texture_wrap;     /* Texture::WrapMode of every texture (texture.h:14-20,
                                 62-83): 0 NoWrap (the reference's setting, render.cpp:36),
                                 1 Repeat, 2 MirroredRepeat, 3 ClampToEdge               */
    int32_t texture_filter;   /* Texture::FilterMode of every texture (texture.h:85-127):
                                 0 Nearest (the reference's setting, render.cpp:37),
                                 1 Linear (bilinear; deferred frames then keep the texture
                                 coordinate in the G-buffer and sample where it is read) */
    int32_t concurrent_passes; /* 1 (default): deferred frames run geometry, SSAO and blur on a
                                 second, high-priority stream while the shadow pass runs on
                                 the frame's stream; both join before lighting (the buffers
                                 are those of the sequential order). 0: every pass in order
                                 on the frame's stream                                   */
    int32_t blur_warmup;      /* FR_BLUR_REFERENCE runs each line's in-place recurrence in
                                 32-position chunks in parallel, each chunk started this
                                 many steps early and kept only where its entry state
                                 equals the previous chunk's results bit for bit (the
                                 others are recomputed in order). 0 = 64. Every value
                                 gives the same floats; small ones only repair more     */
    int32_t pass_timings;     /* 1 (default): fr_render_frame records an event at every pass
                                 boundary and fr_last_timings reports each pass; 0: only the
                                 frame's first and last events (fr_last_timings reports the
                                 total, the passes as 0), which spares the frame the
                                 boundary events' time (about 4 us at 1280x800)          */
} fr_config;

/* Fills cfg with the reference's defaults. */
void fr_config_defaults(fr_config* cfg);

typedef struct fr_ctx fr_ctx;

fr_ctx* fr_create(const fr_config* cfg, char* err, size_t errlen);
void fr_destroy(fr_ctx* ctx);
const char* fr_last_error(const fr_ctx* ctx);

/* Uploads meshes, indices, materials and textures (replaces the per-draw access
 * of Model/Mesh/Texture data, mesh.cpp:10-56, texture.h:41-132). */
int fr_upload_scene(fr_ctx* ctx, const fr_scene* scene);

/* Frame parameters. matrices NULL = compute them from the scene (the normal
 * path); non-NULL = use these exactly (lets tests feed matrices computed on
 * another machine). stream NULL = the context's own stream. */
typedef struct fr_frame_params
{
    const fr_frame_matrices* matrices; /* NULL = the scene's camera (fr_scene_frame_matrices) */
    void* stream;                      /* cudaStream_t; NULL = the context's stream          */
    const float* eye;                  /* camera position (3 floats) for the view vector of
                                          the lighting, with matrices of another camera
                                          (fr_scene_view_matrices); NULL = the scene's eye
                                          (scene.cpp:145-158)                                 */
} fr_frame_params;

/* One frame: Render::Render (render.cpp:40-58) = shadow pass, then forward pass
 * or geometry + lighting (with SSAO) passes, then SSAA. */
int fr_render_frame(fr_ctx* ctx, const fr_frame_params* params);

/* The passes one by one, in the order fr_render_frame runs them. */
int fr_shadow_pass(fr_ctx* ctx, const fr_frame_params* params);   /* render.cpp:60-97  */
int fr_forward_pass(fr_ctx* ctx, const fr_frame_params* params);  /* render.cpp:99-157 */
int fr_geometry_pass(fr_ctx* ctx, const fr_frame_params* params); /* render.cpp:159-193*/
int fr_ssao_pass(fr_ctx* ctx, const fr_frame_params* params);     /* render.cpp:214-289*/
int fr_lighting_pass(fr_ctx* ctx, const fr_frame_params* params); /* render.cpp:195-212,
                                                                     forkergl.cpp:326-380 */
int fr_ssaa_pass(fr_ctx* ctx, const fr_frame_params* params);     /* render.cpp:291-345*/

/* ---- read-back ----------------------------------------------------------------- */
enum fr_buffer_id
{
    FR_BUF_DEPTH = 0,       /* ForkerGL::DepthBuffer       float  W*H  (FLT_MAX = empty) */
    FR_BUF_SHADOW = 1,      /* ForkerGL::ShadowBuffer      float  Sw*Sh                   */
    FR_BUF_GB_NORMAL = 2,   /* NormalGBuffer               float3 W*H                     */
    FR_BUF_GB_POSITION = 3, /* WorldPosGBuffer             float3                          */
    FR_BUF_GB_LIGHTNDC = 4, /* LightSpaceNDCPosGBuffer     float3                          */
    FR_BUF_GB_ALBEDO = 5,   /* AlbedoGBuffer               float3                          */
    FR_BUF_GB_EMISSIVE = 6, /* EmissiveGBuffer             float3                          */
    FR_BUF_GB_PARAM = 7,    /* ParamGBuffer                float3                          */
    FR_BUF_GB_TYPE = 8,     /* ShadingTypeGBuffer          float                           */
    FR_BUF_AO = 9,          /* AmbientOcclusionGBuffer     float  (after blur)             */
    FR_BUF_FRAME_F32 = 10,  /* FrameBuffer                 float3 (needs keep_float_frame) */
    FR_BUF_FRAME_U8 = 11,   /* FrameBuffer.GenerateImage() RGB8 W*H*3 (buffer.cpp:113-126) */
    FR_BUF_SSAA_U8 = 12,    /* ForkerGL::AntiAliasedImage  RGB8 (W/k)*(H/k)*3              */
    FR_BUF_TRIANGLE_ID = 13 /* visible triangle per pixel  int32, -1 = none                */
};

/* Copies one buffer to host memory in the reference's layout (Buffer1f /
 * Buffer3f: index x + y * width, components contiguous). Returns the number of
 * bytes the buffer needs if dst is NULL, else FR_OK / an error. When the frame
 * reports an error (for example FR_ERR_BIN_OVERFLOW), the contents of dst are
 * unspecified. */
int64_t fr_download(fr_ctx* ctx, int32_t buffer_id, void* dst, size_t bytes);

/* The uploaded scene's per-vertex tangents as the device holds them (3 floats a
 * vertex, in fr_scene_view order). Model::generateTangents (model.cpp:430-476)
 * runs at fr_upload_scene on the device for every model with the generateTangent
 * flag that is not normalised; the values equal fr_scene_view.tangents bit for
 * bit. Returns the bytes needed if dst is NULL, else FR_OK / an error. */
int64_t fr_scene_tangents(fr_ctx* ctx, float* dst, size_t bytes);

/* Per-pass device times of the last fr_render_frame (CUDA events on the frame's
 * stream), in milliseconds: [shadow, geometry|forward, ssao, blur, lighting,
 * ssaa, total]. Synchronises on the frame. With concurrent_passes, deferred
 * frames run the shadow pass beside geometry, SSAO and blur: shadow and geometry
 * are then both timed from the frame's start, lighting from the join of the two
 * chains, and total is less than the sum of the parts. With pass_timings = 0
 * only total is measured; the passes read 0. */
int fr_last_timings(fr_ctx* ctx, float* ms, int32_t n);

/* Number of kernels the last fr_render_frame launched. */
int32_t fr_last_launch_count(const fr_ctx* ctx);

/* ---- allocation-free entry point -------------------------------------------- */
/* No counterpart in the reference: the reference runs on the CPU only.
 *
 * The separable ambient-occlusion blur (the FR_BLUR_SEPARABLE blur of
 * fr_ssao_pass) applied in place to a caller-owned device buffer `ao` of
 * width * height floats, on `stream` (a cudaStream_t; NULL = the default
 * stream). It allocates nothing: its intermediate plane is a fixed device
 * array inside the library, of FR_NOALLOC_BLUR_MAX_PIXELS floats (16 MiB),
 * which every GPU that loads the library holds until the process exits. For
 * callers that must not allocate device memory while they run.
 *
 * `ao` and `stream` must belong to the calling thread's current device
 * (cudaGetDevice): the scratch array used is that device's copy. The render
 * context calls (fr_render_frame and the others) make their context's device
 * current and leave it so; set the device again before this call if it
 * differs.
 *
 * Returns FR_OK, FR_ERR_INVALID (null buffer, non-positive size, or more than
 * FR_NOALLOC_BLUR_MAX_PIXELS pixels; checked before any CUDA call) or
 * FR_ERR_CUDA: the launches failed, or a launch error of earlier work was
 * already pending on this thread (then nothing is launched and that error is
 * left pending). The first call on a device looks up the array's device
 * address on that device (cudaGetSymbolAddress); make that first call before
 * any stream capture. All calls share the one array: calls that overlap on the
 * GPU (other streams, other threads) race and must be serialised by the
 * caller. */
#define FR_NOALLOC_BLUR_MAX_PIXELS (4 * 1024 * 1024)
int fr_blur_separable_noalloc(float* ao, int32_t width, int32_t height, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FORKERRENDERER_H */
