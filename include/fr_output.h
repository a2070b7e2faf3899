/* fr_output.h — the frame's TGA files, encoded on the GPU.
 *
 * Replaces the reference's output stage (src/main.cpp:45-54 calling the
 * Output module, src/output.cpp:12-86): each image is converted to bytes the
 * way Buffer1f::GenerateImage (src/buffer.cpp:20-32: value * 255, one gray byte)
 * or Buffer3f::GenerateImage (:113-126: each channel * 254.99f, stored B, G, R)
 * does, then written as TGAImage::WriteTgaFile (src/tgaimage.cpp:172-248) writes
 * it: an 18-byte header, the pixels (run-length packets of unloadRleData,
 * :250-300, or raw), two zero 4-byte area references and the 18-byte
 * "TRUEVISION-XFILE." footer. The bytes are identical to the reference's files.
 *
 * Float to byte: the reference converts float to std::uint8_t implicitly; its
 * x86-64 build truncates toward zero to a 32-bit integer (NaN and values outside
 * the int32 range give INT32_MIN) and keeps the low 8 bits. That meaning is
 * fixed here on every host, so e.g. the background of the depth buffer
 * (FLT_MAX * 255 = inf) writes 0 and a world position of 1.2 writes 49.
 */
#ifndef FR_OUTPUT_H
#define FR_OUTPUT_H

#include <stddef.h>
#include <stdint.h>

#include "forkerrenderer.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The reference's output files, in the order main.cpp writes them. */
enum fr_output_image
{
    FR_OUT_FRAMEBUFFER = 0,      /* framebuffer.tga                 FrameBuffer (always)          */
    FR_OUT_SSAA = 1,             /* framebuffer_SSAA.tga            AntiAliasedImage (SSAA on)    */
    FR_OUT_SHADOWMAP = 2,        /* shadowmap.tga                   ShadowBuffer (shadow on)      */
    FR_OUT_ZBUFFER = 3,          /* zbuffer.tga                     DepthBuffer (always)          */
    FR_OUT_GB_NORMAL = 4,        /* gbuffer_normal.tga              NormalGBuffer (deferred)      */
    FR_OUT_GB_WORLDPOS = 5,      /* gbuffer_worldpos.tga            WorldPosGBuffer (deferred)    */
    FR_OUT_GB_ALBEDO = 6,        /* gbuffer_albedo.tga              AlbedoGBuffer (deferred)      */
    FR_OUT_GB_PARAM = 7,         /* gbuffer_param.tga               ParamGBuffer (deferred)       */
    FR_OUT_GB_SHADING_TYPE = 8,  /* gbuffer_shading_type.tga        ShadingTypeGBuffer (deferred) */
    FR_OUT_GB_AO = 9,            /* gbuffer_ambient_occlusion.tga   AmbientOcclusionGBuffer (deferred) */
    FR_OUT_COUNT = 10
};

/* File name of an output image ("framebuffer.tga", ...), NULL for a bad id. */
const char* fr_output_name(int32_t image);

/* 1 if the reference writes this file for the context's last frame (the
 * buffer exists: output.cpp's GetWidth() != 0 tests), 0 if not, < 0 on error. */
int fr_output_present(fr_ctx* ctx, int32_t image);

/* Size of an output image of the last frame: returns 1 and fills width, height
 * and bytes per pixel if the reference writes it, 0 if not, < 0 on error. */
int fr_output_shape(fr_ctx* ctx, int32_t image, int32_t* width, int32_t* height, int32_t* bytespp);

/* Encodes one output image of the last frame (rle: 1 = the reference's default
 * run-length packets, 0 = raw). Returns the file's size in bytes, 0 if the
 * reference writes no such file for this frame, < 0 on error. The bytes are
 * copied to dst only when dst != NULL and cap >= the size (call with dst = NULL
 * to learn the size). Waits for the context's stream. */
int64_t fr_output_encode(fr_ctx* ctx, int32_t image, int32_t rle, void* dst, size_t cap);

/* Encodes every output image of the last frame into dst, one file after the
 * other in fr_output_image order. sizes[FR_OUT_COUNT] receives each file's
 * size (0 = not written). device_ms (optional) receives the device time of the
 * encoding kernels. Returns the total bytes, < 0 on error (cap too small:
 * FR_ERR_INVALID, with sizes filled in). */
int64_t fr_output_encode_all(fr_ctx* ctx, int32_t rle, void* dst, size_t cap, int64_t* sizes, float* device_ms);

/* Output::Output* of main.cpp:45-54: writes each file the reference would write
 * into directory `dir` (which must exist). Returns the number of files written
 * or < 0 on error. */
int fr_output_write(fr_ctx* ctx, const char* dir, int32_t rle);

/* ---- the encoder on device images -------------------------------------------- */

/* Upper bound of a file's size: 44 + width * height * (1 + bytespp). */
size_t fr_tga_max_bytes(int32_t width, int32_t height, int32_t bytespp);

/* Device scratch bytes fr_tga_encode_device needs for a width x height image. */
size_t fr_tga_scratch_bytes(int32_t width, int32_t height);

/* Encodes device pixels (bytespp 1, 3 or 4, TGA byte order: gray, or B, G, R[, A];
 * row y at byte offset y * width * bytespp) into the device buffer d_out (16-byte
 * aligned, at least fr_tga_max_bytes) on `stream` (a cudaStream_t, NULL = the legacy default
 * stream). vflip: 1 = the reference's default (header origin bottom-left, rows
 * as stored), 0 = top-left. The file's size is written to *d_size (device
 * memory). Stream-ordered; returns FR_OK or FR_ERR_INVALID / FR_ERR_CUDA. */
int fr_tga_encode_device(const void* d_pixels, int32_t width, int32_t height, int32_t bytespp, int32_t rle,
                         int32_t vflip, void* d_out, int64_t* d_size, void* d_scratch, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FR_OUTPUT_H */
