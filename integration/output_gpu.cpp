// Drop-in replacement of the reference renderer's src/output.cpp, used together
// with integration/render_gpu.cpp: the ten Output:: functions (src/output.h:8-21,
// called by src/main.cpp:45-54) encode their TGA files on the GPU from the
// frame's device buffers (include/fr_output.h) instead of converting the host
// ForkerGL:: buffers with GenerateImage() and WriteTgaFile(). The bytes are the
// reference writer's (RLE on, the same header, packets and footer,
// tgaimage.cpp:172-300), and a file is skipped exactly where the reference skips
// it (a buffer of width 0: SSAA off, shadow off, forward rendering).

#include <cstdint>
#include <cstdio>
#include <vector>

#include "fr_output.h"
#include "output.h"
#include "render_gpu.h"

namespace
{

void write(int32_t image)
{
    fr_ctx* ctx = RenderGpuContext();
    if (!ctx) return;  // no frame rendered
    const int64_t n = fr_output_encode(ctx, image, 1, nullptr, 0);  // the file's size, 0 = not written
    if (n <= 0)
    {
        if (n < 0) std::fprintf(stderr, "[output_gpu] %s: %s\n", fr_output_name(image), fr_last_error(ctx));
        return;
    }
    std::vector<uint8_t> bytes((size_t)n);
    if (fr_output_encode(ctx, image, 1, bytes.data(), bytes.size()) != n)
    {
        std::fprintf(stderr, "[output_gpu] %s: %s\n", fr_output_name(image), fr_last_error(ctx));
        return;
    }
    const std::string path = std::string("output/") + fr_output_name(image);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f)
    {
        std::fprintf(stderr, "[output_gpu] cannot write %s\n", path.c_str());
        return;
    }
    std::fwrite(bytes.data(), 1, bytes.size(), f);
    std::fclose(f);
}

}  // namespace

namespace Output
{
void OutputFrameBuffer() { write(FR_OUT_FRAMEBUFFER); }
void OutputSSAAImage() { write(FR_OUT_SSAA); }
void OutputShadowBuffer() { write(FR_OUT_SHADOWMAP); }
void OutputZBuffer() { write(FR_OUT_ZBUFFER); }
void OutputNormalGBuffer() { write(FR_OUT_GB_NORMAL); }
void OutputWorldPosGBuffer() { write(FR_OUT_GB_WORLDPOS); }
void OutputAlbedoGBuffer() { write(FR_OUT_GB_ALBEDO); }
void OutputParamGBuffer() { write(FR_OUT_GB_PARAM); }
void OutputShadingTypeGBuffer() { write(FR_OUT_GB_SHADING_TYPE); }
void OutputAmbientOcclusionGBuffer() { write(FR_OUT_GB_AO); }
}  // namespace Output
