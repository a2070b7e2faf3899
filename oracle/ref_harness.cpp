// Test-infrastructure driver around the reference renderer's own code.
//
// Loads a .scene with the reference loader (src/scene.cpp:19), renders one frame
// with the reference's passes and dumps every ForkerGL buffer as raw little-endian
// float32 / uint8 files, so tests can compare the GB300 path and the CPU
// restatement under oracle/ against the reference itself.
//
// Orchestration:
//   --shadow-size 0 (default): Render::Preconfigure + Render::Render, unmodified
//     (src/render.cpp:33-58): the shadow map is screen sized, as in the reference.
//   --shadow-size S > 0: the same pass sequence, but the shadow pass
//     (render.cpp:60-97) rasterises into an S x S shadow map with an S x S
//     viewport; every other pass is the reference's own function.
//
// --tga 1: afterwards the reference's own Output::Output* calls of main.cpp:45-54
//   (src/output.cpp:12-86) write their TGA files into <out dir>/output/; their
//   wall time is reported as tga_seconds.
//
// --wrap W: ForkerGL::TextureWrapMode(W) before the scene loads (textures take
//   the mode in force when they are created, model.cpp:425-426).
// --filter F: ForkerGL::TextureFilterMode(F) before the scene loads, likewise.
//
// Usage: ref_harness <scene file> <out dir> [--shadow-size S] [--pcf N]
//                    [--blocker N] [--repeat R] [--tga 0|1] [--wrap W] [--filter F]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <sys/stat.h>
#include <unistd.h>

#include "output.h"
#include "render.h"
#include "fr_sample_tables.h"

int fr_ref_pcf_samples = 64;      // shadow.h:20 default
int fr_ref_blocker_samples = 32;  // shadow.h:21 default

static std::vector<float> g_blocker_table, g_pcf_table, g_ssao_table;
static int g_blocker_i = 0, g_pcf_i = 0;
static const int kRefSsaoSamples = 32;  // render.cpp:219

// Deterministic replacement of RandomVectorInUnitDisk() (geometry.h:968) inside
// shadow.cpp: per shaded pixel the blocker search draws taps 0..NB-1 of its
// table, then PCF draws taps 0..NP-1 of its own table.
Vector3f fr_ref_disk_sample(const char* caller)
{
    if (std::strcmp(caller, "FindAverageBlockDepth") == 0)
    {
        int i = g_blocker_i++ % fr_ref_blocker_samples;
        if (i == 0) g_pcf_i = 0;
        return Vector3f(g_blocker_table[2 * i], g_blocker_table[2 * i + 1], 0.f);
    }
    int j = g_pcf_i++ % fr_ref_pcf_samples;
    return Vector3f(g_pcf_table[2 * j], g_pcf_table[2 * j + 1], 0.f);
}

// Deterministic replacement of RandomVectorInHemisphere(normal) (geometry.h:978)
// inside Render::DoSSAO: the tap comes from the pixel's 4x4-noise-cell kernel and
// is flipped into the normal's hemisphere with the reference's own test.
Vector3f fr_ref_hemisphere_sample(const Vector3f& normal, int x, int y, int s)
{
    int cell = (y & 3) * 4 + (x & 3);
    const float* p = &g_ssao_table[3 * (cell * kRefSsaoSamples + s)];
    Vector3f v(p[0], p[1], p[2]);
    if (Dot(v, normal) > 0.f) return v;
    return -v;
}

static void dump(const std::string& path, const void* data, size_t bytes)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f)
    {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fwrite(data, 1, bytes, f);
    std::fclose(f);
}

static void dump1f(const std::string& path, const Buffer1f& b)
{
    int w = b.GetWidth(), h = b.GetHeight();
    std::vector<float> v((size_t)w * h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) v[(size_t)y * w + x] = b.GetValue(x, y);
    dump(path, v.data(), v.size() * 4);
}

static void dump3f(const std::string& path, const Buffer3f& b)
{
    int w = b.GetWidth(), h = b.GetHeight();
    std::vector<float> v((size_t)w * h * 3);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            Vector3f c = b.GetValue(x, y);
            size_t i = ((size_t)y * w + x) * 3;
            v[i] = c.x;
            v[i + 1] = c.y;
            v[i + 2] = c.z;
        }
    dump(path, v.data(), v.size() * 4);
}

static void dumpImageRGB(const std::string& path, const TGAImage& img)
{
    int w = img.GetWidth(), h = img.GetHeight();
    std::vector<unsigned char> v((size_t)w * h * 3);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            TGAColor c = img.Get(x, y);
            size_t i = ((size_t)y * w + x) * 3;
            v[i] = c.r;
            v[i + 1] = c.g;
            v[i + 2] = c.b;
        }
    dump(path, v.data(), v.size());
}

static void printMatrix(FILE* f, const char* name, const Matrix4x4f& m)
{
    std::fprintf(f, "%s", name);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) std::fprintf(f, " %a", (double)m[r][c]);
    std::fprintf(f, "\n");
}

// Shadow pass of render.cpp:60-97 with an S x S shadow map and viewport.
static void shadowPassSized(const Scene& scene, int S)
{
    if (!Shadow::GetShadowStatus()) return;
    ForkerGL::InitShadowBuffer(S, S);
    ForkerGL::InitDepthBuffer(S, S);
    ForkerGL::SetPassType(ForkerGL::ShadowPass);
    ForkerGL::SetViewportMatrix(0, 0, S, S);
    Matrix4x4f view = MakeLookAtMatrix(scene.GetPointLight().position, Vector3f(0.f));
    Matrix4x4f proj = MakeOrthographicMatrix(-3.0f * scene.GetRatio(), 3.0f * scene.GetRatio(),
                                             -3.0f, 3.0f, 0.1f, 20.f);
    ForkerGL::SetLightSpaceMatrix(proj * view);
    for (unsigned i = 0; i < scene.GetModelCount(); ++i)
    {
        DepthShader depthShader;
        depthShader.uModelMatrix = scene.GetModelMatrix(i);
        depthShader.uLightSpaceMatrix = ForkerGL::GetLightSpaceMatrix();
        scene.GetModel(i).Render(depthShader);
    }
}

int main(int argc, char** argv)
{
    if (argc < 3)
    {
        std::fprintf(stderr,
                     "usage: %s <scene> <outdir> [--shadow-size S] [--pcf N] [--blocker N] "
                     "[--repeat R] [--tga 0|1] [--wrap W] [--filter F]\n",
                     argv[0]);
        return 1;
    }
    std::string scenePath = argv[1];
    std::string outDir = argv[2];
    int shadowSize = 0, repeat = 1, writeTga = 0, wrap = 0, filter = 0;
    for (int i = 3; i + 1 < argc; i += 2)
    {
        std::string k = argv[i];
        int v = std::atoi(argv[i + 1]);
        if (k == "--shadow-size") shadowSize = v;
        else if (k == "--pcf") fr_ref_pcf_samples = v;
        else if (k == "--blocker") fr_ref_blocker_samples = v;
        else if (k == "--repeat") repeat = v;
        else if (k == "--tga") writeTga = v;
        else if (k == "--wrap") wrap = v;
        else if (k == "--filter") filter = v;
        else
        {
            std::fprintf(stderr, "unknown option %s\n", k.c_str());
            return 1;
        }
    }
    if (outDir[0] != '/')
    {
        char cwd[4096];
        if (!getcwd(cwd, sizeof cwd)) return 2;
        outDir = std::string(cwd) + "/" + outDir;
    }

    g_blocker_table.resize(2 * fr_ref_blocker_samples);
    g_pcf_table.resize(2 * fr_ref_pcf_samples);
    g_ssao_table.resize(3 * 16 * kRefSsaoSamples);
    fr_make_disk_table(FR_TABLE_SEED_BLOCKER, fr_ref_blocker_samples, g_blocker_table.data());
    fr_make_disk_table(FR_TABLE_SEED_PCF, fr_ref_pcf_samples, g_pcf_table.data());
    fr_make_ssao_table(kRefSsaoSamples, g_ssao_table.data());

    // The reference resolves model paths against the working directory.
    std::string dir = ".", file = scenePath;
    size_t slash = scenePath.find_last_of('/');
    if (slash != std::string::npos)
    {
        dir = scenePath.substr(0, slash);
        file = scenePath.substr(slash + 1);
    }
    if (chdir(dir.c_str()) != 0)
    {
        std::fprintf(stderr, "cannot chdir to %s\n", dir.c_str());
        return 2;
    }

    ForkerGL::TextureWrapMode(static_cast<Texture::WrapMode>(wrap));
    ForkerGL::TextureFilterMode(static_cast<Texture::FilterMode>(filter));
    const auto tl = std::chrono::steady_clock::now();
    Scene scene(file);
    const double loadSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - tl).count();
    Render::Preconfigure(scene);
    int W = scene.IsSSAAOn() ? scene.GetWidth() * scene.GetSSAAKernelSize() : scene.GetWidth();
    int H = scene.IsSSAAOn() ? scene.GetHeight() * scene.GetSSAAKernelSize() : scene.GetHeight();

    double best = 1e30;
    for (int r = 0; r < repeat; ++r)
    {
        g_blocker_i = g_pcf_i = 0;
        auto t0 = std::chrono::steady_clock::now();
        if (shadowSize <= 0)
        {
            Render::Render(scene);
        }
        else
        {
            shadowPassSized(scene, shadowSize);
            ForkerGL::SetViewportMatrix(0, 0, W, H);
            if (ForkerGL::GetRenderMode() == ForkerGL::Forward)
                Render::DoForwardPass(scene);
            else
            {
                Render::DoGeometryPass(scene);
                Render::DoLightingPass(scene);
            }
            Render::DoSSAA(scene);
        }
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (dt < best) best = dt;
    }

    dump1f(outDir + "/depth.f32", ForkerGL::DepthBuffer);
    if (ForkerGL::ShadowBuffer.GetWidth() != 0) dump1f(outDir + "/shadow.f32", ForkerGL::ShadowBuffer);
    dump3f(outDir + "/frame.f32", ForkerGL::FrameBuffer);
    dumpImageRGB(outDir + "/frame8.u8", ForkerGL::FrameBuffer.GenerateImage());
    if (ForkerGL::AntiAliasedImage.GetWidth() != 0)
        dumpImageRGB(outDir + "/ssaa.u8", ForkerGL::AntiAliasedImage);
    if (ForkerGL::GetRenderMode() == ForkerGL::Deferred)
    {
        dump3f(outDir + "/gb_normal.f32", ForkerGL::NormalGBuffer);
        dump3f(outDir + "/gb_pos.f32", ForkerGL::WorldPosGBuffer);
        if (Shadow::GetShadowStatus()) dump3f(outDir + "/gb_lndc.f32", ForkerGL::LightSpaceNDCPosGBuffer);
        dump3f(outDir + "/gb_albedo.f32", ForkerGL::AlbedoGBuffer);
        dump3f(outDir + "/gb_emissive.f32", ForkerGL::EmissiveGBuffer);
        dump3f(outDir + "/gb_param.f32", ForkerGL::ParamGBuffer);
        dump1f(outDir + "/gb_type.f32", ForkerGL::ShadingTypeGBuffer);
        dump1f(outDir + "/gb_ao.f32", ForkerGL::AmbientOcclusionGBuffer);
    }

    FILE* f = std::fopen((outDir + "/info.txt").c_str(), "w");
    std::fprintf(f, "width %d\nheight %d\n", W, H);
    std::fprintf(f, "deferred %d\n", ForkerGL::GetRenderMode() == ForkerGL::Deferred ? 1 : 0);
    std::fprintf(f, "shadow %d\n", Shadow::GetShadowStatus() ? 1 : 0);
    std::fprintf(f, "shadow_width %d\nshadow_height %d\n", ForkerGL::ShadowBuffer.GetWidth(),
                 ForkerGL::ShadowBuffer.GetHeight());
    std::fprintf(f, "seconds %.9f\n", best);
    std::fprintf(f, "load_seconds %.9f\n", loadSeconds);
    printMatrix(f, "viewproj", ForkerGL::GetViewProjectionMatrix());
    printMatrix(f, "lightspace", ForkerGL::GetLightSpaceMatrix());
    printMatrix(f, "viewport", ForkerGL::GetViewportMatrix());
    for (unsigned i = 0; i < scene.GetModelCount(); ++i)
    {
        char name[64];
        std::snprintf(name, sizeof name, "model%u", i);
        printMatrix(f, name, scene.GetModelMatrix(i));
    }
    if (writeTga)
    {
        if (chdir(outDir.c_str()) != 0) return 2;
        mkdir("output", 0755);
        auto t0 = std::chrono::steady_clock::now();
        Output::OutputFrameBuffer();
        Output::OutputSSAAImage();
        Output::OutputShadowBuffer();
        Output::OutputZBuffer();
        Output::OutputNormalGBuffer();
        Output::OutputWorldPosGBuffer();
        Output::OutputAlbedoGBuffer();
        Output::OutputParamGBuffer();
        Output::OutputShadingTypeGBuffer();
        Output::OutputAmbientOcclusionGBuffer();
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(f, "tga_seconds %.9f\n", dt);
    }
    std::fclose(f);
    return 0;
}
