// Device-side data layout and the per-fragment / per-pixel functions of the
// frame, written in the reference's evaluation order so that, compiled with
// --fmad=false and IEEE division / square root (nvcc defaults), every float
// result matches the reference except where a libm function (powf) is called.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fr_exact.cuh"

namespace frd
{

// ---- device scene ---------------------------------------------------------------
struct DevMaterial
{
    float ka[3], kd[3], ks[3], ke[3], pbr_albedo[3];
    float roughness, metalness;
    int map_kd, map_ks, map_ke, map_bump, map_ao, map_pr, map_pm;
    int pad;
};

struct DevTexture
{
    int w, h, bpp, pad;     // bpp 1: one byte per texel; 3/4: packed r|g<<8|b<<16
    float wf, hf;           // (float)(w - 0.001), (float)(h - 0.001)  (texture.h:377)
    unsigned long long off; // byte offset into the texel pool
};

struct DevModel
{
    float M[16], LM[16];
    float N3[9];
    int has_tangents, support_pbr;
    int pad;
};

struct DevScene
{
    int numTris, numVerts, numNormals, numModels;
    int texWrap;        // Texture::WrapMode of every texture (0 NoWrap, 1 Repeat, 2 Mirrored, 3 Clamp)
    int texLinear;      // Texture::FilterMode of every texture: 0 Nearest, 1 Linear (bilinear)
    const float4* pos;  // [V] model-space position
    const float4* tan;  // [V] generated tangent (as loaded)
    const float4* nrm;  // [N] normal (as loaded)
    const float2* uv;   // [Nt]
    const int4* triV;   // [T] (v0, v1, v2, mesh)
    const int4* triT;   // [T] (t0, t1, t2, material)
    const int4* triN;   // [T] (n0, n1, n2, model)
    const int* vmodel;  // [V] model of each vertex
    const int* nmodel;  // [N] model of each normal
    const DevModel* models;
    const DevMaterial* materials;
    const DevTexture* textures;
    const unsigned char* texels;
    const float* gamma8;  // [256] powf(b / 255.f, 2.2f) for every byte b, computed on the device
};

// Per-frame uniforms.
struct FrameConst
{
    float V[16], P[16], VP[16], L[16], VPort[16], SVPort[16];
    float eye[3], lightPos[3], lightColor[3];
    int W, H, SW, SH;
    int shadowOn, deferred, ssaoOn, shadowMode;
    int pcfN, blockerN, ssaoN;
    int vportSimple;  // viewport matrix has the SetViewportMatrix zero pattern
    float ssaoRadius, ssaoBias, ssaoRange;
    int bgBlack;  // light position / colour and eye finite: a zero G-buffer shades to black
};

// Per-vertex outputs of the camera transform (gshader.h:41-92).
struct VertexOut
{
    int4* scr;     // (sx, sy, depth bits, 0)
    float4* pw;    // (posWS * ow, ow)
    float4* lw;    // (lightNDC * ow, 0)
    float4* tw;    // (tangentWS * ow, 0)
    float4* npre;  // [N] normal matrix * Normalize(n)
};

// Packed G-buffer (three 16-byte planes per pixel; see gbuffer flags below).
struct GBuffer
{
    float4* a;      // (pos.x, pos.y, pos.z, lightNDC.x)
    float4* b;      // (normal.x, normal.y, normal.z, lightNDC.y)
    uint4* c;       // Nearest: (bits(lightNDC.z), albedo rgb | flags << 24, params | mat lo, emissive | mat hi)
                    // Linear:  (bits(lightNDC.z), material | flags << 24, bits(u), bits(v)): the
                    //          maps are sampled where the G-buffer is decoded
    float* depth;   // DepthBuffer
    float* ao;      // AmbientOcclusionGBuffer
};

enum GFlags : unsigned
{
    kGCovered = 1u,
    kGPbr = 2u,
    kGAlbedoMap = 4u,
    kGEmissiveMap = 8u,
    kGP0Map = 16u,
    kGP1Map = 32u,
    kGP2Map = 64u
};

// ---- small float vector ops in the reference order ----------------------------------
struct F3
{
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float a) { return F3{a, a, a}; }
__device__ __forceinline__ F3 f3(float a, float b, float c) { return F3{a, b, c}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, F3 b) { return F3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float f) { return F3{a.x * f, a.y * f, a.z * f}; }
__device__ __forceinline__ F3 operator-(F3 a) { return F3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ F3 divs(F3 a, float f)
{
    float inv = 1.f / f;
    return F3{a.x * inv, a.y * inv, a.z * inv};
}
__device__ __forceinline__ F3 divv(F3 a, F3 b) { return F3{a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ float dot(F3 a, F3 b)
{
    float r = 0.f;
    r += a.x * b.x;
    r += a.y * b.y;
    r += a.z * b.z;
    return r;
}
__device__ __forceinline__ float length(F3 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ F3 normalize(F3 v) { return divs(v, length(v)); }
__device__ __forceinline__ F3 cross(F3 a, F3 b)
{
    return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// std::max / std::min semantics (NaN handling included)
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float clamp01(float v) { return smin(1.f, smax(v, 0.f)); }
__device__ __forceinline__ F3 clamp01(F3 v) { return F3{clamp01(v.x), clamp01(v.y), clamp01(v.z)}; }
__device__ __forceinline__ F3 powv(F3 v, float p) { return F3{powf(v.x, p), powf(v.y, p), powf(v.z, p)}; }

struct F4
{
    float x, y, z, w;
};
// Matrix4 * Vector4, rows as Dot from 0.f (geometry.h:774-782).
__device__ __forceinline__ F4 mul4(const float* m, F4 v)
{
    F4 o;
    float* po = &o.x;
    const float in[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int r = 0; r < 4; ++r)
    {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) s += m[r * 4 + k] * in[k];
        po[r] = s;
    }
    return o;
}
__device__ __forceinline__ F3 mul3(const float* m, F3 v)
{
    F3 o;
    float* po = &o.x;
    const float in[3] = {v.x, v.y, v.z};
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) s += m[r * 3 + k] * in[k];
        po[r] = s;
    }
    return o;
}
__device__ __forceinline__ F4 scale4(F4 v, float f) { return F4{v.x * f, v.y * f, v.z * f, v.w * f}; }
__device__ __forceinline__ F4 div4(F4 v, float f)
{
    float inv = 1.f / f;
    return F4{v.x * inv, v.y * inv, v.z * inv, v.w * inv};
}
__device__ __forceinline__ float interp(float a, float b, float c, float b0, float b1, float b2)
{
    float r = 0.f;
    r += a * b0;
    r += b * b1;
    r += c * b2;
    return r;
}

// ---- textures (texture.h:41-132, NoWrap + Nearest; tgaimage.cpp:304-311) --------------
// Texture::wrapCoord (texture.h:62-83) of one coordinate.
__device__ __forceinline__ float wrap_coord(int mode, float c)
{
    if (mode == 1) return c - floorf(c);
    if (mode == 2)
    {
        const int i = frx::f2i_sat(floorf(c));  // int xi = std::floor(coord.x)
        const float rep = c - (float)i;
        return i % 2 == 0 ? rep : 1.f - rep;
    }
    if (mode == 3)
    {
        const float m = c < 0.f ? 0.f : c;  // std::min(1, std::max(c, 0)): NaN -> 1
        return m < 1.f ? m : 1.f;
    }
    return c;
}

__device__ __forceinline__ bool texel_rgb(const DevScene& S, int tex, float u, float v, unsigned& r,
                                          unsigned& g, unsigned& b)
{
    const DevTexture t = S.textures[tex];
    if (S.texWrap) u = wrap_coord(S.texWrap, u), v = wrap_coord(S.texWrap, v);
    float fu = floorf(u * t.wf), fv = floorf(v * t.hf);
    r = g = b = 0;
    if (!(fu == fu) || !(fv == fv)) return false;
    int x = frx::f2i_sat(fu), y = frx::f2i_sat(fv);
    if (x < 0 || y < 0 || x >= t.w || y >= t.h) return false;
    size_t idx = (size_t)x + (size_t)y * t.w;
    if (t.bpp == 1)
    {
        b = __ldg(S.texels + t.off + idx);
    }
    else
    {
        unsigned p = __ldg(reinterpret_cast<const unsigned*>(S.texels + t.off) + idx);
        r = p & 0xffu, g = (p >> 8) & 0xffu, b = (p >> 16) & 0xffu;
    }
    return true;
}

// Texture::getColorFromImage (texture.h:130-134) of image texel (x, y): black outside
// the image (TGAImage::Get, tgaimage.cpp:304-311).
__device__ __forceinline__ F3 image_color(const DevScene& S, const DevTexture& t, int x, int y)
{
    if (x < 0 || y < 0 || x >= t.w || y >= t.h) return f3(0.f);
    size_t idx = (size_t)x + (size_t)y * t.w;
    if (t.bpp == 1) return F3{0.f, 0.f, (float)__ldg(S.texels + t.off + idx)};
    unsigned p = __ldg(reinterpret_cast<const unsigned*>(S.texels + t.off) + idx);
    return F3{(float)(p & 0xffu), (float)((p >> 8) & 0xffu), (float)((p >> 16) & 0xffu)};
}

// Lerp (geometry.h:913-916): (1 - t) * a + t * b, component by component.
__device__ __forceinline__ F3 lerp3(float t, F3 a, F3 b)
{
    const float s = 1.f - t;
    return F3{a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t};
}

// Texture::colorFromFiltering (texture.h:85-127) after wrapCoord: the color in [0, 255].
// Linear: the four texels around p = (u * (w - 0.001), v * (h - 0.001)) with texel
// centres at +0.5, clamped to the image unless the wrap mode is NoWrap.
__device__ __forceinline__ F3 texel_color(const DevScene& S, int tex, float u, float v)
{
    if (!S.texLinear)
    {
        unsigned r, g, b;
        texel_rgb(S, tex, u, v, r, g, b);
        return F3{(float)r, (float)g, (float)b};
    }
    const DevTexture t = S.textures[tex];
    if (S.texWrap) u = wrap_coord(S.texWrap, u), v = wrap_coord(S.texWrap, v);
    const float px = u * t.wf, py = v * t.hf;
    const float lx = floorf(px - 0.5f), ly = floorf(py - 0.5f);
    const float tx = px - (lx + 0.5f), ty = py - (ly + 0.5f);
    int x0 = frx::f2i_sat(lx), y0 = frx::f2i_sat(ly);
    int x1 = frx::f2i_sat(lx + 1.f), y1 = frx::f2i_sat(ly + 1.f);
    if (S.texWrap)
    {
        x0 = min(t.w - 1, max(x0, 0)), x1 = min(t.w - 1, max(x1, 0));
        y0 = min(t.h - 1, max(y0, 0)), y1 = min(t.h - 1, max(y1, 0));
    }
    const F3 c0 = image_color(S, t, x0, y0), c1 = image_color(S, t, x1, y0);
    const F3 c2 = image_color(S, t, x0, y1), c3 = image_color(S, t, x1, y1);
    return lerp3(ty, lerp3(tx, c0, c1), lerp3(tx, c2, c3));
}

__device__ __forceinline__ F3 rgb_to_f3(unsigned r, unsigned g, unsigned b)
{
    return divs(F3{(float)r, (float)g, (float)b}, 255.f);  // Texture::Sample
}
__device__ __forceinline__ float byte_to_float(unsigned v) { return (float)v / 255.f; }  // SampleFloat

// Texture::Sample (texture.h:41-45) and Texture::SampleFloat (:47-51).
__device__ __forceinline__ F3 tex_sample(const DevScene& S, int tex, float u, float v)
{
    return divs(texel_color(S, tex, u, v), 255.f);
}
__device__ __forceinline__ float tex_sample_float(const DevScene& S, int tex, float u, float v)
{
    return texel_color(S, tex, u, v).z / 255.f;
}

// Material values of a packed G-buffer pixel, as the float G-buffers hold them.
struct GDecoded
{
    F3 albedo, emissive, param;
    float type;
    F3 albedoLin, emissiveLin;  // pow(albedo, 2.2), pow(emissive, 2.2): the shaders' sRGB -> linear
};

// pow(c, 2.2) of a texel channel u8 / 255 (phongshader.h:177, pbrshader.h:188): a
// lookup in the per-byte table that holds the same powf results.
__device__ __forceinline__ F3 gamma8_rgb(const DevScene& S, unsigned r, unsigned g, unsigned b)
{
    return F3{__ldg(S.gamma8 + r), __ldg(S.gamma8 + g), __ldg(S.gamma8 + b)};
}

// decode_gbuffer of a bilinear-filtered frame: the G-buffer holds the texture
// coordinate, so the maps are sampled here.
__device__ __forceinline__ GDecoded decode_gbuffer_linear(const DevScene& S, uint4 c, unsigned flags)
{
    GDecoded g;
    const bool isPbr = flags & kGPbr;
    const DevMaterial& mat = S.materials[c.y & 0xffffffu];
    const float u = __uint_as_float(c.z), v = __uint_as_float(c.w);
    g.albedo = (flags & kGAlbedoMap) ? tex_sample(S, mat.map_kd, u, v)
               : isPbr               ? F3{mat.pbr_albedo[0], mat.pbr_albedo[1], mat.pbr_albedo[2]}
                                     : F3{mat.kd[0], mat.kd[1], mat.kd[2]};
    g.emissive = (flags & kGEmissiveMap) ? tex_sample(S, mat.map_ke, u, v) : F3{mat.ke[0], mat.ke[1], mat.ke[2]};
    if (isPbr)
    {
        g.param.x = (flags & kGP0Map) ? tex_sample_float(S, mat.map_ao, u, v) : 1.f;
        g.param.y = (flags & kGP1Map) ? tex_sample_float(S, mat.map_pm, u, v) : mat.metalness;
        g.param.z = (flags & kGP2Map) ? tex_sample_float(S, mat.map_pr, u, v) : mat.roughness;
        g.type = 1.f;
    }
    else
    {
        g.param.x = 1.f;
        g.param.y = mat.ks[0];
        g.param.z = (flags & kGP2Map) ? tex_sample_float(S, mat.map_ks, u, v) + 5 : 1.f;
        g.type = 0.f;
    }
    g.albedoLin = powv(g.albedo, 2.2f);
    g.emissiveLin = powv(g.emissive, 2.2f);
    return g;
}

// kLinear: the frame's filter mode as a compile-time constant, so the lighting
// kernels instantiated for nearest filtering carry none of the sampling code.
template <bool kLinear>
__device__ __forceinline__ GDecoded decode_gbuffer_t(const DevScene& S, uint4 c)
{
    GDecoded g;
    unsigned flags = c.y >> 24;
    if (!(flags & kGCovered))
    {
        g.albedo = g.emissive = g.param = f3(0.f);
        g.albedoLin = g.emissiveLin = f3(0.f);  // powf(0, 2.2) = 0
        g.type = 0.f;
        return g;
    }
    const bool isPbr = flags & kGPbr;
    if (kLinear) return decode_gbuffer_linear(S, c, flags);
    unsigned m = (c.z >> 24) | ((c.w >> 24) << 8);
    const DevMaterial& mat = S.materials[m];
    if (flags & kGAlbedoMap)
    {
        const unsigned r = c.y & 0xffu, gg = (c.y >> 8) & 0xffu, b = (c.y >> 16) & 0xffu;
        g.albedo = rgb_to_f3(r, gg, b);
        g.albedoLin = gamma8_rgb(S, r, gg, b);
    }
    else
    {
        g.albedo = isPbr ? F3{mat.pbr_albedo[0], mat.pbr_albedo[1], mat.pbr_albedo[2]} : F3{mat.kd[0], mat.kd[1], mat.kd[2]};
        g.albedoLin = powv(g.albedo, 2.2f);
    }
    if (flags & kGEmissiveMap)
    {
        const unsigned r = c.w & 0xffu, gg = (c.w >> 8) & 0xffu, b = (c.w >> 16) & 0xffu;
        g.emissive = rgb_to_f3(r, gg, b);
        g.emissiveLin = gamma8_rgb(S, r, gg, b);
    }
    else
    {
        g.emissive = F3{mat.ke[0], mat.ke[1], mat.ke[2]};
        g.emissiveLin = powv(g.emissive, 2.2f);
    }
    unsigned p0 = c.z & 0xffu, p1 = (c.z >> 8) & 0xffu, p2 = (c.z >> 16) & 0xffu;
    if (isPbr)
    {
        g.param.x = (flags & kGP0Map) ? byte_to_float(p0) : 1.f;
        g.param.y = (flags & kGP1Map) ? byte_to_float(p1) : mat.metalness;
        g.param.z = (flags & kGP2Map) ? byte_to_float(p2) : mat.roughness;
        g.type = 1.f;
    }
    else
    {
        g.param.x = 1.f;
        g.param.y = mat.ks[0];
        g.param.z = (flags & kGP2Map) ? byte_to_float(p2) + 5 : 1.f;
        g.type = 0.f;
    }
    return g;
}

__device__ __forceinline__ GDecoded decode_gbuffer(const DevScene& S, uint4 c)
{
    return S.texLinear ? decode_gbuffer_t<true>(S, c) : decode_gbuffer_t<false>(S, c);
}

// ---- shadows (shadow.cpp:23-132) ------------------------------------------------------------
__constant__ float c_blocker[2 * 256];  // disk taps pre-scaled: (float)((double)d * 0.005)
__constant__ float c_pcf[2 * 256];

// Outside [0, 1]^2, and for NaN coordinates (every comparison with NaN is
// false), the reference's lookup returns +inf. Inside, ui <= w - 1 and vi <= h - 1,
// so the texel index fits 32 bits (a shadow map holds at most 2^30 texels).
__device__ __forceinline__ float sample_shadow(const float* __restrict__ sm, int w, int h, float u, float v)
{
    if (!(u >= 0.f && u <= 1.f && v >= 0.f && v <= 1.f)) return __int_as_float(0x7f800000);
    int wi = (int)((float)w - 0.001f);
    int hi = (int)((float)h - 0.001f);
    int ui = (int)((float)wi * u);
    int vi = (int)((float)hi * v);
    float d = __ldg(sm + (ui + vi * w));
    return d < 0.001f ? 1.f : d;  // same as the reference's float < 0.001 (double) test
}

__device__ __forceinline__ float pcf(const FrameConst& F, const float* sm, F3 c, float bias, float filter)
{
    float vis = 0.f;
    float invN = 1.f / (float)F.pcfN;
    for (int i = 0; i < F.pcfN; ++i)
    {
        float s = sample_shadow(sm, F.SW, F.SH, c.x + c_pcf[2 * i] * filter, c.y + c_pcf[2 * i + 1] * filter);
        if (c.z <= s + bias) vis += invN;
    }
    return vis;
}

__device__ __forceinline__ float blocker_depth(const FrameConst& F, const float* sm, F3 c, float bias)
{
    float sum = 0.f, num = 0.f;
    for (int i = 0; i < F.blockerN; ++i)
    {
        float s = sample_shadow(sm, F.SW, F.SH, c.x + c_blocker[2 * i], c.y + c_blocker[2 * i + 1]);
        if (c.z > s + bias)
        {
            sum += s;
            num += 1.f;
        }
    }
    if (num < 1.f) return 0.f;
    return sum / num;
}

__device__ __forceinline__ float shadow_visibility(const FrameConst& F, const float* sm, F3 lndc, F3 n, F3 L)
{
    F3 c = lndc * 0.5f + f3(0.5f);
    float bias = smax(0.009f * (1.f - dot(n, L)), 0.007f);
    if (F.shadowMode == 1) return pcf(F, sm, c, bias, 0.007f);
    if (F.shadowMode == 2)
    {
        float dR = c.z;
        float dB = blocker_depth(F, sm, c, bias);
        if (dB < 0.001f) return 1.f;  // float < 0.001f == float < 0.001 (double)
        float pen = (dR - dB) * 2.5f / dB;
        // (float)(PCF_FILTER_SIZE * (double)pen), PCF_FILTER_SIZE = 0.007 = 0x1cac083126e979 * 2^-60
        float filter = frx::mul_f_d_round(pen, 0.007, 0x1cac083126e979ull, -60);
        return pcf(F, sm, c, bias, filter);
    }
    float d = sample_shadow(sm, F.SW, F.SH, c.x, c.y);
    return (c.z <= d + bias) ? 1.f : 0.f;
}

// ---- lighting models (phongshader.h:171-215, pbrshader.h:182-288) ---------------------
// dl, el: diffuse colour and emission already in linear space (pow(c, 2.2)).
__device__ __forceinline__ F3 blinn_phong_lin(bool shadowOn, F3 L, F3 Hd, F3 N, float vis, F3 dl, F3 el, F3 param,
                                              F3 lightColor)
{
    const float kInvGamma = 1.f / 2.2f;
    float ao = param.x, ks = param.y, shin = param.z;
    float diff = smax(0.f, dot(L, N));
    float spec = powf(smax(0.f, dot(Hd, N)), shin);
    F3 ambient = f3(0.3f) * dl * ao;
    F3 diffuse = dl * diff * ao;
    F3 specular = f3(ks) * spec;
    if (shadowOn)
    {
        float shadow = (1 - vis) * 0.6f;
        vis = 1 - shadow;
        diffuse = diffuse * vis;
        specular = specular * vis;
    }
    F3 color = ambient + (diffuse + specular + el) * lightColor;
    color = divv(color, color + f3(1.f));
    color = powv(color, kInvGamma);
    return clamp01(color);
}

__device__ __forceinline__ F3 blinn_phong(bool shadowOn, F3 L, F3 Hd, F3 N, float vis, F3 diffuseColor,
                                          F3 emissive, F3 param, F3 lightColor)
{
    const float kGamma = 2.2f;
    return blinn_phong_lin(shadowOn, L, Hd, N, vis, powv(diffuseColor, kGamma), powv(emissive, kGamma), param,
                           lightColor);
}

__device__ __forceinline__ float ggx(float NdotH, float r)
{
    const float kInvPi = 0.31830988618379067154f;
    float a = r * r;
    float a2 = a * a;
    float n2 = NdotH * NdotH;
    float d = (n2 * (a2 - 1.f) + 1.f);
    float d2 = d * d;
    return a2 * kInvPi / d2;
}
__device__ __forceinline__ float schlick_ggx(float NdotV, float r)
{
    float a = r + 1.f;
    float k = a * a / 8.f;
    return NdotV / (NdotV * (1 - k) + k);
}

// Direct term of one light (pbrshader.h:194-232): Lo = (kd albedo / pi + specular)
// radiance (N.L), with the shadow's visibility applied as the reference does.
// al: albedo already in linear space (albedo^2.2).
__device__ __forceinline__ F3 pbr_direct(bool shadowOn, F3 L, F3 Vd, F3 Hd, F3 N, float vis, F3 al, float metal,
                                         float rough, F3 radiance)
{
    const float kInvPi = 0.31830988618379067154f;
    float NdotV = smax(dot(N, Vd), 0.f);
    float NdotL = smax(dot(N, L), 0.f);
    float NdotH = smax(dot(N, Hd), 0.f);
    float HdotV = smax(dot(Hd, Vd), 0.f);
    F3 F0 = f3(0.04f);
    F0 = F0 * (1 - metal) + al * metal;
    float NDF = ggx(NdotH, rough);
    float G = schlick_ggx(NdotV, rough) * schlick_ggx(NdotL, rough);
    float om = smax(1.f - HdotV, 0.f);
    F3 Fr = F0 + (f3(1.f) - F0) * powf(om, 5.f);
    F3 DGF = Fr * (NDF * G);
    float denom = 4 * NdotV * NdotL + 0.001f;
    F3 specular = divs(DGF, denom);
    F3 kd = f3(1.f) - Fr;
    kd = kd * (1.f - metal);
    F3 brdf = kd * al * kInvPi + specular;
    F3 Lo = brdf * radiance * NdotL;
    if (shadowOn)
    {
        float shadow = (1 - vis) * 0.6f;
        vis = 1 - shadow;
        Lo = Lo * vis;
    }
    return Lo;
}

// Ambient, emission, Reinhard and gamma (pbrshader.h:234-253) on the summed direct light.
__device__ __forceinline__ F3 pbr_finish(F3 Lo, F3 al, F3 el, float ao)
{
    const float kInvGamma = 1.f / 2.2f;
    F3 color = Lo;
    F3 ambient = f3(0.3f) * al * ao;
    color = color + ambient;
    color = color + el;
    color = divv(color, color + f3(1.f));
    color = powv(color, kInvGamma);
    return clamp01(color);
}

// al, el: albedo and emission already in linear space (pow(c, 2.2)).
__device__ __forceinline__ F3 pbr_lin(bool shadowOn, F3 L, F3 Vd, F3 Hd, F3 N, float vis, F3 al, F3 el, F3 param,
                                      F3 radiance)
{
    float ao = param.x, metal = param.y, rough = param.z;
    return pbr_finish(pbr_direct(shadowOn, L, Vd, Hd, N, vis, al, metal, rough, radiance), al, el, ao);
}

__device__ __forceinline__ F3 pbr(bool shadowOn, F3 L, F3 Vd, F3 Hd, F3 N, float vis, F3 albedo, F3 emissive,
                                  F3 param, F3 radiance)
{
    const float kGamma = 2.2f;
    return pbr_lin(shadowOn, L, Vd, Hd, N, vis, powv(albedo, kGamma), powv(emissive, kGamma), param, radiance);
}
__device__ __forceinline__ unsigned quantize_rgb(F3 c)
{
    unsigned r = (unsigned)(c.x * 254.99f), g = (unsigned)(c.y * 254.99f), b = (unsigned)(c.z * 254.99f);
    return (r & 0xffu) | ((g & 0xffu) << 8) | ((b & 0xffu) << 16);
}

}  // namespace frd
