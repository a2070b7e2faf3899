// CPU oracle of the per-frame pipeline (TEST INFRASTRUCTURE ONLY; see fr_oracle.h).
//
// Restates the reference frame statement by statement, in the reference's own
// evaluation order, float/double types and loop structure:
//   vertex shaders  src/shaders/depthshader.h:21-36, gshader.h:41-92,
//                   phongshader.h:35-85, pbrshader.h:35-85
//   raster          src/forkergl.cpp:165-250 (bbox, px-outer / py-inner loop,
//                   strict-less depth test), Barycentric geometry.cpp:20-56
//   fragment        gshader.h:95-202, phongshader.h:90-169, pbrshader.h:90-180
//   textures        src/texture.h:41-132 (NoWrap + Nearest), tgaimage.cpp:304-311
//   shadows         src/shaders/shadow.cpp:23-132
//   SSAO + blur     src/render.cpp:214-289, buffer.cpp:59-98
//   lighting        forkergl.cpp:326-380, phongshader.h:171-215, pbrshader.h:182-288
//   SSAA            render.cpp:291-345, buffer.cpp:113-126
// The random draws of the reference are replaced by the deterministic tables of
// include/fr_sample_tables.h. Compile with -ffp-contract=off.
//
// Where the reference has undefined behaviour this file fixes one meaning, and
// the GB300 path implements the same one:
//   * float -> int conversion of out-of-range values saturates (NaN -> 0), as on
//     aarch64 and in CUDA; x86 gives INT_MIN;
//   * SSAO depth reads: a linear index x + y * W inside the buffer reads it
//     (rows wrap exactly as the reference's unchecked read does), any other
//     index reads FLT_MAX;
//   * a NaN texture coordinate samples black; a NaN shadow-map coordinate is
//     outside the map (+inf).
#include "fr_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "fr_sample_tables.h"

namespace
{

const float kMaxFloat = 3.40282347e+38f;
const float kPi = 3.14159265358979323846f;
const float kInvPi = 0.31830988618379067154f;
const float kGamma = 2.2f;
const float kInvGamma = 1.f / 2.2f;

struct V2
{
    float x, y;
};
struct V3
{
    float x, y, z;
};
struct V4
{
    float x, y, z, w;
};
struct M4
{
    float m[4][4];
};
struct M3
{
    float m[3][3];
};

inline V3 v3(float a) { return V3{a, a, a}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float f) { return V3{a.x * f, a.y * f, a.z * f}; }
inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
// Vector / f multiplies by the reciprocal (geometry.h:176-182)
inline V3 divs(V3 a, float f)
{
    float inv = 1.f / f;
    return V3{a.x * inv, a.y * inv, a.z * inv};
}
// Vector / Vector divides component-wise (geometry.h:184-187)
inline V3 divv(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float dot(V3 a, V3 b)
{
    float r = 0.f;
    r += a.x * b.x;
    r += a.y * b.y;
    r += a.z * b.z;
    return r;
}
inline float length(V3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
inline V3 normalize(V3 v) { return divs(v * 1.f, length(v)); }
inline V3 cross(V3 a, V3 b)
{
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float clampf(float v, float lo, float hi) { return std::min(hi, std::max(v, lo)); }
inline V3 clamp01(V3 v) { return V3{clampf(v.x, 0.f, 1.f), clampf(v.y, 0.f, 1.f), clampf(v.z, 0.f, 1.f)}; }
inline V3 powv(V3 v, float p) { return V3{std::pow(v.x, p), std::pow(v.y, p), std::pow(v.z, p)}; }
inline float maxf(float a, float b) { return std::max(a, b); }
inline V3 lerp(float t, V3 a, V3 b) { return a * (1 - t) + b * t; }
inline float lerpf(float t, float a, float b) { return (1 - t) * a + t * b; }

inline V4 mul(const M4& m, V4 v)
{
    float in[4] = {v.x, v.y, v.z, v.w}, o[4];
    for (int r = 0; r < 4; ++r)
    {
        float s = 0.f;
        for (int k = 0; k < 4; ++k) s += m.m[r][k] * in[k];
        o[r] = s;
    }
    return V4{o[0], o[1], o[2], o[3]};
}
inline V3 mul(const M3& m, V3 v)
{
    float in[3] = {v.x, v.y, v.z}, o[3];
    for (int r = 0; r < 3; ++r)
    {
        float s = 0.f;
        for (int k = 0; k < 3; ++k) s += m.m[r][k] * in[k];
        o[r] = s;
    }
    return V3{o[0], o[1], o[2]};
}
inline M4 mul(const M4& a, const M4& b)
{
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
        {
            float s = 0.f;
            for (int k = 0; k < 4; ++k) s += a.m[i][k] * b.m[k][j];
            r.m[i][j] = s;
        }
    return r;
}
inline V4 scale4(V4 v, float f) { return V4{v.x * f, v.y * f, v.z * f, v.w * f}; }
inline V4 div4(V4 v, float f)
{
    float inv = 1.f / f;
    return V4{v.x * inv, v.y * inv, v.z * inv, v.w * inv};
}
inline M4 identity()
{
    M4 r;
    std::memset(&r, 0, sizeof r);
    for (int i = 0; i < 4; ++i) r.m[i][i] = 1.f;
    return r;
}

// float -> int with saturation (the meaning fixed for out-of-range values).
inline int f2i(float f)
{
    if (!(f == f)) return 0;
    if (f >= 2147483648.f) return 2147483647;
    if (f < -2147483648.f) return (-2147483647 - 1);
    return (int)f;
}

// ---- matrices (geometry.cpp:60-179, render.cpp:9-14, 73-78, 106-114) -------
float radians(float deg) { return deg * kPi / 180.f; }

M4 look_at(V3 eye, V3 center)
{
    V3 front = normalize(center - eye);
    V3 right = normalize(cross(front, V3{0.f, 1.f, 0.f}));
    V3 up = normalize(cross(right, front));
    M4 R = identity();
    float rows[3][3] = {{right.x, right.y, right.z}, {up.x, up.y, up.z}, {-front.x, -front.y, -front.z}};
    for (int r = 0; r < 3; ++r)
    {
        for (int c = 0; c < 3; ++c) R.m[r][c] = rows[r][c];
        R.m[r][3] = 0.f;
    }
    M4 T = identity();
    T.m[0][3] = -eye.x, T.m[1][3] = -eye.y, T.m[2][3] = -eye.z;
    return mul(R, T);
}

M4 perspective(float fov, float aspect, float n, float f)
{
    float t = std::tan(radians(fov / 2.f));
    M4 m = identity();
    m.m[0][0] = 1.f / (aspect * t);
    m.m[1][1] = 1.f / t;
    m.m[2][2] = -(f + n) / (f - n);
    m.m[2][3] = -2 * f * n / (f - n);
    m.m[3][2] = -1;
    return m;
}

M4 ortho(float l, float r, float b, float t, float n, float f)
{
    M4 m = identity();
    m.m[0][0] = 2.f / (r - l);
    m.m[1][1] = 2.f / (t - b);
    m.m[2][2] = -2.f / (f - n);
    m.m[0][3] = -(r + l) / (r - l);
    m.m[1][3] = -(t + b) / (t - b);
    m.m[2][3] = -(f + n) / (f - n);
    m.m[3][3] = 1.f;
    return m;
}

M4 viewport(int w, int h)
{
    M4 m = identity();
    m.m[0][0] = w / 2.f;
    m.m[1][1] = h / 2.f;
    m.m[0][3] = 0 + w / 2.f;
    m.m[1][3] = 0 + h / 2.f;
    m.m[2][2] = 1 / 2.f;
    m.m[2][3] = 1 / 2.f;
    return m;
}

M4 model_matrix(V3 t, float yrot, float scale)
{
    M4 S = identity();
    S.m[0][0] = S.m[1][1] = S.m[2][2] = scale;
    M4 R = identity();
    float rad = radians(yrot);
    R.m[0][0] = (float)std::cos((double)rad);
    R.m[0][2] = (float)std::sin((double)rad);
    R.m[2][0] = (float)(-std::sin((double)rad));
    R.m[2][2] = (float)std::cos((double)rad);
    M4 T = identity();
    T.m[0][3] = t.x, T.m[1][3] = t.y, T.m[2][3] = t.z;
    return mul(mul(T, R), S);
}

// Matrix::Det / Cofactor / Inverse (geometry.h:605-624, 705-742)
float det_n(const float a[4][4], int n);
float cofactor_n(const float a[4][4], int n, int row, int col)
{
    float mnr[4][4] = {};
    for (int i = 0; i < n - 1; ++i)
        for (int j = 0; j < n - 1; ++j) mnr[i][j] = a[i < row ? i : i + 1][j < col ? j : j + 1];
    return det_n(mnr, n - 1) * ((row + col) % 2 ? -1 : 1);
}
float det_n(const float a[4][4], int n)
{
    if (n == 1) return a[0][0];
    float ret = 0;
    for (int i = 0; i < n; ++i) ret += a[0][i] * cofactor_n(a, n, 0, i);
    return ret;
}

M3 normal_matrix(const M4& M)
{
    float adj[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) adj[j][i] = cofactor_n(M.m, 4, i, j);
    float d = det_n(M.m, 4);
    float inv[4][4];
    for (int i = 0; i < 4; ++i)
    {
        float r = 1.f / d;
        for (int j = 0; j < 4; ++j) inv[i][j] = adj[i][j] * r;
    }
    M3 n;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) n.m[r][c] = inv[c][r];
    return n;
}

// ---- barycentric (geometry.cpp:20-56) ------------------------------------------
inline bool barycentric(const int* X, const int* Y, int px, int py, V3& out)
{
    float ax = (float)X[0], ay = (float)Y[0], bx = (float)X[1], by = (float)Y[1];
    float cx = (float)X[2], cy = (float)Y[2], fx = (float)px, fy = (float)py;
    double s0x = bx - ax, s0y = cx - ax, s0z = ax - fx;
    double s1x = by - ay, s1y = cy - ay, s1z = ay - fy;
    double bxv = s0y * s1z - s0z * s1y;
    double byv = s0z * s1x - s0x * s1z;
    double bzv = s0x * s1y - s0y * s1x;
    if (std::abs(bzv) > 1e-2)
    {
        double inv = 1.f / bzv;
        bxv *= inv;
        byv *= inv;
        V3 r{(float)(1.f - (bxv + byv)), (float)bxv, (float)byv};
        if (r.x < 0.f || r.y < 0.f || r.z < 0.f) return false;
        out = r;
        return true;
    }
    return false;
}

// ---- textures (texture.h:41-132, tgaimage.cpp:304-311) -----------------------
// The wrap and filter modes of the frame being rendered (one render at a time).
int g_texWrap = 0;
int g_texLinear = 0;

// Texture::wrapCoord (texture.h:62-83), component by component.
inline float wrap_coord(int mode, float c)
{
    if (mode == 1) return c - std::floor(c);  // Repeat
    if (mode == 2)                             // MirroredRepeat
    {
        const int i = f2i(std::floor(c));
        const float rep = c - (float)i;
        return i % 2 == 0 ? rep : 1.f - rep;
    }
    if (mode == 3) return std::min(1.f, std::max(c, 0.f));  // ClampToEdge: Clamp01
    return c;                                                // NoWrap
}

// TGAImage::Get (tgaimage.cpp:304-311) as Texture::getColorFromImage's Color3
// (texture.h:130-134): black outside the image.
inline V3 image_texel(const fr_texture_view& t, int x, int y)
{
    if (x < 0 || y < 0 || x >= t.width || y >= t.height) return V3{0.f, 0.f, 0.f};
    const uint8_t* p = t.data + ((size_t)x + (size_t)y * t.width) * t.bytes_per_pixel;
    uint8_t bgra[4] = {0, 0, 0, 0};
    for (int i = 0; i < t.bytes_per_pixel; ++i) bgra[i] = p[i];
    return V3{(float)bgra[2], (float)bgra[1], (float)bgra[0]};
}

// Texture::colorFromFiltering (texture.h:85-127) after wrapCoord: color in [0, 255].
inline V3 texel(const fr_texture_view& t, V2 uv)
{
    if (g_texWrap) uv = V2{wrap_coord(g_texWrap, uv.x), wrap_coord(g_texWrap, uv.y)};
    float w = (float)(t.width - 0.001), h = (float)(t.height - 0.001);
    if (g_texLinear)
    {
        // image-space point, the texel whose centre is up and left of it, weights
        const float px = uv.x * w, py = uv.y * h;
        const float lx = std::floor(px - 0.5f), ly = std::floor(py - 0.5f);
        const float tx = px - (lx + 0.5f), ty = py - (ly + 0.5f);
        int x0 = f2i(lx), y0 = f2i(ly), x1 = f2i(lx + 1.f), y1 = f2i(ly + 1.f);
        if (g_texWrap)  // clampImageCoord (texture.h:140-144); NoWrap reads black outside
        {
            x0 = std::min(t.width - 1, std::max(x0, 0)), x1 = std::min(t.width - 1, std::max(x1, 0));
            y0 = std::min(t.height - 1, std::max(y0, 0)), y1 = std::min(t.height - 1, std::max(y1, 0));
        }
        const V3 top = lerp(tx, image_texel(t, x0, y0), image_texel(t, x1, y0));
        const V3 bottom = lerp(tx, image_texel(t, x0, y1), image_texel(t, x1, y1));
        return lerp(ty, top, bottom);
    }
    float fu = std::floor(uv.x * w), fv = std::floor(uv.y * h);
    if (!(fu == fu) || !(fv == fv)) return V3{0.f, 0.f, 0.f};
    return image_texel(t, f2i(fu), f2i(fv));
}
inline V3 sample(const fr_texture_view& t, V2 uv) { return divs(texel(t, uv), 255.f); }
inline float sample_float(const fr_texture_view& t, V2 uv) { return texel(t, uv).z / 255.f; }

// ---- per-triangle varyings of the vertex shaders ----------------------------------
struct Tri
{
    int X[3], Y[3];
    V3 depths;
    int model, material;
    // camera shaders (gshader.h:41-92, phongshader.h:35-85, pbrshader.h:35-85)
    V3 pw[3];
    V2 uvw[3];
    V3 nw[3];
    V3 tw[3];
    V3 lw[3];
    float ow[3];
    // depth shader (depthshader.h:21-28)
    float ndcz[3];
};

struct Frame
{
    const fr_scene_view* S;
    fr_oracle_config cfg;
    fr_frame_matrices fm;
    M4 V, P, VP, L, VPort, SVPort;
    std::vector<M4> modelM, modelLM;
    std::vector<M3> modelN;
    int W, H, SW, SH;
    bool shadowOn, deferred, ssaoOn, ssaaOn;
    int ssaaK;
    V3 eye, lightPos, lightColor;
    std::vector<float> blocker, pcf, ssaoK;
    // buffers
    std::vector<float> depth, shadow, ao, type;
    std::vector<V3> gNormal, gPos, gLndc, gAlbedo, gEmissive, gParam, frame;
    std::vector<Tri> tris;
};

template <typename F>
void parallel_for(int n, int threads, F fn)
{
    threads = std::max(1, std::min(threads, n));
    if (threads == 1)
    {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
    {
        int a = (int)((long long)n * t / threads), b = (int)((long long)n * (t + 1) / threads);
        pool.emplace_back([=]() { fn(a, b); });
    }
    for (auto& th : pool) th.join();
}

const fr_material_view& material_of(const Frame& F, int t)
{
    return F.S->materials[F.S->meshes[F.S->tri_mesh[t]].material];
}

V3 load3(const float* p, int64_t i) { return V3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

// Vertex stage of the camera shaders for triangle t.
void vertex_camera(const Frame& F, int t, Tri& T)
{
    const fr_scene_view* S = F.S;
    int mesh = S->tri_mesh[t];
    T.model = S->meshes[mesh].model;
    T.material = S->meshes[mesh].material;
    const fr_model_view& mv = S->models[T.model];
    const M4& M = F.modelM[T.model];
    const M3& N3 = F.modelN[T.model];
    V4 ndc[3];
    for (int k = 0; k < 3; ++k)
    {
        int vi = S->tri_v[3 * t + k], ti = S->tri_vt[3 * t + k], ni = S->tri_vn[3 * t + k];
        V3 p = load3(S->positions, vi);
        V4 posWS = mul(M, V4{p.x, p.y, p.z, 1.f});
        V4 posVS = mul(F.V, posWS);
        V4 posCS = mul(F.P, posVS);
        V2 uv{S->uvs[2 * ti], S->uvs[2 * ti + 1]};
        V3 nWS = mul(N3, normalize(load3(S->normals, ni)));
        V3 tWS{0.f, 0.f, 0.f};
        if (mv.has_tangents) tWS = mul(N3, normalize(load3(S->tangents, vi)));
        V4 lndc{0.f, 0.f, 0.f, 0.f};
        if (F.shadowOn)
        {
            lndc = mul(F.L, posWS);
            lndc = div4(lndc, lndc.w);
        }
        float ow = 1.f / posCS.w;
        T.ow[k] = ow;
        posWS = scale4(posWS, ow);
        uv = V2{uv.x * ow, uv.y * ow};
        nWS = nWS * ow;
        if (mv.has_tangents) tWS = tWS * ow;
        if (F.shadowOn) lndc = scale4(lndc, ow);
        T.pw[k] = V3{posWS.x, posWS.y, posWS.z};
        T.uvw[k] = uv;
        T.nw[k] = nWS;
        T.tw[k] = tWS;
        T.lw[k] = V3{lndc.x, lndc.y, lndc.z};
        ndc[k] = div4(posCS, posCS.w);
    }
    for (int k = 0; k < 3; ++k)
    {
        V4 c = mul(F.VPort, ndc[k]);
        T.X[k] = f2i(c.x);
        T.Y[k] = f2i(c.y);
        (&T.depths.x)[k] = c.z;
    }
}

// DepthShader (depthshader.h:21-28): (L * M) * v, then / w.
void vertex_light(const Frame& F, int t, Tri& T)
{
    const fr_scene_view* S = F.S;
    int mesh = S->tri_mesh[t];
    T.model = S->meshes[mesh].model;
    const M4& LM = F.modelLM[T.model];
    for (int k = 0; k < 3; ++k)
    {
        V3 p = load3(S->positions, S->tri_v[3 * t + k]);
        V4 cs = mul(LM, V4{p.x, p.y, p.z, 1.f});
        V4 ndc = div4(cs, cs.w);
        T.ndcz[k] = ndc.z;
        V4 c = mul(F.SVPort, ndc);
        T.X[k] = f2i(c.x);
        T.Y[k] = f2i(c.y);
        (&T.depths.x)[k] = c.z;
    }
}

inline float interp(float a, float b, float c, V3 bary) { return dot(V3{a, b, c}, bary); }

// Interpolated, perspective-corrected fragment inputs (gshader.h:95-143 and the
// identical prologue of phongshader.h:292-330 / pbrshader.h:90-129).
struct Frag
{
    V3 pos, normal, lndc;
    V2 uv;
};

Frag fragment_inputs(const Frame& F, const Tri& T, V3 b)
{
    const fr_material_view& mat = F.S->materials[T.material];
    const fr_model_view& mv = F.S->models[T.model];
    Frag f;
    V3 pos{interp(T.pw[0].x, T.pw[1].x, T.pw[2].x, b), interp(T.pw[0].y, T.pw[1].y, T.pw[2].y, b),
           interp(T.pw[0].z, T.pw[1].z, T.pw[2].z, b)};
    V2 uv{interp(T.uvw[0].x, T.uvw[1].x, T.uvw[2].x, b), interp(T.uvw[0].y, T.uvw[1].y, T.uvw[2].y, b)};
    V3 n{interp(T.nw[0].x, T.nw[1].x, T.nw[2].x, b), interp(T.nw[0].y, T.nw[1].y, T.nw[2].y, b),
         interp(T.nw[0].z, T.nw[1].z, T.nw[2].z, b)};
    float w = 1.f / dot(V3{T.ow[0], T.ow[1], T.ow[2]}, b);
    pos = pos * w;
    uv = V2{uv.x * w, uv.y * w};
    n = n * w;
    V3 N = normalize(n);
    V3 normal;
    if (mv.has_tangents && mat.map_bump >= 0)
    {
        V3 tg{interp(T.tw[0].x, T.tw[1].x, T.tw[2].x, b), interp(T.tw[0].y, T.tw[1].y, T.tw[2].y, b),
              interp(T.tw[0].z, T.tw[1].z, T.tw[2].z, b)};
        tg = tg * w;
        V3 Tn = normalize(tg + v3(0.001f));
        Tn = normalize(Tn - N * dot(Tn, N));
        V3 B = normalize(cross(N, Tn));
        M3 tbn;
        tbn.m[0][0] = Tn.x, tbn.m[0][1] = B.x, tbn.m[0][2] = N.x;
        tbn.m[1][0] = Tn.y, tbn.m[1][1] = B.y, tbn.m[1][2] = N.y;
        tbn.m[2][0] = Tn.z, tbn.m[2][1] = B.z, tbn.m[2][2] = N.z;
        V3 s = sample(F.S->textures[mat.map_bump], uv);
        s = normalize(s * 2.f - v3(1.f));
        normal = normalize(mul(tbn, s));
    }
    else
    {
        normal = N;
    }
    V3 l{0.f, 0.f, 0.f};
    if (F.shadowOn)
    {
        l = V3{interp(T.lw[0].x, T.lw[1].x, T.lw[2].x, b), interp(T.lw[0].y, T.lw[1].y, T.lw[2].y, b),
               interp(T.lw[0].z, T.lw[1].z, T.lw[2].z, b)};
        l = l * w;
    }
    f.pos = pos;
    f.normal = normal;
    f.lndc = l;
    f.uv = uv;
    return f;
}

// ---- shadows (shadow.cpp:23-132) ---------------------------------------------------
struct ShadowMap
{
    const float* data;
    int w, h;
};

inline float sample_shadow(const ShadowMap& m, V2 uv)
{
    if (uv.x < 0.f || uv.x > 1.f || uv.y < 0.f || uv.y > 1.f) return INFINITY;
    if (!(uv.x == uv.x) || !(uv.y == uv.y)) return INFINITY;
    int w = (int)(m.w - 0.001f);
    int h = (int)(m.h - 0.001f);
    int u = (int)((float)w * uv.x);
    int v = (int)((float)h * uv.y);
    float depth = m.data[(size_t)u + (size_t)v * m.w];
    return depth < 0.001 ? 1.f : depth;
}

float pcf(const Frame& F, const ShadowMap& m, V3 c, float bias, float filter)
{
    float vis = 0.f;
    float invN = 1.f / (float)F.cfg.pcf_samples;
    for (int i = 0; i < F.cfg.pcf_samples; ++i)
    {
        V2 uv{c.x + F.pcf[2 * i] * filter, c.y + F.pcf[2 * i + 1] * filter};
        float s = sample_shadow(m, uv);
        if (c.z <= s + bias) vis += invN;
    }
    return vis;
}

float blocker_depth(const Frame& F, const ShadowMap& m, V3 c, float bias)
{
    float sum = 0.f, num = 0.f;
    for (int i = 0; i < F.cfg.blocker_samples; ++i)
    {
        float ox = (float)((double)F.blocker[2 * i] * 0.005);
        float oy = (float)((double)F.blocker[2 * i + 1] * 0.005);
        V2 uv{c.x + ox, c.y + oy};
        float s = sample_shadow(m, uv);
        if (c.z > s + bias)
        {
            sum += s;
            num += 1.f;
        }
    }
    if (num < 1.f) return 0.f;
    return sum / num;
}

float shadow_visibility(const Frame& F, V3 lndc, V3 normal, V3 lightDir)
{
    ShadowMap m{F.shadow.data(), F.SW, F.SH};
    V3 c = lndc * 0.5f + v3(0.5f);
    float bias = maxf(0.009f * (1.f - dot(normal, lightDir)), 0.007f);
    if (F.cfg.shadow_mode == 1) return pcf(F, m, c, bias, (float)0.007);
    if (F.cfg.shadow_mode == 2)
    {
        float dR = c.z;
        float dB = blocker_depth(F, m, c, bias);
        if (dB < 0.001) return 1.f;
        float pen = (dR - dB) * 2.5f / dB;
        float filter = (float)(0.007 * (double)pen);
        return pcf(F, m, c, bias, filter);
    }
    float d = sample_shadow(m, V2{c.x, c.y});
    return (c.z <= d + bias) ? 1.f : 0.f;
}

// ---- lighting models -------------------------------------------------------------------
V3 blinn_phong(const Frame& F, V3 L, V3 Hd, V3 N, float vis, V3 diffuseColor, V3 emissive, V3 param,
               V3 lightColor)
{
    V3 dl = powv(diffuseColor, kGamma);
    V3 el = powv(emissive, kGamma);
    float ao = param.x, ks = param.y, shin = param.z;
    float diff = maxf(0.f, dot(L, N));
    float spec = std::pow(maxf(0.f, dot(Hd, N)), shin);
    V3 ambient = v3(0.3f) * dl * ao;
    V3 diffuse = dl * diff * ao;
    V3 specular = v3(ks) * spec;
    if (F.shadowOn)
    {
        float shadow = (1 - vis) * 0.6f;
        vis = 1 - shadow;
        diffuse = diffuse * vis;
        specular = specular * vis;
    }
    V3 color = ambient + (diffuse + specular + el) * lightColor;
    color = divv(color, color + v3(1.f));
    color = powv(color, kInvGamma);
    return clamp01(color);
}

float ggx(float NdotH, float r)
{
    float a = r * r;
    float a2 = a * a;
    float n2 = NdotH * NdotH;
    float d = (n2 * (a2 - 1.f) + 1.f);
    float d2 = d * d;
    return a2 * kInvPi / d2;
}
float schlick_ggx(float NdotV, float r)
{
    float a = r + 1.f;
    float k = a * a / 8.f;
    return NdotV / (NdotV * (1 - k) + k);
}

V3 pbr(const Frame& F, V3 L, V3 Vd, V3 Hd, V3 N, float vis, V3 albedo, V3 emissive, V3 param, V3 radiance)
{
    V3 al = powv(albedo, kGamma);
    V3 el = powv(emissive, kGamma);
    float ao = param.x, metal = param.y, rough = param.z;
    float NdotV = maxf(dot(N, Vd), 0.f);
    float NdotL = maxf(dot(N, L), 0.f);
    float NdotH = maxf(dot(N, Hd), 0.f);
    float HdotV = maxf(dot(Hd, Vd), 0.f);
    V3 F0 = v3(0.04f);
    F0 = lerp(metal, F0, al);
    float NDF = ggx(NdotH, rough);
    float G = schlick_ggx(NdotV, rough) * schlick_ggx(NdotL, rough);
    float om = maxf(1.f - HdotV, 0.f);
    V3 Fr = F0 + (v3(1.f) - F0) * std::pow(om, 5.f);
    V3 DGF = Fr * (NDF * G);
    float denom = 4 * NdotV * NdotL + 0.001f;
    V3 ks = Fr;
    V3 specular = divs(DGF, denom);
    V3 kd = v3(1.f) - ks;
    kd = kd * (1.f - metal);
    V3 brdf = kd * al * kInvPi + specular;
    V3 Lo = brdf * radiance * NdotL;
    if (F.shadowOn)
    {
        float shadow = (1 - vis) * 0.6f;
        vis = 1 - shadow;
        Lo = Lo * vis;
    }
    V3 color = Lo;
    V3 ambient = v3(0.3f) * al * ao;
    color = color + ambient;
    color = color + el;
    color = divv(color, color + v3(1.f));
    color = powv(color, kInvGamma);
    return clamp01(color);
}

// ---- passes ----------------------------------------------------------------------------
void bbox(const Tri& T, int w, int h, int& x0, int& x1, int& y0, int& y1)
{
    auto clampi = [](int v, int lo, int hi) { return std::min(hi, std::max(v, lo)); };
    x0 = clampi(std::min(T.X[0], std::min(T.X[1], T.X[2])), 0, w - 1);
    y0 = clampi(std::min(T.Y[0], std::min(T.Y[1], T.Y[2])), 0, h - 1);
    x1 = clampi(std::max(T.X[0], std::max(T.X[1], T.X[2])), 0, w - 1);
    y1 = clampi(std::max(T.Y[0], std::max(T.Y[1], T.Y[2])), 0, h - 1);
}

void shadow_pass(Frame& F)
{
    const int T = (int)F.S->info.num_triangles;
    F.tris.assign(T, Tri());
    parallel_for(T, F.cfg.threads, [&](int a, int b) {
        for (int t = a; t < b; ++t) vertex_light(F, t, F.tris[t]);
    });
    std::vector<float> zb((size_t)F.SW * F.SH, kMaxFloat);
    F.shadow.assign((size_t)F.SW * F.SH, 0.f);
    parallel_for(F.SH, F.cfg.threads, [&](int ya, int yb) {
        for (int t = 0; t < T; ++t)
        {
            const Tri& tr = F.tris[t];
            int x0, x1, y0, y1;
            bbox(tr, F.SW, F.SH, x0, x1, y0, y1);
            y0 = std::max(y0, ya);
            y1 = std::min(y1, yb - 1);
            for (int px = x0; px <= x1; ++px)
                for (int py = y0; py <= y1; ++py)
                {
                    V3 b;
                    if (!barycentric(tr.X, tr.Y, px, py, b)) continue;
                    float cur = dot(b, tr.depths);
                    size_t i = (size_t)px + (size_t)py * F.SW;
                    if (cur >= zb[i]) continue;
                    zb[i] = cur;
                    float z = interp(tr.ndcz[0], tr.ndcz[1], tr.ndcz[2], b);
                    F.shadow[i] = z * 0.5f + 0.5f;
                }
        }
    });
}

// Geometry pass (deferred) or forward pass over the camera.
void camera_pass(Frame& F)
{
    const int T = (int)F.S->info.num_triangles;
    const size_t P = (size_t)F.W * F.H;
    F.tris.assign(T, Tri());
    parallel_for(T, F.cfg.threads, [&](int a, int b) {
        for (int t = a; t < b; ++t) vertex_camera(F, t, F.tris[t]);
    });
    F.depth.assign(P, kMaxFloat);
    if (F.deferred)
    {
        V3 z{0.f, 0.f, 0.f};
        F.gNormal.assign(P, z), F.gPos.assign(P, z), F.gLndc.assign(P, z), F.gAlbedo.assign(P, z);
        F.gEmissive.assign(P, z), F.gParam.assign(P, z);
        F.type.assign(P, 0.f);
        F.ao.assign(P, 1.f);
        F.frame.assign(P, z);
    }
    else
    {
        F.frame.assign(P, v3(0.12f));  // ClearColor (render.cpp:103)
    }
    parallel_for(F.H, F.cfg.threads, [&](int ya, int yb) {
        for (int t = 0; t < T; ++t)
        {
            const Tri& tr = F.tris[t];
            int x0, x1, y0, y1;
            bbox(tr, F.W, F.H, x0, x1, y0, y1);
            y0 = std::max(y0, ya);
            y1 = std::min(y1, yb - 1);
            for (int px = x0; px <= x1; ++px)
                for (int py = y0; py <= y1; ++py)
                {
                    V3 b;
                    if (!barycentric(tr.X, tr.Y, px, py, b)) continue;
                    float cur = dot(b, tr.depths);
                    size_t i = (size_t)px + (size_t)py * F.W;
                    if (cur >= F.depth[i]) continue;
                    F.depth[i] = cur;
                    Frag fr = fragment_inputs(F, tr, b);
                    const fr_material_view& mat = F.S->materials[tr.material];
                    const fr_model_view& mv = F.S->models[tr.model];
                    const fr_texture_view* tx = F.S->textures;
                    if (F.deferred)
                    {
                        F.gNormal[i] = fr.normal;
                        F.gPos[i] = fr.pos;
                        if (F.shadowOn) F.gLndc[i] = fr.lndc;
                        if (mv.support_pbr)
                        {
                            V3 albedo = mat.map_kd >= 0 ? sample(tx[mat.map_kd], fr.uv)
                                                        : V3{mat.pbr_albedo[0], mat.pbr_albedo[1], mat.pbr_albedo[2]};
                            V3 emissive = mat.map_ke >= 0 ? sample(tx[mat.map_ke], fr.uv)
                                                          : V3{mat.ke[0], mat.ke[1], mat.ke[2]};
                            float rough = mat.map_pr >= 0 ? sample_float(tx[mat.map_pr], fr.uv) : mat.roughness;
                            float metal = mat.map_pm >= 0 ? sample_float(tx[mat.map_pm], fr.uv) : mat.metalness;
                            float ao = mat.map_ao >= 0 ? sample_float(tx[mat.map_ao], fr.uv) : 1.f;
                            F.gAlbedo[i] = albedo;
                            F.gEmissive[i] = emissive;
                            F.gParam[i] = V3{ao, metal, rough};
                            F.type[i] = 1.f;
                        }
                        else
                        {
                            V3 emissive = mat.map_ke >= 0 ? sample(tx[mat.map_ke], fr.uv)
                                                          : V3{mat.ke[0], mat.ke[1], mat.ke[2]};
                            V3 diffuse = mat.map_kd >= 0 ? sample(tx[mat.map_kd], fr.uv)
                                                         : V3{mat.kd[0], mat.kd[1], mat.kd[2]};
                            float shin = mat.map_ks >= 0 ? sample_float(tx[mat.map_ks], fr.uv) + 5 : 1.f;
                            F.gAlbedo[i] = diffuse;
                            F.gEmissive[i] = emissive;
                            F.gParam[i] = V3{1.f, mat.ks[0], shin};
                            F.type[i] = 0.f;
                        }
                    }
                    else
                    {
                        V3 L = normalize(F.lightPos - fr.pos);
                        V3 Vd = normalize(F.eye - fr.pos);
                        V3 Hd = normalize(L + Vd);
                        float vis = 0.f;
                        if (F.shadowOn) vis = shadow_visibility(F, fr.lndc, fr.normal, L);
                        V3 c;
                        if (!mv.support_pbr)
                        {
                            V3 diffuse = mat.map_kd >= 0 ? sample(tx[mat.map_kd], fr.uv)
                                                         : V3{mat.kd[0], mat.kd[1], mat.kd[2]};
                            V3 emissive = mat.map_ke >= 0 ? sample(tx[mat.map_ke], fr.uv)
                                                          : V3{mat.ke[0], mat.ke[1], mat.ke[2]};
                            float shin = 1.f;
                            if (mat.map_ks >= 0) shin = sample_float(tx[mat.map_ks], fr.uv) + 5;
                            V3 param{mat.ka[0], mat.ks[0], shin};
                            c = blinn_phong(F, L, Hd, fr.normal, vis, diffuse, emissive, param, F.lightColor);
                        }
                        else
                        {
                            V3 albedo = mat.map_kd >= 0 ? sample(tx[mat.map_kd], fr.uv)
                                                        : V3{mat.pbr_albedo[0], mat.pbr_albedo[1], mat.pbr_albedo[2]};
                            V3 emissive = mat.map_ke >= 0 ? sample(tx[mat.map_ke], fr.uv)
                                                          : V3{mat.ke[0], mat.ke[1], mat.ke[2]};
                            float rough = mat.map_pr >= 0 ? sample_float(tx[mat.map_pr], fr.uv) : mat.roughness;
                            float metal = mat.map_pm >= 0 ? sample_float(tx[mat.map_pm], fr.uv) : mat.metalness;
                            float ao = mat.map_ao >= 0 ? sample_float(tx[mat.map_ao], fr.uv) : 1.f;
                            c = pbr(F, L, Vd, Hd, fr.normal, vis, albedo, emissive, V3{ao, metal, rough},
                                    F.lightColor);
                        }
                        F.frame[i] = c;
                    }
                }
        }
    });
}

void ssao_pass(Frame& F)
{
    const int N = F.cfg.ssao_samples;
    const float kernelScale = 1.f / N;
    const float radius = F.cfg.ssao_radius, bias = F.cfg.ssao_bias, range = F.cfg.ssao_range;
    const size_t P = (size_t)F.W * F.H;
    parallel_for(F.H, F.cfg.threads, [&](int ya, int yb) {
        for (int y = ya; y < yb; ++y)
            for (int x = 0; x < F.W; ++x)
            {
                size_t i = (size_t)x + (size_t)y * F.W;
                V3 pos = F.gPos[i], nrm = F.gNormal[i];
                float fragDepth = F.depth[i];
                float occ = 0.f;
                int cell = (y & 3) * 4 + (x & 3);
                for (int s = 0; s < N; ++s)
                {
                    const float* k = &F.ssaoK[3 * (cell * N + s)];
                    V3 dir{k[0], k[1], k[2]};
                    if (!(dot(dir, nrm) > 0.f)) dir = -dir;
                    float sc = length(dir);
                    sc = lerpf(0.1f, 1.0f, sc * sc);
                    dir = dir * sc;
                    V3 sp = pos + dir * radius;
                    V4 cs = mul(F.VP, V4{sp.x, sp.y, sp.z, 1.f});
                    V4 ndc = div4(cs, cs.w);
                    V4 ss = mul(F.VPort, ndc);
                    int sx = f2i(ss.x), sy = f2i(ss.y);
                    float sd = ss.z;
                    long long li = (long long)sx + (long long)sy * F.W;
                    float cached = (li >= 0 && li < (long long)P) ? F.depth[(size_t)li] : kMaxFloat;
                    if (sd >= cached + bias)
                    {
                        float rc = std::abs(fragDepth - cached) < range ? 1.f : 0.f;
                        occ += kernelScale * rc;
                    }
                }
                occ = 1.f - occ;
                occ = std::pow(occ, 3.f);
                F.ao[i] = occ;
            }
    });
}

const float kBlurW[5] = {0.227027f, 0.1945946f, 0.1216216f, 0.054054f, 0.016216f};

void blur_reference(Frame& F)
{
    float* a = F.ao.data();
    const int W = F.W, H = F.H;
    parallel_for(H, F.cfg.threads, [&](int ha, int hb) {
        for (int h = ha; h < hb; ++h)
            for (int w = 0; w < W; ++w)
            {
                float r = a[w + (size_t)h * W] * kBlurW[0];
                for (int i = 1; i < 5; ++i)
                {
                    int w1 = std::min(W - 1, std::max(w + i, 0));
                    int w2 = std::min(W - 1, std::max(w - i, 0));
                    r += a[w1 + (size_t)h * W] * kBlurW[i];
                    r += a[w2 + (size_t)h * W] * kBlurW[i];
                }
                a[w + (size_t)h * W] = r;
            }
    });
    parallel_for(W, F.cfg.threads, [&](int wa, int wb) {
        for (int h = 0; h < H; ++h)
            for (int w = wa; w < wb; ++w)
            {
                float r = a[w + (size_t)h * W] * kBlurW[0];
                for (int i = 1; i < 5; ++i)
                {
                    int h1 = std::min(H - 1, std::max(h + i, 0));
                    int h2 = std::min(H - 1, std::max(h - i, 0));
                    r += a[w + (size_t)h1 * W] * kBlurW[i];
                    r += a[w + (size_t)h2 * W] * kBlurW[i];
                }
                a[w + (size_t)h * W] = r;
            }
    });
}

// Ping-pong separable variant: same taps and order, every read from the
// previous sweep's values.
void blur_separable(Frame& F)
{
    const int W = F.W, H = F.H;
    std::vector<float> src = F.ao, tmp(F.ao.size());
    parallel_for(H, F.cfg.threads, [&](int ha, int hb) {
        for (int h = ha; h < hb; ++h)
            for (int w = 0; w < W; ++w)
            {
                float r = src[w + (size_t)h * W] * kBlurW[0];
                for (int i = 1; i < 5; ++i)
                {
                    r += src[std::min(W - 1, w + i) + (size_t)h * W] * kBlurW[i];
                    r += src[std::max(0, w - i) + (size_t)h * W] * kBlurW[i];
                }
                tmp[w + (size_t)h * W] = r;
            }
    });
    parallel_for(H, F.cfg.threads, [&](int ha, int hb) {
        for (int h = ha; h < hb; ++h)
            for (int w = 0; w < W; ++w)
            {
                float r = tmp[w + (size_t)h * W] * kBlurW[0];
                for (int i = 1; i < 5; ++i)
                {
                    r += tmp[w + (size_t)std::min(H - 1, h + i) * W] * kBlurW[i];
                    r += tmp[w + (size_t)std::max(0, h - i) * W] * kBlurW[i];
                }
                F.ao[w + (size_t)h * W] = r;
            }
    });
}

void lighting_pass(Frame& F)
{
    parallel_for(F.H, F.cfg.threads, [&](int ya, int yb) {
        for (int y = ya; y < yb; ++y)
            for (int x = 0; x < F.W; ++x)
            {
                size_t i = (size_t)x + (size_t)y * F.W;
                V3 pos = F.gPos[i], n = F.gNormal[i], l = F.gLndc[i], albedo = F.gAlbedo[i];
                V3 emissive = F.gEmissive[i], param = F.gParam[i];
                float type = F.type[i];
                param.x *= F.ao[i];
                V3 L = normalize(F.lightPos - pos);
                V3 Vd = normalize(F.eye - pos);
                float vis = 0.f;
                if (F.shadowOn) vis = shadow_visibility(F, l, n, L);
                V3 c;
                if (type < 0.5f) c = blinn_phong(F, L, Vd, n, vis, albedo, emissive, param, F.lightColor);
                else
                {
                    V3 Hd = normalize(L + Vd);
                    c = pbr(F, L, Vd, Hd, n, vis, albedo, emissive, param, F.lightColor);
                }
                F.frame[i] = c;
            }
    });
}

// ---- several lights (the batched renderer's lighting, include/fr_batch.h) ---------------
// The batch has no counterpart in the reference, which lights with one point light
// (render.cpp:74): for physically based materials it sums the lights' direct terms
// (the part of pbrshader.h:194-232 before the ambient term, each with its own
// light's shadow visibility) in light order and then adds ambient and emission and
// tone-maps once (pbrshader.h:234-253); Blinn-Phong materials are lit by light 0
// alone. When light 0 is a point light its light-space position is the G-buffer's
// (interpolated from the vertices); every other light, and a directional light 0,
// projects the pixel's world position with its own light-space matrix. A
// directional light's direction is normalised once, d / |d| in float.
V3 pbr_direct(const Frame& F, V3 L, V3 Vd, V3 Hd, V3 N, float vis, V3 al, float metal, float rough, V3 radiance)
{
    float NdotV = maxf(dot(N, Vd), 0.f);
    float NdotL = maxf(dot(N, L), 0.f);
    float NdotH = maxf(dot(N, Hd), 0.f);
    float HdotV = maxf(dot(Hd, Vd), 0.f);
    V3 F0 = v3(0.04f);
    F0 = lerp(metal, F0, al);
    float NDF = ggx(NdotH, rough);
    float G = schlick_ggx(NdotV, rough) * schlick_ggx(NdotL, rough);
    float om = maxf(1.f - HdotV, 0.f);
    V3 Fr = F0 + (v3(1.f) - F0) * std::pow(om, 5.f);
    V3 DGF = Fr * (NDF * G);
    float denom = 4 * NdotV * NdotL + 0.001f;
    V3 specular = divs(DGF, denom);
    V3 kd = v3(1.f) - Fr;
    kd = kd * (1.f - metal);
    V3 brdf = kd * al * kInvPi + specular;
    V3 Lo = brdf * radiance * NdotL;
    if (F.shadowOn)
    {
        float shadow = (1 - vis) * 0.6f;
        vis = 1 - shadow;
        Lo = Lo * vis;
    }
    return Lo;
}

V3 pbr_finish(V3 Lo, V3 al, V3 el, float ao)
{
    V3 color = Lo;
    V3 ambient = v3(0.3f) * al * ao;
    color = color + ambient;
    color = color + el;
    color = divv(color, color + v3(1.f));
    color = powv(color, kInvGamma);
    return clamp01(color);
}

struct LightFrame
{
    fr_light_desc d;
    Frame F;  // the light's shadow map and its sampling constants
};

void lighting_pass_lights(Frame& F, const std::vector<LightFrame>& lights)
{
    parallel_for(F.H, F.cfg.threads, [&](int ya, int yb) {
        for (int y = ya; y < yb; ++y)
            for (int x = 0; x < F.W; ++x)
            {
                size_t i = (size_t)x + (size_t)y * F.W;
                if (!(F.depth[i] < kMaxFloat))
                {
                    F.frame[i] = v3(0.f);  // no triangle: black
                    continue;
                }
                V3 pos = F.gPos[i], n = F.gNormal[i], albedo = F.gAlbedo[i], emissive = F.gEmissive[i];
                V3 param = F.gParam[i];
                param.x *= F.ao[i];
                V3 Vd = normalize(F.eye - pos);
                bool pbrMat = F.type[i] >= 0.5f;
                V3 al = powv(albedo, kGamma), el = powv(emissive, kGamma);
                V3 Lo = v3(0.f), c = v3(0.f);
                for (size_t k = 0; k < lights.size(); ++k)
                {
                    const LightFrame& LF = lights[k];
                    V3 lc{LF.d.color[0], LF.d.color[1], LF.d.color[2]};
                    V3 L;
                    if (LF.d.type == 0)
                        L = normalize(V3{LF.d.position[0], LF.d.position[1], LF.d.position[2]} - pos);
                    else
                    {
                        const float* d = LF.d.direction;
                        float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                        V3 u = len > 0.f ? V3{d[0] / len, d[1] / len, d[2] / len} : v3(0.f);
                        L = V3{-u.x, -u.y, -u.z};
                    }
                    float vis = 0.f;
                    if (F.shadowOn)
                    {
                        V3 l = F.gLndc[i];
                        if (k != 0 || lights[0].d.type != 0)
                        {
                            V4 q = mul(LF.F.L, V4{pos.x, pos.y, pos.z, 1.f});
                            l = V3{q.x / q.w, q.y / q.w, q.z / q.w};
                        }
                        vis = shadow_visibility(LF.F, l, n, L);
                    }
                    if (pbrMat)
                    {
                        V3 d = pbr_direct(F, L, Vd, normalize(L + Vd), n, vis, al, param.y, param.z, lc);
                        Lo = k == 0 ? d : Lo + d;
                    }
                    else if (k == 0)
                        c = blinn_phong(F, L, Vd, n, vis, albedo, emissive, param, lc);
                }
                F.frame[i] = pbrMat ? pbr_finish(Lo, al, el, param.x) : c;
            }
    });
}

// Light-space matrix of a light: a point light uses the reference's shadow frustum
// (render.cpp:73-78); a directional light looks at the origin from -direction * d,
// d = 2 extent + 10, with ortho +-extent, near 0.1, far 2 d.
M4 light_matrix(const fr_scene_view* S, const fr_light_desc& L)
{
    const fr_scene_info& I = S->info;
    if (L.type == 0)
    {
        float ratio = (float)I.width / I.height;
        M4 lview = look_at(V3{L.position[0], L.position[1], L.position[2]}, V3{0.f, 0.f, 0.f});
        M4 lproj = ortho(-3.f * ratio, 3.f * ratio, -3.f, 3.f, 0.1f, 20.f);
        return mul(lproj, lview);
    }
    float e = L.extent > 0.f ? L.extent : 6.f;
    float d = 2.f * e + 10.f;
    V3 eye{-L.direction[0] * d, -L.direction[1] * d, -L.direction[2] * d};
    M4 lview = look_at(eye, V3{0.f, 0.f, 0.f});
    M4 lproj = ortho(-e, e, -e, e, 0.1f, 2.f * d);
    return mul(lproj, lview);
}

void setup_frame(Frame& F, const fr_scene_view* S, const fr_oracle_config* cfg, const fr_frame_matrices* mats);
void run_frame(Frame& F, fr_oracle_out* out, std::chrono::steady_clock::time_point t0);
void finish_frame(Frame& F, fr_oracle_out* out, std::chrono::steady_clock::time_point t0);

}  // namespace

extern "C" {

int fr_oracle_matrices(const fr_scene_view* S, int32_t shadow_size, fr_frame_matrices* out)
{
    if (!S || !out) return -1;
    const fr_scene_info& I = S->info;
    std::memset(out, 0, sizeof *out);
    int W = I.ssaa_on ? I.width * I.ssaa_kernel : I.width;
    int H = I.ssaa_on ? I.height * I.ssaa_kernel : I.height;
    float ratio = (float)I.width / I.height;
    M4 view = look_at(V3{I.eye[0], I.eye[1], I.eye[2]}, V3{I.target[0], I.target[1], I.target[2]});
    M4 proj = I.perspective ? perspective(45.f, ratio, 0.01f, 20.f)
                            : ortho(-1.f * ratio, 1.f * ratio, -1.f, 1.f, 0.01f, 20.f);
    M4 vp = mul(proj, view);
    M4 lview = look_at(V3{I.light_pos[0], I.light_pos[1], I.light_pos[2]}, V3{0.f, 0.f, 0.f});
    M4 lproj = ortho(-3.0f * ratio, 3.0f * ratio, -3.0f, 3.0f, 0.1f, 20.f);
    M4 ls = mul(lproj, lview);
    int SW = shadow_size > 0 ? shadow_size : W, SH = shadow_size > 0 ? shadow_size : H;
    M4 vpm = viewport(W, H), svpm = viewport(SW, SH);
    std::memcpy(out->view, view.m, 64);
    std::memcpy(out->projection, proj.m, 64);
    std::memcpy(out->view_projection, vp.m, 64);
    std::memcpy(out->light_space, ls.m, 64);
    std::memcpy(out->viewport, vpm.m, 64);
    std::memcpy(out->shadow_viewport, svpm.m, 64);
    out->width = W, out->height = H, out->shadow_width = SW, out->shadow_height = SH;
    return 0;
}

int fr_oracle_render(const fr_scene_view* S, const fr_oracle_config* cfg, const fr_frame_matrices* mats,
                     fr_oracle_out* out)
{
    if (!S || !cfg || !out) return -1;
    auto t0 = std::chrono::steady_clock::now();
    Frame F;
    setup_frame(F, S, cfg, mats);
    run_frame(F, out, t0);
    return 0;
}

int fr_oracle_render_lights(const fr_scene_view* S, const fr_oracle_config* cfg, const fr_frame_matrices* view,
                            const float eye[3], const fr_light_desc* lights, int32_t nLights, fr_oracle_out* out,
                            float* const* shadows)
{
    if (!S || !cfg || !view || !eye || !lights || nLights < 1 || nLights > 4 || !out) return -1;
    if (!S->info.deferred) return -1;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<LightFrame> LF(nLights);
    for (int k = 0; k < nLights; ++k)
    {
        LF[k].d = lights[k];
        const int s = lights[k].shadow_size;
        fr_frame_matrices m = *view;
        M4 Lk = light_matrix(S, lights[k]);
        std::memcpy(m.light_space, Lk.m, 64);
        M4 sv = viewport(s, s);
        std::memcpy(m.shadow_viewport, sv.m, 64);
        m.shadow_width = m.shadow_height = s;
        setup_frame(LF[k].F, S, cfg, &m);
        if (LF[k].F.shadowOn) shadow_pass(LF[k].F);
        if (shadows && shadows[k]) std::memcpy(shadows[k], LF[k].F.shadow.data(), LF[k].F.shadow.size() * 4);
    }
    // the camera: light 0's light-space position in the G-buffer
    fr_frame_matrices m = *view;
    std::memcpy(m.light_space, LF[0].F.fm.light_space, 64);
    std::memcpy(m.shadow_viewport, LF[0].F.fm.shadow_viewport, 64);
    m.shadow_width = LF[0].F.SW, m.shadow_height = LF[0].F.SH;
    Frame F;
    setup_frame(F, S, cfg, &m);
    F.eye = V3{eye[0], eye[1], eye[2]};
    F.lightPos = V3{lights[0].position[0], lights[0].position[1], lights[0].position[2]};
    F.lightColor = V3{lights[0].color[0], lights[0].color[1], lights[0].color[2]};
    camera_pass(F);
    if (F.ssaoOn)
    {
        ssao_pass(F);
        if (cfg->blur_mode == 0) blur_reference(F);
        else if (cfg->blur_mode == 1) blur_separable(F);
    }
    lighting_pass_lights(F, LF);
    finish_frame(F, out, t0);
    return 0;
}

}  // extern "C"

namespace
{

void setup_frame(Frame& F, const fr_scene_view* S, const fr_oracle_config* cfg, const fr_frame_matrices* mats)
{
    F.S = S;
    F.cfg = *cfg;
    if (F.cfg.threads < 1) F.cfg.threads = 1;
    g_texWrap = cfg->texture_wrap;
    g_texLinear = cfg->texture_filter == 1;
    if (mats) F.fm = *mats;
    else fr_oracle_matrices(S, cfg->shadow_size, &F.fm);
    std::memcpy(F.V.m, F.fm.view, 64);
    std::memcpy(F.P.m, F.fm.projection, 64);
    std::memcpy(F.VP.m, F.fm.view_projection, 64);
    std::memcpy(F.L.m, F.fm.light_space, 64);
    std::memcpy(F.VPort.m, F.fm.viewport, 64);
    std::memcpy(F.SVPort.m, F.fm.shadow_viewport, 64);
    F.W = F.fm.width, F.H = F.fm.height, F.SW = F.fm.shadow_width, F.SH = F.fm.shadow_height;
    const fr_scene_info& I = S->info;
    F.shadowOn = I.shadow_on != 0;
    F.deferred = I.deferred != 0;
    F.ssaoOn = I.ssao_on != 0;
    F.ssaaOn = I.ssaa_on != 0;
    F.ssaaK = I.ssaa_kernel;
    F.eye = V3{I.eye[0], I.eye[1], I.eye[2]};
    F.lightPos = V3{I.light_pos[0], I.light_pos[1], I.light_pos[2]};
    F.lightColor = V3{I.light_color[0], I.light_color[1], I.light_color[2]};
    for (int m = 0; m < I.num_models; ++m)
    {
        const fr_model_view& mv = S->models[m];
        M4 M = model_matrix(V3{mv.position[0], mv.position[1], mv.position[2]}, mv.rotate_y, mv.scale);
        F.modelM.push_back(M);
        F.modelN.push_back(normal_matrix(M));
        F.modelLM.push_back(mul(F.L, M));
    }
    F.blocker.resize(2 * std::max(1, cfg->blocker_samples));
    F.pcf.resize(2 * std::max(1, cfg->pcf_samples));
    F.ssaoK.resize(3 * 16 * std::max(1, cfg->ssao_samples));
    fr_make_disk_table(FR_TABLE_SEED_BLOCKER, cfg->blocker_samples, F.blocker.data());
    fr_make_disk_table(FR_TABLE_SEED_PCF, cfg->pcf_samples, F.pcf.data());
    fr_make_ssao_table(cfg->ssao_samples, F.ssaoK.data());
}

void run_frame(Frame& F, fr_oracle_out* out, std::chrono::steady_clock::time_point t0)
{
    if (F.shadowOn) shadow_pass(F);
    camera_pass(F);
    if (F.deferred)
    {
        if (F.ssaoOn)
        {
            ssao_pass(F);
            if (F.cfg.blur_mode == 0) blur_reference(F);
            else if (F.cfg.blur_mode == 1) blur_separable(F);
        }
        lighting_pass(F);
    }
    finish_frame(F, out, t0);
}

// 8-bit frame, SSAA resolve and the copies into the caller's buffers.
void finish_frame(Frame& F, fr_oracle_out* out, std::chrono::steady_clock::time_point t0)
{
    const size_t P = (size_t)F.W * F.H;
    std::vector<uint8_t> img(P * 3);
    for (size_t i = 0; i < P; ++i)
    {
        img[3 * i] = (uint8_t)(F.frame[i].x * 254.99f);
        img[3 * i + 1] = (uint8_t)(F.frame[i].y * 254.99f);
        img[3 * i + 2] = (uint8_t)(F.frame[i].z * 254.99f);
    }
    std::vector<uint8_t> ssaa;
    if (F.ssaaOn)
    {
        int k = F.ssaaK, kk = k * k, ow = F.W / k, oh = F.H / k;
        ssaa.assign((size_t)ow * oh * 3, 0);
        for (int x = 0; x < ow; ++x)
            for (int y = 0; y < oh; ++y)
            {
                int R = 0, G = 0, B = 0;
                for (int i = 0; i < k; ++i)
                    for (int j = 0; j < k; ++j)
                    {
                        int xx = x * k + i, yy = y * k + j;
                        uint8_t r = 0, g = 0, b = 0;
                        if (xx < F.W && yy < F.H)
                        {
                            size_t q = ((size_t)xx + (size_t)yy * F.W) * 3;
                            r = img[q], g = img[q + 1], b = img[q + 2];
                        }
                        R += r, G += g, B += b;
                    }
                R = (int)(R / (float)kk);
                G = (int)(G / (float)kk);
                B = (int)(B / (float)kk);
                size_t o = ((size_t)x + (size_t)y * ow) * 3;
                ssaa[o] = (uint8_t)R, ssaa[o + 1] = (uint8_t)G, ssaa[o + 2] = (uint8_t)B;
            }
    }
    out->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    auto put3 = [&](float* dst, const std::vector<V3>& src) {
        if (!dst || src.empty()) return;
        std::memcpy(dst, src.data(), src.size() * sizeof(V3));
    };
    if (out->depth) std::memcpy(out->depth, F.depth.data(), P * 4);
    if (out->shadow && F.shadowOn) std::memcpy(out->shadow, F.shadow.data(), F.shadow.size() * 4);
    put3(out->gb_normal, F.gNormal);
    put3(out->gb_position, F.gPos);
    put3(out->gb_lightndc, F.gLndc);
    put3(out->gb_albedo, F.gAlbedo);
    put3(out->gb_emissive, F.gEmissive);
    put3(out->gb_param, F.gParam);
    if (out->gb_type && !F.type.empty()) std::memcpy(out->gb_type, F.type.data(), P * 4);
    if (out->ao && !F.ao.empty()) std::memcpy(out->ao, F.ao.data(), P * 4);
    put3(out->frame, F.frame);
    if (out->frame8) std::memcpy(out->frame8, img.data(), img.size());
    if (out->ssaa8 && !ssaa.empty()) std::memcpy(out->ssaa8, ssaa.data(), ssaa.size());
}

}  // namespace
