// Host-side float math with the reference's exact operation order.
//
// The reference computes its matrices on the CPU in float with a fixed
// evaluation order: Dot() accumulates from 0.f left to right (src/geometry.h:881-889),
// matrix products are row x column Dots (geometry.h:784-793), Vector / f
// multiplies by 1/f (geometry.h:176-182), Normalize(v) = v * (1 / |v|)
// (geometry.h:906-910). Results only match bit for bit if this file is
// compiled without floating-point contraction (-ffp-contract=off), which the
// build does for every host translation unit.
#pragma once

#include <cmath>
#include <cstring>

namespace fr
{

struct V3
{
    float x, y, z;
};

struct M4
{
    float m[4][4];
    static M4 identity()
    {
        M4 r;
        std::memset(&r, 0, sizeof r);
        for (int i = 0; i < 4; ++i) r.m[i][i] = 1.f;
        return r;
    }
};

inline float dot3(V3 a, V3 b)
{
    float r = 0.f;
    r += a.x * b.x;
    r += a.y * b.y;
    r += a.z * b.z;
    return r;
}

inline float length3(V3 v)
{
    return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
}

inline V3 scale3(V3 v, float f) { return V3{v.x * f, v.y * f, v.z * f}; }
inline V3 sub3(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add3(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }

// Vector / f  (geometry.h:176-182): multiply by the float reciprocal.
inline V3 div3(V3 v, float f)
{
    float inv = 1.f / f;
    return V3{v.x * inv, v.y * inv, v.z * inv};
}

inline V3 normalize3(V3 v) { return div3(v, length3(v)); }

inline V3 cross3(V3 a, V3 b)
{
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
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

// Radians (src/utility.h:51-54) with Pi as the float constant of constant.h:20.
inline float radians(float deg)
{
    const float Pi = 3.14159265358979323846f;
    return deg * Pi / 180.f;
}

// MakeModelMatrix (geometry.cpp:92-108): T * R_y * S. cos/sin are the double
// library functions on the float angle, as the reference's unqualified calls
// resolve, rounded back to float.
inline M4 make_model(V3 t, float yrot, float scale)
{
    M4 S = M4::identity();
    S.m[0][0] = S.m[1][1] = S.m[2][2] = scale;
    M4 R = M4::identity();
    float rad = radians(yrot);
    double c = std::cos((double)rad), s = std::sin((double)rad);
    R.m[0][0] = (float)c;
    R.m[0][2] = (float)s;
    R.m[2][0] = (float)(-s);
    R.m[2][2] = (float)c;
    M4 T = M4::identity();
    T.m[0][3] = t.x;
    T.m[1][3] = t.y;
    T.m[2][3] = t.z;
    return mul(mul(T, R), S);
}

// MakeLookAtMatrix (geometry.cpp:110-128), world up (0, 1, 0).
inline M4 make_look_at(V3 eye, V3 center)
{
    V3 up{0.f, 1.f, 0.f};
    V3 front = normalize3(sub3(center, eye));
    V3 right = normalize3(cross3(front, up));
    V3 up2 = normalize3(cross3(right, front));
    M4 R = M4::identity();
    R.m[0][0] = right.x, R.m[0][1] = right.y, R.m[0][2] = right.z, R.m[0][3] = 0.f;
    R.m[1][0] = up2.x, R.m[1][1] = up2.y, R.m[1][2] = up2.z, R.m[1][3] = 0.f;
    R.m[2][0] = -front.x, R.m[2][1] = -front.y, R.m[2][2] = -front.z, R.m[2][3] = 0.f;
    M4 T = M4::identity();
    T.m[0][3] = -eye.x;
    T.m[1][3] = -eye.y;
    T.m[2][3] = -eye.z;
    return mul(R, T);
}

// MakePerspectiveMatrix(fov, aspect, n, f) (geometry.cpp:130-145). Starts from
// the identity, so m[3][3] stays 1: w_clip = 1 - z_view.
inline M4 make_perspective(float fov, float aspect, float n, float f)
{
    float t = std::tan(radians(fov / 2.f));
    M4 m = M4::identity();
    m.m[0][0] = 1.f / (aspect * t);
    m.m[1][1] = 1.f / t;
    m.m[2][2] = -(f + n) / (f - n);
    m.m[2][3] = -2 * f * n / (f - n);
    m.m[3][2] = -1;
    return m;
}

// MakeOrthographicMatrix (geometry.cpp:166-179).
inline M4 make_ortho(float l, float r, float b, float t, float n, float f)
{
    M4 m = M4::identity();
    m.m[0][0] = 2.f / (r - l);
    m.m[1][1] = 2.f / (t - b);
    m.m[2][2] = -2.f / (f - n);
    m.m[0][3] = -(r + l) / (r - l);
    m.m[1][3] = -(t + b) / (t - b);
    m.m[2][3] = -(f + n) / (f - n);
    m.m[3][3] = 1.f;
    return m;
}

// ForkerGL::SetViewportMatrix(0, 0, w, h) (forkergl.cpp:89-102).
inline M4 make_viewport(int w, int h)
{
    M4 m = M4::identity();
    m.m[0][0] = w / 2.f;
    m.m[1][1] = h / 2.f;
    m.m[0][3] = 0 + w / 2.f;
    m.m[1][3] = 0 + h / 2.f;
    m.m[2][2] = 1 / 2.f;
    m.m[2][3] = 1 / 2.f;
    return m;
}

// Determinant / cofactors by first-row expansion (geometry.h:605-624, 705-732).
template <int N>
struct Det
{
    static float det(const float (*a)[4])
    {
        float ret = 0;
        for (int i = 0; i < N; ++i) ret += a[0][i] * cofactor(a, 0, i);
        return ret;
    }
    static float cofactor(const float (*a)[4], int row, int col)
    {
        float minor[4][4] = {};
        for (int i = 0; i < N - 1; ++i)
            for (int j = 0; j < N - 1; ++j)
                minor[i][j] = a[i < row ? i : i + 1][j < col ? j : j + 1];
        return Det<N - 1>::det(minor) * ((row + col) % 2 ? -1 : 1);
    }
};
template <>
struct Det<1>
{
    static float det(const float (*a)[4]) { return a[0][0]; }
};

// MakeNormalMatrix (geometry.cpp:60-68): upper 3x3 of Inverse().Transpose(),
// with Inverse() = Adjugate() / Det() (geometry.h:723-732). Row major 3x3.
inline void make_normal_matrix(const M4& M, float out[9])
{
    float adjT[4][4];  // Adjugate(): cofactor matrix transposed
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) adjT[j][i] = Det<4>::cofactor(M.m, i, j);
    float d = Det<4>::det(M.m);
    float inv = 1.f / d;  // Matrix / scalar divides each row Vector (geometry.h:360-365)
    float invm[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) invm[i][j] = adjT[i][j] * inv;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[r * 3 + c] = invm[c][r];  // Transpose()
}

}  // namespace fr
