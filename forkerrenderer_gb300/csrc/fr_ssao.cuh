// SSAO sample projection: the reference's exact float arithmetic and a cheap
// estimate with a proven error bound (render.cpp:240-262).
//
// Per sample the reference computes the sample point s = pos + (+-o) (one
// rounding), the clip vector c = VP (s, 1) (per row three products and three
// sums, in order), n = c * RN(1 / c.w), and the viewport transform; the pixel
// (trunc x, trunc y) selects a depth and the z value is compared with it. Only
// the two truncations and the comparison see these values, so a sample whose
// estimate lies farther than the estimate's error bound from every integer
// (x, y) and from the comparison threshold (z) is decided by the estimate; the
// others run the exact arithmetic.
//
// Estimate: c' = P + (+-Q) with P = VP (pos, 1) per pixel and Q = VP (o, 0) per
// table entry (fused multiply-adds), n' = c' * rcp(c'.w) with an approximate
// reciprocal, e = fma(Vp_ii, n', Vp_i3).
//
// Bound (u = 2^-24, R >= |o_i|, S_i = |pos_i| + R, A_r = sum_i |VP_ri| S_i +
// |VP_r3|, and w_lo > 0 a lower bound of the exact and estimated c.w over every
// sample of the pixel): relative to the real-valued projection of the real
// sample point, the exact clip row is off by at most 5u A_r (two roundings in
// each product counting the sample point's, three in the sums), the estimate's
// by 8u A_r (P: 4u A_r, Q: 3u A_r, the fma: u A_r); the divisions add 2u
// (exact) and 5u (estimate, reciprocal within 2 ulp) relative, |n_r| <= nh_r =
// (|P_r| + R sum_i |VP_ri| + 2^-20 A_r) / w_lo, and the viewport sums 4u resp. u
// relative. So |exact - estimate| <= E = 14u |Vp_ii| (A_r + nh_r A_w) / w_lo +
// 11u (|Vp_ii| nh_r + |Vp_i3|) (ssao_bound). The kernel tests the estimate
// against twice that; since E >= 11u |e|, the rounded ends e -+ 2E still
// enclose the exact value. tests/cpp/test_ssao.cpp checks the bound on random
// matrices, points and samples against the exact arithmetic, with the
// reciprocal pushed 2 ulp either way.
#pragma once

#include "fr_exact.cuh"

namespace frx
{

// The exact projection (the reference's operation order): the viewport-space
// x, y, z of sample point pos + sg * o, sg = +-1. simple: the viewport has the
// SetViewportMatrix zero pattern; the result is then Vp_ii n_i + Vp_i3 n_w
// (the zero entries add exact +-0 terms to finite values).
struct SsaoProj
{
    float x, y, z;
    bool simple;  // the simple form was taken (all of n finite)
};

FR_HD float fmul_x(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

FR_HD float fadd_x(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

FR_HD float fabs_x(float a) { return a < 0.f ? -a : a; }

FR_HD SsaoProj ssao_project(const float* M, const float* Vp, bool vportSimple, float px, float py, float pz,
                            float sg, float ox, float oy, float oz)
{
    // pos + (sg * o) rounded once: sg * o is exact, so the fused form is that sum
    const float sx = ffma(sg, ox, px), sy = ffma(sg, oy, py), sz = ffma(sg, oz, pz);
    float c[4];
    for (int r = 0; r < 4; ++r)
        c[r] = fadd_x(fadd_x(fadd_x(fmul_x(M[4 * r], sx), fmul_x(M[4 * r + 1], sy)), fmul_x(M[4 * r + 2], sz)),
                      M[4 * r + 3]);
    const float inv = frcp_rn(c[3]);
    const float nx = fmul_x(c[0], inv), ny = fmul_x(c[1], inv), nz = fmul_x(c[2], inv), nw = fmul_x(c[3], inv);
    const float sum = fadd_x(fadd_x(nx, ny), fadd_x(nz, nw));
    SsaoProj o;
    o.simple = vportSimple && fabs_x(sum) < bitsf(0x7f800000u);  // all four finite (else the sum is inf or NaN)
    if (o.simple)
    {
        o.x = fadd_x(fmul_x(Vp[0], nx), fmul_x(Vp[3], nw));
        o.y = fadd_x(fmul_x(Vp[5], ny), fmul_x(Vp[7], nw));
        o.z = fadd_x(fmul_x(Vp[10], nz), fmul_x(Vp[11], nw));
    }
    else
    {
        const float n[4] = {nx, ny, nz, nw};
        float v[3];
        for (int r = 0; r < 3; ++r)
            v[r] = fadd_x(fadd_x(fadd_x(fadd_x(0.f, fmul_x(Vp[4 * r], n[0])), fmul_x(Vp[4 * r + 1], n[1])),
                                 fmul_x(Vp[4 * r + 2], n[2])),
                          fmul_x(Vp[4 * r + 3], n[3]));
        o.x = v[0], o.y = v[1], o.z = v[2];
    }
    return o;
}

// Per-pixel part of the estimate: P = VP (pos, 1) and the test half-widths
// d = 2E of x, y, z; ok = false where the bound does not hold or is useless
// (c.w not bounded away from 0, a non-simple viewport, non-finite values, or
// half-widths beyond a quarter pixel), and every sample then runs exactly.
struct SsaoPlane
{
    float P[4];
    float dx, dy, dz;
    bool ok;
};

// The bound's E for one viewport axis: Vii, Vi3 the viewport entries, A_r and
// nh_r of the axis' clip row, A_w of the w row.
FR_HD float ssao_bound(float Vii, float Vi3, float Ar, float nh, float Aw, float wlo)
{
    const float u = 5.9604644775390625e-08f;  // 2^-24
    const float a = fabs_x(Vii), b = fabs_x(Vi3);
    return (14.f * u) * a * ((Ar + nh * Aw) / wlo) + (11.f * u) * (a * nh + b);
}

FR_HD SsaoPlane ssao_plane(const float* M, const float* Vp, bool vportSimple, float radius, float px, float py,
                           float pz)
{
    const float up = 1.f + 9.5367431640625e-07f;  // 1 + 2^-20: rounds each bound term up past its own roundings
    const float R = fabs_x(radius) * up;
    const float S[3] = {(fabs_x(px) + R) * up, (fabs_x(py) + R) * up, (fabs_x(pz) + R) * up};
    SsaoPlane q;
    float A[4], G[4];
    for (int r = 0; r < 4; ++r)
    {
        const float* m = M + 4 * r;
        q.P[r] = ffma(m[2], pz, ffma(m[1], py, ffma(m[0], px, m[3])));
        A[r] = ((fabs_x(m[0]) * S[0] + fabs_x(m[1]) * S[1]) + fabs_x(m[2]) * S[2] + fabs_x(m[3])) * up * up;
        G[r] = ((fabs_x(m[0]) + fabs_x(m[1])) + fabs_x(m[2])) * R * up * up;
    }
    const float e20 = 9.5367431640625e-07f;  // 2^-20
    const float wlo = (q.P[3] - G[3] - e20 * A[3]) * (1.f - e20);
    float nh[3];
    for (int r = 0; r < 3; ++r) nh[r] = (fabs_x(q.P[r]) + G[r] + e20 * A[r]) / wlo * up;
    q.dx = 2.f * ssao_bound(Vp[0], Vp[3], A[0], nh[0], A[3], wlo) * up;
    q.dy = 2.f * ssao_bound(Vp[5], Vp[7], A[1], nh[1], A[3], wlo) * up;
    q.dz = 2.f * ssao_bound(Vp[10], Vp[11], A[2], nh[2], A[3], wlo) * up;
    // wlo >= 2^-64 keeps every estimated c.w normal (the approximate reciprocal
    // flushes subnormals); the comparisons are false for NaN
    q.ok = vportSimple && wlo >= 5.421010862427522e-20f && q.dx <= 0.25f && q.dy <= 0.25f && q.dz <= 1e30f;
    return q;
}

// Per-table-entry part: Q = VP (o, 0), rows x, y, z, w.
FR_HD void ssao_q(const float* M, float ox, float oy, float oz, float* Q)
{
    for (int r = 0; r < 4; ++r) Q[r] = ffma(M[4 * r + 2], oz, ffma(M[4 * r + 1], oy, fmul_x(M[4 * r], ox)));
}

}  // namespace frx
