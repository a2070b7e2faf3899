// Bit-exact barycentric coordinates and depth of the reference rasteriser.
//
// The reference evaluates Barycentric (src/geometry.cpp:20-56) at every pixel of
// a triangle's clamped bounding box: float copies of the int-snapped vertices,
// float differences widened to double, a double cross product, then
//     inv = 1.0 / bz;  u = bx * inv;  v = by * inv;
//     result = float3(float(1.0 - (u + v)), float(u), float(v))
// rejecting the pixel if any component is negative, and the depth
// Dot(bary, depths) in float (forkergl.cpp:173-184).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so this file
// reaches the same float results without FP64 on almost every pixel:
//   * When all vertex coordinates lie in [-2^23, 2^23], every difference is an
//     exact integer below 2^24, so the double cross product is exact: bx, by, bz
//     are the integer edge functions (int64 here). Coverage u >= 0, v >= 0 is the
//     exact sign test, and w = (bz - bx - by) / bz >= 0 is exact unless
//     bz - bx - by == 0.
//   * If moreover |bz| < 2^24, float(u) == RN_float(bx / bz): u_double carries a
//     relative error below 2^-52, while a quotient of integers below 2^24 is at
//     relative distance >= 2^-49 from every float rounding boundary (and never
//     on one). So u and v are single correctly rounded float divisions.
//   * For w, the double path's absolute error is below 2^-51 (two products,
//     a sum, a subtraction). The float candidate RN_float(c / bz) is accepted
//     when an exact integer remainder shows the quotient is farther than that
//     from the float rounding boundary (w_fast); otherwise, and when c == 0,
//     the double path is evaluated as the reference does. The test is
//     conservative, never approximate.
//   * Triangles outside these bounds use the reference's double arithmetic
//     per pixel (bary_reference).
// Host builds of this header (tests) use the same code with IEEE float/double
// arithmetic; every translation unit is compiled without FP contraction.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define FR_HD __host__ __device__ __forceinline__
#else
#define FR_HD inline
#include <cmath>
#endif

namespace frx
{

constexpr int kCoordLimit = 1 << 23;
constexpr long long kBzFastLimit = 1ll << 24;
// Triangles and pixels within +-kSmallLimit: every edge-function factor is below
// 2^15 in magnitude, so products stay below 2^30 and their differences inside int32.
constexpr int kSmallLimit = 16383;

// Triangle classes for rasterisation.
enum TriClass : int
{
    kTriEmpty = 0,      // never covers a pixel (bz == 0 / |bz| <= 1e-2)
    kTriFast = 1,       // integer edges, float divisions
    kTriIntDouble = 2,  // integer coverage, double values (|bz| >= 2^24)
    kTriReference = 3   // reference double arithmetic per pixel
};

FR_HD int f2i_sat(float f)
{
#ifdef __CUDA_ARCH__
    return __float2int_rz(f);  // saturating, NaN -> 0
#else
    if (!(f == f)) return 0;
    if (f >= 2147483648.f) return 2147483647;
    if (f < -2147483648.f) return (-2147483647 - 1);
    return (int)f;
#endif
}

FR_HD float fdiv_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

FR_HD float frcp_rn(float b)
{
#ifdef __CUDA_ARCH__
    return __frcp_rn(b);
#else
    return 1.0f / b;
#endif
}

FR_HD float ffma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// RN(a / b) from y = RN(1 / b): q0 = RN(a y), r = a - q0 b (exact by FMA),
// q = RN(q0 + r y) (Markstein). Exact for the integer operands below 2^24 used
// here (no overflow or underflow); checked exhaustively / on 2.4e8 random pairs
// in tests/cpp/test_exact.cpp.
FR_HD float fdiv_y(float a, float b, float y)
{
#ifdef __CUDA_ARCH__
    float q0 = __fmul_rn(a, y);
#else
    float q0 = a * y;
#endif
    float r = ffma(-q0, b, a);
    return ffma(r, y, q0);
}

FR_HD int clz64(unsigned long long v)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return __builtin_clzll(v);
#endif
}

FR_HD unsigned int fbits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned int u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}

FR_HD float bitsf(unsigned int u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}

// Per-triangle raster setup: int-snapped screen vertices and viewport depths.
struct RTri
{
    int x[3], y[3];
    float d[3];
    int cls;
    float fbz;                // (float)bz (class kTriFast: exact, |bz| < 2^24)
    float rbz;                // RN(1 / bz) (class kTriFast)
    int s53;                  // RN53(1 / |bz|) = m53 * 2^-s53 (class kTriFast)
    int small;                // all coordinates within +-kSmallLimit: edge functions fit int32
    long long bz;             // integer edge determinant (classes kTriFast / kTriIntDouble)
    unsigned long long m53;
};

FR_HD bool coords_in_range(const int* X, const int* Y)
{
    for (int k = 0; k < 3; ++k)
        if (X[k] < -kCoordLimit || X[k] > kCoordLimit || Y[k] < -kCoordLimit || Y[k] > kCoordLimit)
            return false;
    return true;
}

// The reference's double determinant (geometry.cpp:31-39) for any coordinates.
FR_HD double bz_reference(const int* X, const int* Y)
{
    float ax = (float)X[0], ay = (float)Y[0], bx = (float)X[1], by = (float)Y[1];
    float cx = (float)X[2], cy = (float)Y[2];
    double s0x = bx - ax, s0y = cx - ax, s1x = by - ay, s1y = cy - ay;
    return s0x * s1y - s0y * s1x;
}

FR_HD void recip53(unsigned long long B, unsigned long long& M, int& S);

FR_HD void classify(RTri& t, bool withRecip = true)
{
    if (coords_in_range(t.x, t.y))
    {
        long long bz = (long long)(t.x[1] - t.x[0]) * (t.y[2] - t.y[0]) -
                       (long long)(t.x[2] - t.x[0]) * (t.y[1] - t.y[0]);
        t.bz = bz;
        if (bz == 0) t.cls = kTriEmpty;
        else if (bz > -kBzFastLimit && bz < kBzFastLimit) t.cls = kTriFast;
        else t.cls = kTriIntDouble;
        t.fbz = (float)(int)(t.cls == kTriFast ? bz : 0);
        t.rbz = t.cls == kTriFast ? frcp_rn(t.fbz) : 0.f;
        t.m53 = 0, t.s53 = 0;
        if (t.cls == kTriFast && withRecip) recip53((unsigned long long)(bz < 0 ? -bz : bz), t.m53, t.s53);
        t.small = 1;
        for (int k = 0; k < 3; ++k)
            if (t.x[k] < -kSmallLimit || t.x[k] > kSmallLimit || t.y[k] < -kSmallLimit || t.y[k] > kSmallLimit)
                t.small = 0;
    }
    else
    {
        t.bz = 0;
        t.fbz = 0.f;
        t.rbz = 0.f;
        t.m53 = 0, t.s53 = 0;
        t.small = 0;
        double bzd = bz_reference(t.x, t.y);
        t.cls = (bzd > 1e-2 || bzd < -1e-2) ? kTriReference : kTriEmpty;
    }
}

// Literal reference Barycentric for any coordinates (geometry.cpp:20-56).
FR_HD bool bary_reference(const int* X, const int* Y, int px, int py, float& b0, float& b1, float& b2)
{
    float ax = (float)X[0], ay = (float)Y[0], bx = (float)X[1], by = (float)Y[1];
    float cx = (float)X[2], cy = (float)Y[2], fx = (float)px, fy = (float)py;
    double s0x = bx - ax, s0y = cx - ax, s0z = ax - fx;
    double s1x = by - ay, s1y = cy - ay, s1z = ay - fy;
    double X_ = s0y * s1z - s0z * s1y;
    double Y_ = s0z * s1x - s0x * s1z;
    double Z_ = s0x * s1y - s0y * s1x;
    if (!(Z_ > 1e-2 || Z_ < -1e-2)) return false;
    double inv = 1.0 / Z_;
    X_ *= inv;
    Y_ *= inv;
    float r0 = (float)(1.0 - (X_ + Y_)), r1 = (float)X_, r2 = (float)Y_;
    if (r0 < 0.f || r1 < 0.f || r2 < 0.f) return false;
    b0 = r0, b1 = r1, b2 = r2;
    return true;
}

// Double-path weights from exact integer edge values (|ex|,|ey|,|bz| < 2^53).
FR_HD bool bary_from_ints_double(long long ex, long long ey, long long bz, float& b0, float& b1,
                                 float& b2)
{
    double inv = 1.0 / (double)bz;
    double u = (double)ex * inv, v = (double)ey * inv;
    float r0 = (float)(1.0 - (u + v)), r1 = (float)u, r2 = (float)v;
    if (r0 < 0.f || r1 < 0.f || r2 < 0.f) return false;
    b0 = r0, b1 = r1, b2 = r2;
    return true;
}

// float(1 - (u + v)) of the double path for a covered fast-class pixel with
// integer numerator c = bz - ex - ey != 0 (so 0 < c / bz <= 1, |bz| < 2^24).
// q = RN_float(c / bz) equals the double path's result unless the quotient lies
// within E = 2^-51 (the double path's absolute error: two products, a sum and a
// subtraction, 0.875 * 2^-51 at most) of the float rounding boundary on its side
// of q, at distance h (half the float spacing there). With the exact remainder
// r = c - q bz (one FMA), the quotient is safe when |r| < (h - E) |bz|. The test
// uses T = h - m g, the largest float <= h - E on the grid g = h 2^-24
// (m = max(1, E / g)), and the sign of fma(|bz|, -T, |r|), which is exact.
FR_HD bool w_fast(float fc, float fbz, float rbz, float& w)
{
    float q = fdiv_y(fc, fbz, rbz);
    float r = ffma(-q, fbz, fc);
    unsigned int qb = fbits(q);
    unsigned int e = qb >> 23;  // q in [2^-24, 1]: e in [103, 127]
    bool below = (r != 0.f) && ((r > 0.f) != (fbz > 0.f));
    bool pow2 = (qb & 0x7fffffu) == 0u;
    // h = ulp(q) / 2 (/ 4 below a power of two); g = h * 2^-24
    unsigned int he = e - 24u - ((below && pow2) ? 1u : 0u);  // exponent of h
    float g = bitsf((he - 24u) << 23);
    int mexp = 76 - (int)(he - 24u);                         // log2(E / g) = -51 - log2(g)
    float m = mexp <= 0 ? 1.f : bitsf((unsigned)(127 + mexp) << 23);
    float T = (16777216.f - m) * g;                          // exact: integer < 2^24 times 2^k
    float az = fbz < 0.f ? -fbz : fbz, ar = r < 0.f ? -r : r;
    w = q;
    return ffma(az, -T, ar) < 0.f;
}

// RN53(1 / B) = M * 2^-S for an integer 1 <= B < 2^24 (M < 2^53), exactly and
// without division instructions: the float reciprocal gives Q0 within 2^29 of
// floor(2^S / B); two float-estimated corrections and a final +-1 step make the
// remainder R = 2^S - Q B land in [0, B) (R is exact in wrapped 64-bit
// arithmetic because |R| < 2^62), then Q is rounded to nearest even.
FR_HD void recip53(unsigned long long B, unsigned long long& M, int& S)
{
    int k = 63 - clz64(B);  // 2^k <= B < 2^(k+1)
    if ((B & (B - 1ull)) == 0ull)
    {
        M = 1ull << 52;
        S = 52 + k;
        return;
    }
    S = 53 + k;  // 2^S / B in (2^52, 2^53)
    float y = frcp_rn((float)(unsigned)B);
    unsigned yb = fbits(y);
    unsigned long long my = (unsigned long long)((yb & 0x7fffffu) | 0x800000u);
    int sh = S + (int)((yb >> 23) & 0xffu) - 150;  // y = my * 2^(e-150): 2^S y = my * 2^sh
    long long Q = (long long)(my << sh);
    unsigned long long twoS = S >= 64 ? 0ull : (1ull << S);
    long long R = (long long)(twoS - (unsigned long long)Q * B);
    for (int it = 0; it < 2; ++it)
    {
        // dq ~ R / B from the float reciprocal (R split into exact int32 halves)
        float fr = (float)(int)(R >> 24) * 16777216.0f + (float)(int)(R & 0xffffffll);
        long long dq = (long long)(int)floorf(fr * y);
        Q += dq;
        R -= dq * (long long)B;
    }
    while (R < 0)
    {
        --Q;
        R += (long long)B;
    }
    while (R >= (long long)B)
    {
        ++Q;
        R -= (long long)B;
    }
    if (2 * R > (long long)B || (2 * R == (long long)B && (Q & 1ll))) ++Q;
    if (Q == (1ll << 53))
    {
        Q = 1ll << 52;
        S -= 1;
    }
    M = (unsigned long long)Q;
}

// Rounding error RN53(P) - P of P = a * M, for 0 <= a < 2^24 and 2^52 < M < 2^53
// (P < 2^77), in integers: the k = bitlength(P) - 53 <= 24 low bits of P are
// rounded away (to nearest, ties to even), and they are the low bits of a * (M mod
// 2^24), so two 32 x 32 -> 64-bit products suffice.
FR_HD long long rn53_error(unsigned a, unsigned long long M)
{
    if (a == 0u) return 0;
    const unsigned long long lo = (unsigned long long)a * (M & 0xffffffull);  // < 2^48
    const unsigned long long hi = (unsigned long long)a * (M >> 24) + (lo >> 24);  // P >> 24 (< 2^54)
    const int k = (64 - clz64(hi)) + 24 - 53;
    if (k <= 0) return 0;
    const unsigned long long mask = (1ull << k) - 1ull, low = lo & mask, half = 1ull << (k - 1);
    const unsigned long long lsb = k < 24 ? (lo >> k) & 1ull : hi & 1ull;  // bit k of P
    return (low > half || (low == half && lsb)) ? (long long)(mask + 1ull - low) : -(long long)low;
}

// float(1 - (u + v)) of the double path for a covered pixel with c == 0, i.e.
// u + v == 1 exactly (every triangle's vertex B and C pixels, lattice points of
// edge BC). The sign of this tiny value decides coverage, so it is reproduced
// exactly, in integers (no FP64 instruction). With a = |ex|, b = |ey|, a + b = |bz|
// = B and inv = RN53(1 / B) = M * 2^-S: u = RN53(a M) 2^-S, v = RN53(b M) 2^-S,
// so u + v = 1 + T 2^-S exactly, where T = (B M - 2^S) + the two rounding errors
// (|T| < 3 B, a small integer). s = RN53(u + v) lies on the grid 2^-52 above 1
// and 2^-53 below it, and w = 1 - s is exact (Sterbenz): -round(T / 2^(S-52)) 2^-52
// for T >= 0, round(-T / 2^(S-53)) 2^-53 otherwise (ties to even significands).
FR_HD float w_on_edge(unsigned a, unsigned b, unsigned long long M, int S)
{
    const unsigned long long twoS = S >= 64 ? 0ull : (1ull << S);
    // B M - 2^S in wrapped 64-bit arithmetic: exact, |B M - 2^S| <= B / 2
    const long long e = (long long)((unsigned long long)(a + b) * M - twoS);
    const long long T = e + rn53_error(a, M) + rn53_error(b, M);
    const bool above = T >= 0;
    const unsigned long long x = (unsigned long long)(above ? T : -T);
    const int sh = above ? S - 52 : S - 53;  // >= 0
    unsigned long long j = x >> sh;
    if (sh > 0)
    {
        const unsigned long long rem = x & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (j & 1ull))) ++j;
    }
    const int n = above ? -(int)j : (int)j;  // w = n * 2^-52 (above) or n * 2^-53
    return (float)n * (above ? 2.22044604925031308085e-16f : 1.11022302462515654042e-16f);
}

// Sign of a zero edge value as the reference's double cross product yields it:
// p1 - p2 with p1 = a1 * b1, p2 = a2 * b2 (exact integer-valued factors) is -0
// only when p1 is -0 and p2 is +0. The sign carries into u = bx * inv and only
// ever shows as the sign of a zero weight.
FR_HD bool neg_zero_product(long long a, long long b) { return (a == 0 && b < 0) || (b == 0 && a < 0); }
FR_HD bool ref_edge_neg_zero(long long a1, long long b1, long long a2, long long b2)
{
    bool p1neg = neg_zero_product(a1, b1);
    bool p2pos = (a2 == 0 || b2 == 0) && !neg_zero_product(a2, b2);
    return p1neg && p2pos;
}

FR_HD bool neg_zero_product32(int a, int b) { return (a == 0 && b < 0) || (b == 0 && a < 0); }
FR_HD bool ref_edge_neg_zero32(int a1, int b1, int a2, int b2)
{
    return neg_zero_product32(a1, b1) && (a2 == 0 || b2 == 0) && !neg_zero_product32(a2, b2);
}

FR_HD float signed_zero(bool negative) { return negative ? -0.f : 0.f; }

// Cheap conservative pre-test for a fast-class triangle: false only if the
// pixel is certainly rejected (a strict sign violation of an exact edge value);
// pixels with c == 0 pass and are decided by bary().
FR_HD bool small_pixel(int px, int py)
{
    return px >= -kSmallLimit && px <= kSmallLimit && py >= -kSmallLimit && py <= kSmallLimit;
}

FR_HD bool maybe_covered(const RTri& t, int px, int py)
{
    if (t.small && small_pixel(px, py))
    {
        const int ex = (t.x[2] - t.x[0]) * (t.y[0] - py) - (t.x[0] - px) * (t.y[2] - t.y[0]);
        const int ey = (t.x[0] - px) * (t.y[1] - t.y[0]) - (t.x[1] - t.x[0]) * (t.y[0] - py);
        if (t.bz > 0) return ex >= 0 && ey >= 0 && (long long)ex + ey <= t.bz;
        return ex <= 0 && ey <= 0 && (long long)ex + ey >= t.bz;
    }
    long long s0x = t.x[1] - t.x[0], s0y = t.x[2] - t.x[0], s0z = t.x[0] - px;
    long long s1x = t.y[1] - t.y[0], s1y = t.y[2] - t.y[0], s1z = t.y[0] - py;
    long long ex = s0y * s1z - s0z * s1y, ey = s0z * s1x - s0x * s1z;
    bool pos = t.bz > 0;
    if (ex != 0 && ((ex > 0) != pos)) return false;
    if (ey != 0 && ((ey > 0) != pos)) return false;
    long long c = t.bz - ex - ey;
    return c == 0 || ((c > 0) == pos);
}

// maybe_covered for the setup kernel's queues: 0 = certainly rejected, 1 =
// maybe covered, 2 = maybe covered on edge BC (c == 0, small path): bary() of
// kind 2 pixels takes the on-edge weight, of kind 1 pixels never does.
FR_HD int pretest_kind(const RTri& t, int px, int py)
{
    if (t.small && small_pixel(px, py))
    {
        const int ex = (t.x[2] - t.x[0]) * (t.y[0] - py) - (t.x[0] - px) * (t.y[2] - t.y[0]);
        const int ey = (t.x[0] - px) * (t.y[1] - t.y[0]) - (t.x[1] - t.x[0]) * (t.y[0] - py);
        const long long c = t.bz - ex - ey;
        const bool ok = t.bz > 0 ? (ex >= 0 && ey >= 0 && c >= 0) : (ex <= 0 && ey <= 0 && c <= 0);
        return ok ? (c == 0 ? 2 : 1) : 0;
    }
    return maybe_covered(t, px, py) ? 1 : 0;
}

// Exact coverage + barycentric for one pixel, bit-identical to Barycentric()
// including the sign of zero weights. Returns false if the reference rejects
// the pixel.
// bary() of a fast-class triangle (|bz| < 2^24) with every coordinate and the
// pixel within +-kSmallLimit: the same values, with every edge value and test in
// int32 (the common case of the raster and resolve kernels).
// kOnly: 0 = any pixel, 1 = pixels off edge BC (c != 0), 2 = pixels on it (c == 0);
// a pixel of the other kind is handed to the general form (it does not happen
// when the kind comes from pretest_kind), so each form carries one weight path.
// kZeroSigns: reproduce the sign of zero weights too. Every consumer of the
// weights (Dot from 0.f for depth and varyings, sign tests for coverage) gives the
// same bits whatever the sign of a zero weight: a sum that starts at +0 stays +0
// while its terms are zero (+0 + -0 = +0) and is unchanged by a zero term once it
// is not, and -0 < 0 is false. The raster and resolve kernels therefore skip the
// fix-ups (false); tests/cpp/test_exact.cpp checks both the weights (true) and
// the consumers' results (false) against the reference's double arithmetic.
template <int kOnly = 0, bool kZeroSigns = true>
FR_HD bool bary_small(const RTri& t, int px, int py, float& b0, float& b1, float& b2)
{
    const int s0x = t.x[1] - t.x[0], s0y = t.x[2] - t.x[0], s0z = t.x[0] - px;
    const int s1x = t.y[1] - t.y[0], s1y = t.y[2] - t.y[0], s1z = t.y[0] - py;
    const int ex = s0y * s1z - s0z * s1y, ey = s0z * s1x - s0x * s1z;
    const int bz = (int)t.bz;
    const bool pos = bz > 0;
    // a nonzero edge value of the wrong sign rejects the pixel, and so does one
    // beyond bz (c = bz - ex - ey then has the wrong sign)
    if (pos ? (ex < 0 || ey < 0 || ex > bz || ey > bz) : (ex > 0 || ey > 0 || ex < bz || ey < bz)) return false;
    const int c = bz - ex - ey;  // |bz - ex| <= |bz| and |ey| <= |bz| < 2^24: no overflow
    if (c != 0 && ((c > 0) != pos)) return false;
    if ((kOnly == 1 && c == 0) || (kOnly == 2 && c != 0)) return bary_small<0, kZeroSigns>(t, px, py, b0, b1, b2);
    b1 = fdiv_y((float)ex, t.fbz, t.rbz);
    b2 = fdiv_y((float)ey, t.fbz, t.rbz);
    if (kOnly == 1 || (kOnly == 0 && c != 0))
    {
        if (!w_fast((float)c, t.fbz, t.rbz, b0))
        {
            float d0, d1, d2;  // near a rounding boundary: the double path decides
            if (!bary_from_ints_double(ex, ey, bz, d0, d1, d2)) return false;
            b0 = d0;
        }
    }
    else
    {
        unsigned long long m53 = t.m53;
        int s53 = t.s53;
        if (s53 == 0) recip53((unsigned long long)(pos ? bz : -bz), m53, s53);  // not cached
        b0 = w_on_edge((unsigned)(pos ? ex : -ex), (unsigned)(pos ? ey : -ey), m53, s53);
        if (b0 < 0.f) return false;
    }
    if (kZeroSigns)
    {
        if (ex == 0) b1 = signed_zero(ref_edge_neg_zero32(s0y, s1z, s0z, s1y) != !pos);
        if (ey == 0) b2 = signed_zero(ref_edge_neg_zero32(s0z, s1x, s0x, s1z) != !pos);
    }
    return true;
}

template <int kOnly = 0, bool kZeroSigns = true>
FR_HD bool bary(const RTri& t, int px, int py, float& b0, float& b1, float& b2)
{
    if (t.cls == kTriReference) return bary_reference(t.x, t.y, px, py, b0, b1, b2);
    if (t.cls == kTriEmpty) return false;
    if (t.cls == kTriFast && t.small && small_pixel(px, py))
        return bary_small<kOnly, kZeroSigns>(t, px, py, b0, b1, b2);
    long long s0x = t.x[1] - t.x[0], s0y = t.x[2] - t.x[0], s0z = t.x[0] - px;
    long long s1x = t.y[1] - t.y[0], s1y = t.y[2] - t.y[0], s1z = t.y[0] - py;
    long long ex = s0y * s1z - s0z * s1y, ey = s0z * s1x - s0x * s1z;
    long long bz = t.bz;
    bool pos = bz > 0;
    if (ex != 0 && ((ex > 0) != pos)) return false;
    if (ey != 0 && ((ey > 0) != pos)) return false;
    long long c = bz - ex - ey;
    if (c != 0 && ((c > 0) != pos)) return false;
    if (t.cls == kTriIntDouble)
    {
        if (!bary_from_ints_double(ex, ey, bz, b0, b1, b2)) return false;
    }
    else
    {
        // |ex|, |ey|, |c| <= |bz| < 2^24 here: int32 conversions are exact (and,
        // unlike 64-bit ones, do not run on the FP64 pipe)
        b1 = fdiv_y((float)(int)ex, t.fbz, t.rbz);
        b2 = fdiv_y((float)(int)ey, t.fbz, t.rbz);
        if (c != 0)
        {
            if (!w_fast((float)(int)c, t.fbz, t.rbz, b0))
            {
                float d0, d1, d2;  // near a rounding boundary: the double path decides
                if (!bary_from_ints_double(ex, ey, bz, d0, d1, d2)) return false;
                b0 = d0;
            }
        }
        else
        {
            unsigned long long m53 = t.m53;
            int s53 = t.s53;
            if (s53 == 0) recip53((unsigned long long)(bz < 0 ? -bz : bz), m53, s53);  // not cached
            b0 = w_on_edge((unsigned)(ex < 0 ? -ex : ex), (unsigned)(ey < 0 ? -ey : ey), m53, s53);
            if (b0 < 0.f) return false;
        }
    }
    if (kZeroSigns)
    {
        if (ex == 0) b1 = signed_zero(ref_edge_neg_zero(s0y, s1z, s0z, s1y) != !pos);
        if (ey == 0) b2 = signed_zero(ref_edge_neg_zero(s0z, s1x, s0x, s1z) != !pos);
    }
    return true;
}

// (float)(c * (double)p) for a positive normal double constant c with 53-bit
// significand cm and exponent ce (c = cm * 2^ce), computed exactly in integers:
// the 77-bit product is rounded to 53 bits, then to 24 bits, both to nearest
// even, as the two IEEE roundings of the reference do. No FP64 instruction is
// issued except for zero / non-finite inputs or results outside the normal
// float range, which fall back to the literal double expression. Used for
// PCF_FILTER_SIZE * penumbra (shadow.cpp:102).
FR_HD float mul_f_d_round(float p, double c, unsigned long long cm, int ce)
{
    unsigned int pb = fbits(p);
    unsigned int pe = (pb >> 23) & 0xffu;
    if (pe == 0u || pe == 0xffu) return (float)(c * (double)p);  // zero, subnormal, inf, NaN
    unsigned long long pm = (pb & 0x7fffffu) | 0x800000u;
    unsigned long long lo = pm * cm;  // pm < 2^24, cm < 2^53: product < 2^77
#ifdef __CUDA_ARCH__
    unsigned long long hi = __umul64hi(pm, cm);
#else
    unsigned long long hi = (unsigned long long)(((unsigned __int128)pm * cm) >> 64);
#endif
    int e = (int)pe - 150 + ce;  // value = (hi:lo) * 2^e
    int nbits = hi ? 128 - clz64(hi) : 64 - clz64(lo);  // 47 <= nbits <= 77
    int sh = nbits - 53;                                 // -6 <= sh <= 24
    unsigned long long m;
    if (sh > 0)
    {
        unsigned long long q = (lo >> sh) | (hi << (64 - sh));
        unsigned long long rem = lo & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull))) ++q;
        if (q >> 53)
        {
            q >>= 1;
            ++sh;
        }
        m = q;
    }
    else
    {
        m = lo << (-sh);
    }
    e += sh;  // double result = m * 2^e, 2^52 <= m < 2^53
    unsigned long long q = m >> 29, rem = m & ((1ull << 29) - 1ull), half = 1ull << 28;
    if (rem > half || (rem == half && (q & 1ull))) ++q;
    int fe = e + 29;
    if (q >> 24)
    {
        q >>= 1;
        ++fe;
    }
    int biased = fe + 150;  // float result = q * 2^fe, 2^23 <= q < 2^24
    if (biased <= 0 || biased >= 255) return (float)(c * (double)p);
    return bitsf((pb & 0x80000000u) | ((unsigned)biased << 23) | ((unsigned)q & 0x7fffffu));
}

// Dot(bary, depths) (geometry.h:881-889): accumulated from 0.f in order.
FR_HD float depth_of(const RTri& t, float b0, float b1, float b2)
{
    float r = 0.f;
    r += b0 * t.d[0];
    r += b1 * t.d[1];
    r += b2 * t.d[2];
    return r;
}

// 64-bit visibility key: order-preserving depth bits above the draw index, so
// an unsigned minimum selects the smallest depth and, among equal depths, the
// first-drawn triangle: the survivor of the reference's in-order strict-less
// test (forkergl.cpp:184-199). The depth is never -0 (it starts from 0.f + x).
constexpr unsigned long long kEmptyKey = ~0ull;

FR_HD unsigned long long make_key(float depth, unsigned int tri)
{
    unsigned int b = fbits(depth);
    b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return ((unsigned long long)b << 32) | tri;
}

FR_HD float key_depth(unsigned long long key)
{
    unsigned int b = (unsigned int)(key >> 32);
    b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
    return bitsf(b);
}

// A fragment takes part in the depth test iff depth < FLT_MAX (the initial
// buffer value, forkergl.cpp:62); NaN depths never pass here.
FR_HD bool depth_passes_clear(float depth) { return depth < 3.40282347e+38f; }

}  // namespace frx
