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
    long long bz;  // integer edge determinant (classes kTriFast / kTriIntDouble)
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

FR_HD void classify(RTri& t)
{
    if (coords_in_range(t.x, t.y))
    {
        long long bz = (long long)(t.x[1] - t.x[0]) * (t.y[2] - t.y[0]) -
                       (long long)(t.x[2] - t.x[0]) * (t.y[1] - t.y[0]);
        t.bz = bz;
        if (bz == 0) t.cls = kTriEmpty;
        else if (bz > -kBzFastLimit && bz < kBzFastLimit) t.cls = kTriFast;
        else t.cls = kTriIntDouble;
    }
    else
    {
        t.bz = 0;
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
// q = RN_float(c / bz) is exact for the double path unless the quotient lies
// within 2^-51 (the double path's absolute error: two products, a sum and a
// subtraction, 0.875 * 2^-51 at most) of the float rounding boundary on its
// side of q. With q = M * 2^-s (M a 24-bit integer, 23 <= s <= 47) the scaled
// remainder R = c * 2^s - M * bz is an exact integer (|R| <= |bz| / 2, so the
// wrapped 64-bit arithmetic below is exact), and the test
//     4 |R| + ceil(|bz| * 2^(s-49)) < 2 |bz|   (|bz| when q is a power of two
//                                               and the quotient lies below q)
// is that distance condition scaled by 2^(s+2). Otherwise the double path runs.
FR_HD bool w_fast(long long c, long long ex, long long ey, long long bz, float& w)
{
    float q = fdiv_rn((float)c, (float)bz);
    unsigned int qb = fbits(q);
    int s = 150 - (int)(qb >> 23);
    unsigned long long M = (unsigned long long)((qb & 0x7fffffu) | 0x800000u);
    long long R = (long long)(((unsigned long long)c << s) - M * (unsigned long long)bz);
    long long az = bz < 0 ? -bz : bz;
    long long aR = R < 0 ? -R : R;
    bool below = (R != 0) && ((R > 0) != (bz > 0));
    long long lim = (below && (qb & 0x7fffffu) == 0u) ? az : 2 * az;
    int sh = 49 - s;
    long long eterm = (az + ((1ll << sh) - 1)) >> sh;
    if (4 * aR + eterm < lim)
    {
        w = q;
        return true;
    }
    float b0, b1, b2;
    if (!bary_from_ints_double(ex, ey, bz, b0, b1, b2)) return false;
    w = b0;
    return true;
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

FR_HD float signed_zero(bool negative) { return negative ? -0.f : 0.f; }

// Exact coverage + barycentric for one pixel, bit-identical to Barycentric()
// including the sign of zero weights. Returns false if the reference rejects
// the pixel.
FR_HD bool bary(const RTri& t, int px, int py, float& b0, float& b1, float& b2)
{
    if (t.cls == kTriReference) return bary_reference(t.x, t.y, px, py, b0, b1, b2);
    if (t.cls == kTriEmpty) return false;
    long long s0x = t.x[1] - t.x[0], s0y = t.x[2] - t.x[0], s0z = t.x[0] - px;
    long long s1x = t.y[1] - t.y[0], s1y = t.y[2] - t.y[0], s1z = t.y[0] - py;
    long long ex = s0y * s1z - s0z * s1y;
    long long ey = s0z * s1x - s0x * s1z;
    long long bz = t.bz;
    bool pos = bz > 0;
    if (ex != 0 && ((ex > 0) != pos)) return false;
    if (ey != 0 && ((ey > 0) != pos)) return false;
    long long c = bz - ex - ey;
    if (c != 0 && ((c > 0) != pos)) return false;
    if (t.cls == kTriIntDouble || c == 0)
    {
        if (!bary_from_ints_double(ex, ey, bz, b0, b1, b2)) return false;
    }
    else
    {
        float fz = (float)bz;
        b1 = fdiv_rn((float)ex, fz);
        b2 = fdiv_rn((float)ey, fz);
        if (!w_fast(c, ex, ey, bz, b0)) return false;
    }
    if (ex == 0) b1 = signed_zero(ref_edge_neg_zero(s0y, s1z, s0z, s1y) != !pos);
    if (ey == 0) b2 = signed_zero(ref_edge_neg_zero(s0z, s1x, s0x, s1z) != !pos);
    return true;
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
