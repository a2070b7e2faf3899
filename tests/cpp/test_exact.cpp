// Host check of the fast barycentric path (forkerrenderer_gb300/csrc/fr_exact.cuh)
// against the reference's literal double arithmetic (geometry.cpp:20-56).
// Exit status 0 = identical float results and coverage on every tested pixel.
// Usage: test_exact <num_triangles> <seed>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <random>

#include "fr_exact.cuh"

int main(int argc, char** argv)
{
    long n = argc > 1 ? std::atol(argv[1]) : 200000;
    unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1;
    std::mt19937_64 rng(seed);
    long pixels = 0, covered = 0, fallbacks = 0, bad = 0;
    for (long t = 0; t < n; ++t)
    {
        frx::RTri tri;
        int mode = (int)(rng() % 7);
        int span = mode == 0 ? 4 : mode == 1 ? 16 : mode == 2 ? 200 : mode == 3 ? 3000
                 : mode == 4 ? 100000 : mode == 5 ? 9000000 : 300;
        int cx = (int)(rng() % 2000) - 500, cy = (int)(rng() % 2000) - 500;
        if (mode == 6)  // around the int32 small-path limit (+-16383) on both sides
        {
            cx = (rng() & 1 ? 1 : -1) * (16383 - 150 + (int)(rng() % 300));
            cy = (rng() & 1 ? 1 : -1) * (16383 - 150 + (int)(rng() % 300));
        }
        for (int k = 0; k < 3; ++k)
        {
            tri.x[k] = cx + (int)(rng() % (2 * span + 1)) - span;
            tri.y[k] = cy + (int)(rng() % (2 * span + 1)) - span;
        }
        if (rng() % 8 == 0) tri.y[1] = tri.y[0];  // axis-aligned edges hit many lattice points
        if (rng() % 8 == 0) tri.x[2] = tri.x[1];
        frx::classify(tri);
        int x0 = std::min(tri.x[0], std::min(tri.x[1], tri.x[2]));
        int y0 = std::min(tri.y[0], std::min(tri.y[1], tri.y[2]));
        int x1 = std::max(tri.x[0], std::max(tri.x[1], tri.x[2]));
        int y1 = std::max(tri.y[0], std::max(tri.y[1], tri.y[2]));
        // sample up to 64 pixels of the bbox (all of it when small)
        long area = (long)(x1 - x0 + 1) * (y1 - y0 + 1);
        int samples = area <= 64 ? (int)area : 64;
        for (int i = 0; i < samples; ++i)
        {
            int px, py;
            if (area <= 64)
            {
                px = x0 + (int)(i % (x1 - x0 + 1));
                py = y0 + (int)(i / (x1 - x0 + 1));
            }
            else
            {
                px = x0 + (int)(rng() % (unsigned long)(x1 - x0 + 1));
                py = y0 + (int)(rng() % (unsigned long)(y1 - y0 + 1));
            }
            float a0 = 0, a1 = 0, a2 = 0, r0 = 0, r1 = 0, r2 = 0;
            bool fa = frx::bary(tri, px, py, a0, a1, a2);
            bool fr = frx::bary_reference(tri.x, tri.y, px, py, r0, r1, r2);
            ++pixels;
            covered += fr;
            {
                // the kernels' form without the zero-sign fix-ups: same coverage, and every
                // consumer (a Dot from 0.f, as depth and each varying) gives the same bits
                float n0 = 0, n1 = 0, n2 = 0;
                const bool fn = frx::bary<0, false>(tri, px, py, n0, n1, n2);
                bool same = fn == fr;
                if (fr && fn)
                {
                    const float attrs[6][3] = {{0.3f, 0.7f, 0.25f}, {0.f, -0.f, 0.f}, {-0.f, -0.f, -0.f},
                                               {1.f, -2.f, 0.5f}, {-0.f, 3.f, -0.f}, {-1.5f, -0.f, 2.5f}};
                    for (const auto& a : attrs)
                    {
                        float w = 0.f, g = 0.f;
                        w += r0 * a[0], w += r1 * a[1], w += r2 * a[2];
                        g += n0 * a[0], g += n1 * a[1], g += n2 * a[2];
                        same = same && std::memcmp(&w, &g, 4) == 0;
                    }
                }
                if (!same)
                {
                    if (bad < 10) std::printf("CONSUMER MISMATCH px (%d,%d)\n", px, py);
                    ++bad;
                }
            }
            if (tri.cls == frx::kTriFast && fr && !frx::maybe_covered(tri, px, py))
            {
                if (bad < 10) std::printf("PRETEST REJECTS covered pixel (%d,%d)\n", px, py);
                ++bad;
            }
            if (tri.cls == frx::kTriFast)
            {
                // the setup kernel's queues: the kind-specialised forms agree with bary()
                int kind = frx::pretest_kind(tri, px, py);
                float k0 = 0, k1 = 0, k2 = 0;
                bool fk = kind == 1 ? frx::bary<1>(tri, px, py, k0, k1, k2)
                        : kind == 2 ? frx::bary<2>(tri, px, py, k0, k1, k2) : false;
                if ((kind == 0 && fr) || fk != fr ||
                    (fr && (std::memcmp(&k0, &r0, 4) || std::memcmp(&k1, &r1, 4) || std::memcmp(&k2, &r2, 4))))
                {
                    if (bad < 10) std::printf("KIND %d MISMATCH px (%d,%d)\n", kind, px, py);
                    ++bad;
                }
            }
            if (fa != fr || (fr && (std::memcmp(&a0, &r0, 4) || std::memcmp(&a1, &r1, 4) ||
                                    std::memcmp(&a2, &r2, 4))))
            {
                if (bad < 10)
                    std::printf("MISMATCH tri (%d,%d)(%d,%d)(%d,%d) px (%d,%d): %d %a %a %a vs %d %a %a %a\n",
                                tri.x[0], tri.y[0], tri.x[1], tri.y[1], tri.x[2], tri.y[2], px, py, fa,
                                a0, a1, a2, fr, r0, r1, r2);
                ++bad;
            }
        }
    }
    (void)fallbacks;
    // Markstein division RN(a / b) = fdiv_y(a, b, RN(1 / b)) for integers |a| <= |b| < 2^24
    long divs = 0, divbad = 0;
    const int bs[] = {1, 2, 3, 7, 255, 256, 257, 65535, 65537, 1048577, 8388607, 8388608, 8388609, 16777215};
    for (int b : bs)
        for (int sgn = -1; sgn <= 1; sgn += 2)
        {
            float fb = (float)(sgn * b), y = frx::frcp_rn(fb);
            int stepa = b > 1000000 ? 97 : 1;
            for (int a = -b; a <= b; a += stepa)
            {
                float q = (float)a / fb, m = frx::fdiv_y((float)a, fb, y);
                ++divs;
                divbad += std::memcmp(&q, &m, 4) != 0;
            }
        }
    for (long i = 0; i < 20 * n; ++i)
    {
        long b = (long)(rng() % 16777215) + 1, a = (long)(rng() % (2 * b + 1)) - b;
        if (rng() & 1) b = -b;
        float fb = (float)b, q = (float)a / fb, m = frx::fdiv_y((float)a, fb, frx::frcp_rn(fb));
        ++divs;
        divbad += std::memcmp(&q, &m, 4) != 0;
    }
    // (float)(0.007 * (double)p) without FP64 (PCSS filter size)
    long muls = 0, mulbad = 0;
    for (long i = 0; i < 20 * n; ++i)
    {
        unsigned u = (unsigned)rng();
        float p;
        std::memcpy(&p, &u, 4);
        if (i & 1) p = std::ldexp((float)(rng() % 16777216), (int)(rng() % 40) - 40);
        float a = (float)(0.007 * (double)p), b = frx::mul_f_d_round(p, 0.007, 0x1cac083126e979ull, -60);
        ++muls;
        mulbad += (std::memcmp(&a, &b, 4) != 0) && !(a != a && b != b);
    }
    // float(1 - (u + v)) on edge BC (ex + ey == bz): every split of every |bz| <= 4096,
    // then random |bz| < 2^24, both signs, against the literal double expression
    long edges = 0, edgebad = 0;
    auto edge_check = [&](long long B, long long a, int sgn) {
        long long bz = sgn * B, ex = sgn * a, ey = sgn * (B - a);
        unsigned long long M;
        int S;
        frx::recip53((unsigned long long)B, M, S);
        double inv = 1.0 / (double)bz, u = (double)ex * inv, v = (double)ey * inv;
        float want = (float)(1.0 - (u + v)), got = frx::w_on_edge((unsigned)a, (unsigned)(B - a), M, S);
        ++edges;
        if (std::memcmp(&want, &got, 4) != 0)
        {
            if (edgebad < 10) std::printf("EDGE MISMATCH B %lld a %lld sgn %d: %a vs %a\n", B, a, sgn, want, got);
            ++edgebad;
        }
    };
    for (long long B = 1; B <= 4096; ++B)
        for (long long a = 0; a <= B; ++a)
            for (int sgn = -1; sgn <= 1; sgn += 2) edge_check(B, a, sgn);
    for (long i = 0; i < 20 * n; ++i)
    {
        long long B = (long long)(rng() % 16777215) + 1, a = (long long)(rng() % (unsigned long long)(B + 1));
        edge_check(B, a, (rng() & 1) ? 1 : -1);
        edge_check(B, (long long)(rng() % 3) * (B / 2), 1);  // vertices and midpoints
    }
    std::printf("pixels %ld covered %ld mismatches %ld; divisions %ld mismatches %ld; products %ld mismatches %ld; "
                "edge weights %ld mismatches %ld\n",
                pixels, covered, bad, divs, divbad, muls, mulbad, edges, edgebad);
    return (bad == 0 && divbad == 0 && mulbad == 0 && edgebad == 0) ? 0 : 1;
}
