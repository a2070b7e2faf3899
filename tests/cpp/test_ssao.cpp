// Host check of the SSAO estimate bound (forkerrenderer_gb300/csrc/fr_ssao.cuh):
// for random cameras, projections, points, normals and sample offsets, every
// sample the estimate would decide has its exact viewport x, y, z inside the
// estimate's test interval [RN(e - d), RN(e + d)], with the approximate
// reciprocal of the estimate pushed 2 ulp either way. Also reports how many
// samples the estimate decides. Exit status 0 = no violation.
// Usage: test_ssao <num_points> <seed>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "fr_ssao.cuh"

namespace
{

void mat_mul(const float* a, const float* b, float* o)
{
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
        {
            float s = 0.f;
            for (int k = 0; k < 4; ++k) s += a[4 * r + k] * b[4 * k + c];
            o[4 * r + c] = s;
        }
}

// A right-handed look-at view and an OpenGL-style perspective projection.
void camera(std::mt19937_64& rng, float* VP, float dist)
{
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    float e[3] = {U(rng) * dist, U(rng) * dist, U(rng) * dist}, t[3] = {U(rng), U(rng), U(rng)};
    float f[3] = {t[0] - e[0], t[1] - e[1], t[2] - e[2]};
    float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (float& v : f) v /= fl;
    float up[3] = {0.f, 1.f, 0.f};
    float s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    float sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (float& v : s) v /= sl;
    float u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    float V[16] = {s[0], s[1], s[2], -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]),
                   u[0], u[1], u[2], -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]),
                   -f[0], -f[1], -f[2], (f[0] * e[0] + f[1] * e[1] + f[2] * e[2]),
                   0.f, 0.f, 0.f, 1.f};
    float fov = 0.3f + 1.2f * (0.5f + 0.5f * U(rng)), aspect = 0.5f + 1.5f * (0.5f + 0.5f * U(rng));
    float n = 0.01f, fa = 20.f + 100.f * (0.5f + 0.5f * U(rng)), tf = std::tan(fov / 2);
    float P[16] = {1.f / (aspect * tf), 0, 0, 0, 0, 1.f / tf, 0, 0, 0, 0, -(fa + n) / (fa - n), -2 * fa * n / (fa - n),
                   0, 0, -1.f, 0};
    mat_mul(P, V, VP);
}

}  // namespace

int main(int argc, char** argv)
{
    const long npts = argc > 1 ? std::atol(argv[1]) : 20000;
    const unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    long samples = 0, decided = 0, bad = 0, pixelsOk = 0, pixels = 0;
    double worst = 0.0;  // largest |exact - estimate| / (d / 2): the bound's E is d / 2
    for (long i = 0; i < npts; ++i)
    {
        const int scale = (int)(rng() % 4);
        const float dist = scale == 0 ? 3.f : scale == 1 ? 10.f : scale == 2 ? 60.f : 800.f;
        float VP[16];
        camera(rng, VP, dist);
        if (rng() % 6 == 0)  // a generic matrix with a positive w row offset
            for (int k = 0; k < 12; ++k) VP[k] = U(rng) * (rng() % 2 ? 3.f : 0.01f);
        const int W = 64 + (int)(rng() % 4000), H = 64 + (int)(rng() % 3000);
        const float Vp[16] = {W / 2.f, 0, 0, W / 2.f, 0, H / 2.f, 0, H / 2.f, 0, 0, 0.5f, 0.5f, 0, 0, 0, 1};
        const float radius = rng() % 3 == 0 ? 0.075f : rng() % 2 ? 0.5f : 4.f;
        const float pos[3] = {U(rng) * dist * 0.5f, U(rng) * dist * 0.5f, U(rng) * dist * 0.5f};
        const float nrm[3] = {U(rng), U(rng), U(rng)};
        const frx::SsaoPlane q = frx::ssao_plane(VP, Vp, true, radius, pos[0], pos[1], pos[2]);
        ++pixels;
        if (!q.ok) continue;
        ++pixelsOk;
        for (int s = 0; s < 32; ++s)
        {
            float k[3];
            do
            {
                k[0] = U(rng), k[1] = U(rng), k[2] = U(rng);
            } while (k[0] * k[0] + k[1] * k[1] + k[2] * k[2] >= 1.f);
            float sc = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
            sc = (1 - 0.1f) * 1.0f + 0.1f * (sc * sc);
            const float o[3] = {(k[0] * sc) * radius, (k[1] * sc) * radius, (k[2] * sc) * radius};
            const float sg = (k[0] * nrm[0] + k[1] * nrm[1]) + k[2] * nrm[2] > 0.f ? 1.f : -1.f;
            const frx::SsaoProj ex = frx::ssao_project(VP, Vp, true, pos[0], pos[1], pos[2], sg, o[0], o[1], o[2]);
            float Q[4];
            frx::ssao_q(VP, o[0], o[1], o[2], Q);
            const float cx = std::fma(sg, Q[0], q.P[0]), cy = std::fma(sg, Q[1], q.P[1]);
            const float cz = std::fma(sg, Q[2], q.P[2]), cw = std::fma(sg, Q[3], q.P[3]);
            const float r0 = 1.f / cw;
            for (int push = -2; push <= 2; ++push)
            {
                float r = r0;
                for (int m = 0; m < (push < 0 ? -push : push); ++m) r = std::nextafter(r, push < 0 ? 0.f : 1e30f);
                const float e[3] = {std::fma(Vp[0], cx * r, Vp[3]), std::fma(Vp[5], cy * r, Vp[7]),
                                    std::fma(Vp[10], cz * r, Vp[11])};
                const float d[3] = {q.dx, q.dy, q.dz}, x[3] = {ex.x, ex.y, ex.z};
                ++samples;
                bool inside = ex.simple;
                for (int a = 0; a < 3; ++a)
                {
                    inside = inside && (e[a] - d[a]) <= x[a] && x[a] <= (e[a] + d[a]);
                    if (d[a] > 0.f) worst = std::fmax(worst, std::fabs((double)x[a] - (double)e[a]) / (0.5 * d[a]));
                }
                if (!inside)
                {
                    if (bad < 10)
                        std::printf("BOUND VIOLATION pos (%g %g %g) radius %g push %d: exact (%a %a %a) estimate "
                                    "(%a %a %a) half-widths (%g %g %g)\n", pos[0], pos[1], pos[2], radius, push,
                                    ex.x, ex.y, ex.z, e[0], e[1], e[2], d[0], d[1], d[2]);
                    ++bad;
                }
                decided += frx::f2i_sat(e[0] - d[0]) == frx::f2i_sat(e[0] + d[0]) &&
                           frx::f2i_sat(e[1] - d[1]) == frx::f2i_sat(e[1] + d[1]);
            }
        }
    }
    std::printf("pixels %ld with the bound %ld; sample estimates %ld, outside the interval %ld; pixel decided by the "
                "estimate %.4f; largest error %.3f of the bound\n", pixels, pixelsOk, samples, bad,
                samples ? (double)decided / samples : 0.0, worst);
    return bad == 0 && pixelsOk * 2 > pixels ? 0 : 1;
}
