/*
 * Deterministic sample tables for the stochastic passes of the frame.
 *
 * The reference renderer draws the PCSS blocker-search / PCF disk taps
 * (src/shaders/shadow.cpp:56,76 via RandomVectorInUnitDisk, src/geometry.h:968)
 * and the SSAO hemisphere taps (src/render.cpp:240 via RandomVectorInHemisphere,
 * src/geometry.h:978) from one global sequential std::mt19937 stream whose
 * consumption is data dependent. A GPU cannot replay that stream, so every
 * implementation here (CUDA kernels, CPU oracle, reference harness) replaces the
 * draws with the fixed tables defined in this header:
 *
 *   - tap i of the PCSS blocker search uses blocker[i]   (i < num_blocker)
 *   - tap j of PCF (standalone or inside PCSS) uses pcf[j]  (j < num_pcf)
 *   - SSAO sample s of pixel (x, y) uses kernel[((y & 3) * 4 + (x & 3)) * N + s]
 *     (a 4x4 grid of independent N-sample kernels: the rotation-noise tile),
 *     flipped into the hemisphere of the normal exactly as the reference does.
 *
 * Points are drawn by rejection sampling, like the reference's samplers, from
 * SplitMix64 streams. Coordinates are k / 2^23 - 1 (exact in float), and the
 * acceptance test is evaluated in double where it is exact, so the tables are
 * bit-identical on every compiler and architecture.
 */
#ifndef FR_SAMPLE_TABLES_H
#define FR_SAMPLE_TABLES_H

#include <stdint.h>

#define FR_TABLE_SEED_BLOCKER 0x5EED0001ull
#define FR_TABLE_SEED_PCF 0x5EED0002ull
#define FR_TABLE_SEED_SSAO 0x5EED0003ull

static inline uint64_t fr_splitmix64(uint64_t* state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Uniform in [-1, 1): (k - 2^23) / 2^23 with k a 24-bit integer; exact in float. */
static inline float fr_table_sym01(uint64_t* state)
{
    int32_t k = (int32_t)(fr_splitmix64(state) >> 40);
    return (float)(k - 8388608) * (1.0f / 8388608.0f);
}

/* n points (x, y) of the open unit disk, interleaved xy. */
static inline void fr_make_disk_table(uint64_t seed, int n, float* xy)
{
    uint64_t st = seed;
    int i = 0;
    while (i < n)
    {
        float x = fr_table_sym01(&st);
        float y = fr_table_sym01(&st);
        double r2 = (double)x * (double)x + (double)y * (double)y;
        if (r2 >= 1.0) continue;
        xy[2 * i + 0] = x;
        xy[2 * i + 1] = y;
        ++i;
    }
}

/* n points (x, y, z) of the open unit ball, interleaved xyz. */
static inline void fr_make_ball_table(uint64_t seed, int n, float* xyz)
{
    uint64_t st = seed;
    int i = 0;
    while (i < n)
    {
        float x = fr_table_sym01(&st);
        float y = fr_table_sym01(&st);
        float z = fr_table_sym01(&st);
        double r2 = (double)x * (double)x + (double)y * (double)y + (double)z * (double)z;
        if (r2 >= 1.0) continue;
        xyz[3 * i + 0] = x;
        xyz[3 * i + 1] = y;
        xyz[3 * i + 2] = z;
        ++i;
    }
}

/* The SSAO kernel for N samples per pixel: 16 * N points (one N-point kernel per
 * cell of the 4x4 noise tile). */
static inline void fr_make_ssao_table(int samples_per_pixel, float* xyz)
{
    fr_make_ball_table(FR_TABLE_SEED_SSAO, 16 * samples_per_pixel, xyz);
}

#endif /* FR_SAMPLE_TABLES_H */
