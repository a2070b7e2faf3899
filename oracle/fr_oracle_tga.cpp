// CPU oracle of the TGA output (TEST INFRASTRUCTURE ONLY): the reference's
// image conversions and TGA writer restated in plain C++, used by tests/ and
// bench.py's CPU baseline as the checker of the GPU encoder.
//
//   * fr_oracle_u8: the implicit float -> std::uint8_t conversion of the
//     reference's TGAColor constructors (src/tgaimage.h:44-55) as its x86-64 build
//     executes it: truncation toward zero to a 32-bit integer (NaN and values
//     outside the int32 range give INT32_MIN), then the low 8 bits.
//   * fr_oracle_image_1f / _3f: Buffer1f::GenerateImage (src/buffer.cpp:20-32,
//     value * 255, one gray byte) and Buffer3f::GenerateImage (:113-126, each
//     channel * 254.99f, stored B, G, R as TGAColor does).
//   * fr_oracle_tga_encode: TGAImage::WriteTgaFile (src/tgaimage.cpp:172-248): an
//     18-byte header, the pixel bytes (raw, or the RLE packets of unloadRleData,
//     :250-300), two zero 4-byte area references and the 18-byte footer.
//
// The RLE packer is a greedy left-to-right parse. At a packet start s:
//   * if pixel s equals pixel s + 1 the packet is a run: it covers s and every
//     following pixel equal to it, at most 128 pixels (header 127 + length);
//   * otherwise it is a raw packet (header length - 1): it grows one pixel at a
//     time and stops before a pixel that equals its successor, except that the
//     128th pixel is taken without looking at its successor.
// Parity is pinned against the reference's own writer (oracle/ref_tga.cpp and the
// reference's Output module run by oracle/ref_harness.cpp --tga 1) through
// tests/golden/.
#include <cmath>
#include <cstring>

#include "fr_oracle.h"

namespace
{

bool same_pixel(const uint8_t* a, const uint8_t* b, int bpp)
{
    for (int c = 0; c < bpp; ++c)
        if (a[c] != b[c]) return false;
    return true;
}

// Pixels in the packet starting at s (of n), and whether it is a raw packet.
int64_t packet_at(const uint8_t* px, int64_t n, int bpp, int64_t s, bool& raw)
{
    const auto eq = [&](int64_t i) { return i + 1 < n && same_pixel(px + i * bpp, px + (i + 1) * bpp, bpp); };
    raw = !eq(s);
    int64_t len = 1;
    if (!raw)
    {
        while (len < 128 && eq(s + len - 1)) ++len;
        return len;
    }
    // raw: pixel s + len joins while it exists, the packet is below 128 pixels,
    // and (for the first 126 candidates) the pixel before it does not start a run
    while (len < 128 && s + len < n)
    {
        if (len >= 2 && eq(s + len - 1)) return len - 1;
        ++len;
    }
    return len;
}

void put16(uint8_t* p, int v)
{
    p[0] = (uint8_t)(v & 0xff);
    p[1] = (uint8_t)((v >> 8) & 0xff);
}

}  // namespace

extern "C" {

uint8_t fr_oracle_u8(float v)
{
    if (!(v >= -2147483648.f && v < 2147483648.f)) return 0;  // NaN / out of range: INT32_MIN
    return (uint8_t)((uint32_t)(int32_t)v & 0xffu);
}

void fr_oracle_image_1f(const float* v, int64_t n, uint8_t* out)
{
    for (int64_t i = 0; i < n; ++i) out[i] = fr_oracle_u8(v[i] * 255);
}

void fr_oracle_image_3f(const float* v, int64_t n, uint8_t* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        out[3 * i] = fr_oracle_u8(v[3 * i + 2] * 254.99f);
        out[3 * i + 1] = fr_oracle_u8(v[3 * i + 1] * 254.99f);
        out[3 * i + 2] = fr_oracle_u8(v[3 * i] * 254.99f);
    }
}

int64_t fr_oracle_tga_max_bytes(int64_t width, int64_t height, int32_t bytespp)
{
    return 18 + 26 + width * height * (1 + (int64_t)bytespp);
}

int64_t fr_oracle_tga_encode(const uint8_t* px, int32_t width, int32_t height, int32_t bpp, int32_t rle,
                             int32_t vflip, uint8_t* out, int64_t cap)
{
    if (width < 0 || height < 0 || (bpp != 1 && bpp != 3 && bpp != 4)) return -1;
    if (cap < fr_oracle_tga_max_bytes(width, height, bpp)) return -1;
    const int64_t n = (int64_t)width * height;
    uint8_t* o = out;
    std::memset(o, 0, 18);
    o[2] = (uint8_t)(bpp == 1 ? (rle ? 11 : 3) : (rle ? 10 : 2));
    put16(o + 12, width);
    put16(o + 14, height);
    o[16] = (uint8_t)(bpp * 8);
    o[17] = vflip ? 0x00 : 0x20;
    o += 18;
    if (!rle)
    {
        std::memcpy(o, px, (size_t)(n * bpp));
        o += n * bpp;
    }
    else
    {
        for (int64_t s = 0; s < n;)
        {
            bool raw = false;
            const int64_t len = packet_at(px, n, bpp, s, raw);
            *o++ = (uint8_t)(raw ? len - 1 : len + 127);
            const int64_t bytes = raw ? len * bpp : bpp;
            std::memcpy(o, px + s * bpp, (size_t)bytes);
            o += bytes;
            s += len;
        }
    }
    std::memset(o, 0, 8);
    o += 8;
    static const char kFooter[18] = {'T', 'R', 'U', 'E', 'V', 'I', 'S', 'I', 'O',
                                     'N', '-', 'X', 'F', 'I', 'L', 'E', '.', '\0'};
    std::memcpy(o, kFooter, 18);
    o += 18;
    return o - out;
}

}  // extern "C"
