// Test-infrastructure driver around the reference's TGA writer.
//
// Reads raw pixel bytes (TGA byte order: B, G, R[, A] or one gray byte per
// pixel; row y at offset y * width * bytespp), stores them with the reference's
// own TGAImage::Set (src/tgaimage.cpp:313-317) and writes the file with its own
// TGAImage::WriteTgaFile (src/tgaimage.cpp:172-248, RLE packer :250-300), so
// tests can pin the encoder restatement under oracle/ on crafted images.
//
// Usage: ref_tga <pixels.raw> <width> <height> <bytespp> <rle 0|1> <vflip 0|1> <out.tga>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "tgaimage.h"

int main(int argc, char** argv)
{
    if (argc != 8)
    {
        std::fprintf(stderr, "usage: %s <pixels.raw> <w> <h> <bytespp> <rle> <vflip> <out.tga>\n", argv[0]);
        return 1;
    }
    const int w = std::atoi(argv[2]), h = std::atoi(argv[3]), bpp = std::atoi(argv[4]);
    const bool rle = std::atoi(argv[5]) != 0, vflip = std::atoi(argv[6]) != 0;
    std::vector<unsigned char> px((size_t)w * h * bpp);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(px.data(), 1, px.size(), f) != px.size())
    {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    std::fclose(f);
    TGAImage img(w, h, bpp);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) img.Set(x, y, TGAColor(px.data() + ((size_t)y * w + x) * bpp, (uint8_t)bpp));
    return img.WriteTgaFile(argv[7], vflip, rle) ? 0 : 3;
}
