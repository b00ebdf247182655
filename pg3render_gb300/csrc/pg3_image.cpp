// Image files of a mean image: the reference's Framebuffer::SaveBMP and SaveHDR
// (src/frame_buffer.hxx:114-200), chosen by the file extension as its main program does
// (src/pg3render.cxx:266-273). Host code; the pixels come from the fp64 framebuffer.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pg3_host.h"

namespace pg3 {

namespace {

void put16(std::vector<unsigned char> &b, uint16_t v)
{
    b.push_back((unsigned char)(v & 0xff));
    b.push_back((unsigned char)(v >> 8));
}
void put32(std::vector<unsigned char> &b, uint32_t v)
{
    for (int i = 0; i < 4; ++i) b.push_back((unsigned char)((v >> (8 * i)) & 0xff));
}

bool writeAll(const char *path, const std::vector<unsigned char> &b)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    return (std::fclose(f) == 0) && ok;
}

// 24-bit BMP, rows stored bottom-up in BGR order, each channel pow(v, 1/gamma) * 255 clamped to
// [0, 255] and truncated (src/frame_buffer.hxx:114-163). Rows are padded to 4 bytes as the
// format requires (the reference writes no padding, which only matters for widths that are not
// multiples of 4) and the header's file size is that of the file written.
bool saveBmp(const double *rgb, uint32_t W, uint32_t H, const char *path, float gamma)
{
    const uint32_t row = 3 * W, pad = (4 - row % 4) % 4;
    const uint32_t imageSize = (row + pad) * H;
    std::vector<unsigned char> b;
    b.reserve(54 + imageSize);
    b.push_back('B');
    b.push_back('M');
    put32(b, 54 + imageSize);   // file size
    put32(b, 0);                // reserved
    put32(b, 54);               // pixel data offset
    put32(b, 40);               // info header size
    put32(b, W);
    put32(b, H);
    put16(b, 1);                // colour planes
    put16(b, 24);               // bits per pixel
    put32(b, 0);                // BI_RGB
    put32(b, imageSize);
    put32(b, 2953);             // 75 dpi
    put32(b, 2953);
    put32(b, 0);
    put32(b, 0);
    const double invGamma = 1.0 / (double)gamma;
    for (uint32_t y = 0; y < H; ++y) {
        const double *src = rgb + 3 * (size_t)(H - 1 - y) * W;   // bottom-up
        for (uint32_t x = 0; x < W; ++x) {
            for (int c = 2; c >= 0; --c) {
                const double v = std::pow(src[3 * x + c], invGamma) * 255.0;
                b.push_back((unsigned char)std::fmin(255.0, std::fmax(0.0, v)));
            }
        }
        for (uint32_t p = 0; p < pad; ++p) b.push_back(0);
    }
    return writeAll(path, b);
}

// Radiance RGBE, flat scanlines from the top (src/frame_buffer.hxx:165-200): the largest
// channel's binary exponent e and mantissas c * frexp(max) * 256 / max.
bool saveHdr(const double *rgb, uint32_t W, uint32_t H, const char *path)
{
    std::vector<unsigned char> b;
    const std::string hdr = "#?RADIANCE\n# pg3-gb300\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(H) + " +X " +
                            std::to_string(W) + "\n";
    b.insert(b.end(), hdr.begin(), hdr.end());
    b.reserve(b.size() + 4 * (size_t)W * H);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        const double r = rgb[3 * i], g = rgb[3 * i + 1], bl = rgb[3 * i + 2];
        double v = std::fmax(r, std::fmax(g, bl));
        unsigned char e4[4] = {0, 0, 0, 0};
        if (v >= 1e-32) {
            int e;
            v = std::frexp(v, &e) * 256.0 / v;
            e4[0] = (unsigned char)(r * v);
            e4[1] = (unsigned char)(g * v);
            e4[2] = (unsigned char)(bl * v);
            e4[3] = (unsigned char)(e + 128);
        }
        b.insert(b.end(), e4, e4 + 4);
    }
    return writeAll(path, b);
}

}  // namespace

int writeImage(const double *rgb, uint32_t width, uint32_t height, const char *path, float gamma, std::string &err)
{
    if (!rgb || !path || width == 0 || height == 0) {
        err = "image: NULL data or path, or an empty image";
        return PG3GPU_ERR_INVALID_ARGUMENT;
    }
    const size_t n = std::strlen(path);
    const bool hdr = n >= 4 && (std::strcmp(path + n - 4, ".hdr") == 0 || std::strcmp(path + n - 4, ".HDR") == 0);
    if (!hdr && !(gamma > 0.f && std::isfinite(gamma))) {
        err = "image: gamma must be positive";
        return PG3GPU_ERR_INVALID_ARGUMENT;
    }
    const bool ok = hdr ? saveHdr(rgb, width, height, path) : saveBmp(rgb, width, height, path, gamma);
    if (!ok) {
        err = std::string("image: cannot write ") + path;
        return PG3GPU_ERR_INVALID_ARGUMENT;
    }
    return PG3GPU_OK;
}

}  // namespace pg3
