/* Test-infrastructure stub (oracle build only). OpenEXR is not part of this
 * image; the reference only uses it to read a lat-long RGB image
 * (em_image.hxx:51-93). This stand-in exposes the same four calls and reads
 * the repository's raw environment-map format instead:
 *   bytes 0-3  magic "PG3F"
 *   bytes 4-15 uint32 width, height, channels (= 3), little endian
 *   then width*height*3 float32, rows top (theta = 0) to bottom.
 * Synthetic environment maps reach the unmodified reference loader this way. */
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace Imath {
struct V2i { int x, y; };
struct Box2i { V2i min, max; };
}

namespace Imf {
struct Rgba { float r, g, b, a; };

class RgbaInputFile {
public:
    RgbaInputFile(const char *name, int /*numThreads*/)
    {
        FILE *f = std::fopen(name, "rb");
        if (!f) throw std::runtime_error("cannot open environment map");
        char magic[4];
        uint32_t hdr[3];
        if (std::fread(magic, 1, 4, f) != 4 || std::memcmp(magic, "PG3F", 4) != 0 ||
            std::fread(hdr, 4, 3, f) != 3 || hdr[2] != 3) {
            std::fclose(f);
            throw std::runtime_error("bad environment map header");
        }
        mW = (int)hdr[0];
        mH = (int)hdr[1];
        mPix.resize((size_t)mW * mH * 3);
        if (std::fread(mPix.data(), 4, mPix.size(), f) != mPix.size()) {
            std::fclose(f);
            throw std::runtime_error("truncated environment map");
        }
        std::fclose(f);
    }
    Imath::Box2i dataWindow() const
    {
        Imath::Box2i b;
        b.min.x = 0; b.min.y = 0; b.max.x = mW - 1; b.max.y = mH - 1;
        return b;
    }
    void setFrameBuffer(Rgba *base, size_t xStride, size_t yStride)
    {
        mBase = base; mXs = xStride; mYs = yStride;
    }
    void readPixels(int y0, int y1)
    {
        for (int y = y0; y <= y1; ++y)
            for (int x = 0; x < mW; ++x) {
                Rgba &p = mBase[(size_t)y * mYs + (size_t)x * mXs];
                const float *s = &mPix[((size_t)y * mW + x) * 3];
                p.r = s[0]; p.g = s[1]; p.b = s[2]; p.a = 1.f;
            }
    }
private:
    int mW = 0, mH = 0;
    std::vector<float> mPix;
    Rgba *mBase = nullptr;
    size_t mXs = 1, mYs = 0;
};
}
