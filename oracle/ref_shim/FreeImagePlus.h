/*
 * Minimal stand-in for FreeImagePlus's fipImage, used only to compile the reference's
 * own sources into the checker binary oracle/_ref/pma_ref (test infrastructure).
 *
 * It implements the calls of ImageProcessing/Model/Headers/Image.h on an in-memory
 * bitmap stored bottom-up like FreeImage (scanline 0 is the last image row). Files use a
 * private uncompressed format ("PMASHIM1", width, height, bits per pixel, rows top to
 * bottom) that the test harness writes and reads; TIFF decoding is not reproduced.
 */
#ifndef PMA_REF_SHIM_FREEIMAGEPLUS_H
#define PMA_REF_SHIM_FREEIMAGEPLUS_H

#include <cstdio>
#include <cstring>
#include <vector>

#include "FreeImage.h"

#define TIFF_DEFAULT 0
#define TIFF_CMYK 0x0001
#define TIFF_LZW 0x4000
#define FILTER_BILINEAR 2
#define FIT_RGBA16 10

extern "C" int pma_shim_rescale8(const unsigned char* bits, unsigned w, unsigned h, unsigned nw, unsigned nh,
                                 unsigned char* out);

class fipImage {
  public:
    fipImage() : width_(0), height_(0), bpp_(0) {}

    bool load(const char* path, int /*flags*/ = 0) {
        FILE* f = std::fopen(path, "rb");
        if (!f) return false;
        char magic[8];
        unsigned hdr[3];
        bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "PMASHIM1", 8) == 0 &&
                  std::fread(hdr, sizeof(unsigned), 3, f) == 3;
        if (ok) {
            width_ = hdr[0];
            height_ = hdr[1];
            bpp_ = hdr[2];
            bits_.assign(static_cast<size_t>(getScanWidth()) * height_, 0);
            for (unsigned r = 0; r < height_ && ok; ++r)
                ok = std::fread(&bits_[static_cast<size_t>(height_ - 1 - r) * getScanWidth()], 1,
                                getScanWidth(), f) == getScanWidth();
        }
        std::fclose(f);
        if (!ok) {
            width_ = height_ = bpp_ = 0;
            bits_.clear();
        }
        return ok;
    }

    bool save(const char* path, int /*flags*/ = 0) const {
        FILE* f = std::fopen(path, "wb");
        if (!f) return false;
        unsigned hdr[3] = {width_, height_, bpp_};
        bool ok = std::fwrite("PMASHIM1", 1, 8, f) == 8 && std::fwrite(hdr, sizeof(unsigned), 3, f) == 3;
        for (unsigned r = 0; r < height_ && ok; ++r)
            ok = std::fwrite(&bits_[static_cast<size_t>(height_ - 1 - r) * getScanWidth()], 1,
                             getScanWidth(), f) == getScanWidth();
        std::fclose(f);
        return ok;
    }

    unsigned getWidth() const { return width_; }
    unsigned getHeight() const { return height_; }
    unsigned getBitsPerPixel() const { return bpp_; }
    unsigned getScanWidth() const { return width_ * (bpp_ / 8); }
    BYTE* accessPixels() const { return bits_.empty() ? 0 : const_cast<BYTE*>(&bits_[0]); }

    // Pixel values are overwritten after every conversion in Image.h, so a conversion
    // only changes the pixel size.
    bool convertTo4Bits() { return setBpp(8); }
    bool convertTo8Bits() { return setBpp(8); }
    bool convertTo24Bits() { return setBpp(24); }
    bool convertTo32Bits() { return setBpp(32); }
    bool convertToType(int, bool) { return setBpp(64); }

    // FreeImage's own bilinear rescale for 8-bit images (its Resize.cpp compiled with
    // fi_resize_shim.cpp); other sizes are only reallocated, as their pixels are overwritten.
    bool rescale(unsigned w, unsigned h, int) {
        if (bpp_ == 8 && width_ && height_) {
            std::vector<BYTE> out(static_cast<size_t>(w) * h);
            if (pma_shim_rescale8(&bits_[0], width_, height_, w, h, &out[0]) != 0) return false;
            width_ = w;
            height_ = h;
            bits_.swap(out);
            return true;
        }
        width_ = w;
        height_ = h;
        bits_.assign(static_cast<size_t>(getScanWidth()) * height_, 0);
        return true;
    }

  private:
    bool setBpp(unsigned b) {
        bpp_ = b;
        bits_.assign(static_cast<size_t>(getScanWidth()) * height_, 0);
        return true;
    }
    unsigned width_, height_, bpp_;
    std::vector<BYTE> bits_;
};

#endif
