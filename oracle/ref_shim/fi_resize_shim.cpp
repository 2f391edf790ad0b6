/*
 * Bitmap functions for compiling FreeImage's own resize engine (the reference's vendored
 * Externals/FreeImage/Source/FreeImageToolkit/Resize.cpp and Rescale.cpp) into the checker
 * binary oracle/_ref/pma_ref, test infrastructure only. The reference saves its in-plane
 * resampled slices through FreeImage_Rescale with the bilinear filter (Image.h:120-131);
 * with this file the checker does the same, so its resampled stacks are the reference's.
 *
 * A bitmap here is a plain bottom-up pixel buffer with FreeImage's 4-byte-aligned pitch and
 * a linear greyscale palette for 8-bit images. Only what the resize engine reaches for 8-bit
 * greyscale, non-transparent images is implemented; the other entry points return NULL.
 */
#include <cstdlib>
#include <cstring>

#include <FreeImage.h>  // the reference's header (Externals/FreeImage/Source)

namespace {

struct Bitmap {
    FREE_IMAGE_TYPE type;
    unsigned width, height, bpp, pitch;
    BYTE* bits;
    RGBQUAD palette[256];
};

Bitmap* B(FIBITMAP* dib) { return dib ? static_cast<Bitmap*>(dib->data) : nullptr; }

}  // namespace

FIBITMAP* DLL_CALLCONV FreeImage_AllocateT(FREE_IMAGE_TYPE type, int width, int height, int bpp, unsigned, unsigned,
                                           unsigned) {
    if (type != FIT_BITMAP || width <= 0 || height <= 0 || bpp != 8) return NULL;
    Bitmap* b = new Bitmap;
    b->type = type;
    b->width = width;
    b->height = height;
    b->bpp = bpp;
    b->pitch = ((width * bpp / 8) + 3) & ~3u;
    b->bits = static_cast<BYTE*>(std::calloc(static_cast<size_t>(b->pitch) * height, 1));
    for (int i = 0; i < 256; ++i) {
        b->palette[i].rgbRed = b->palette[i].rgbGreen = b->palette[i].rgbBlue = static_cast<BYTE>(i);
        b->palette[i].rgbReserved = 0;
    }
    FIBITMAP* dib = new FIBITMAP;
    dib->data = b;
    return dib;
}

void DLL_CALLCONV FreeImage_Unload(FIBITMAP* dib) {
    if (!dib) return;
    std::free(B(dib)->bits);
    delete B(dib);
    delete dib;
}

FIBITMAP* DLL_CALLCONV FreeImage_Clone(FIBITMAP* dib) {
    Bitmap* s = B(dib);
    if (!s) return NULL;
    FIBITMAP* c = FreeImage_AllocateT(s->type, s->width, s->height, s->bpp, 0, 0, 0);
    if (c) std::memcpy(B(c)->bits, s->bits, static_cast<size_t>(s->pitch) * s->height);
    return c;
}

BOOL DLL_CALLCONV FreeImage_HasPixels(FIBITMAP* dib) { return B(dib) && B(dib)->bits ? TRUE : FALSE; }
FREE_IMAGE_TYPE DLL_CALLCONV FreeImage_GetImageType(FIBITMAP* dib) { return B(dib)->type; }
unsigned DLL_CALLCONV FreeImage_GetBPP(FIBITMAP* dib) { return B(dib)->bpp; }
unsigned DLL_CALLCONV FreeImage_GetWidth(FIBITMAP* dib) { return B(dib)->width; }
unsigned DLL_CALLCONV FreeImage_GetHeight(FIBITMAP* dib) { return B(dib)->height; }
unsigned DLL_CALLCONV FreeImage_GetLine(FIBITMAP* dib) { return B(dib)->width * B(dib)->bpp / 8; }
unsigned DLL_CALLCONV FreeImage_GetPitch(FIBITMAP* dib) { return B(dib)->pitch; }
BYTE* DLL_CALLCONV FreeImage_GetBits(FIBITMAP* dib) { return B(dib)->bits; }
BYTE* DLL_CALLCONV FreeImage_GetScanLine(FIBITMAP* dib, int scanline) {
    return B(dib)->bits + static_cast<size_t>(scanline) * B(dib)->pitch;
}
RGBQUAD* DLL_CALLCONV FreeImage_GetPalette(FIBITMAP* dib) { return B(dib)->bpp <= 8 ? B(dib)->palette : NULL; }
unsigned DLL_CALLCONV FreeImage_GetColorsUsed(FIBITMAP* dib) { return B(dib)->bpp <= 8 ? 1u << B(dib)->bpp : 0; }
FREE_IMAGE_COLOR_TYPE DLL_CALLCONV FreeImage_GetColorType(FIBITMAP*) { return FIC_MINISBLACK; }
BOOL DLL_CALLCONV FreeImage_IsTransparent(FIBITMAP*) { return FALSE; }
unsigned DLL_CALLCONV FreeImage_GetTransparencyCount(FIBITMAP*) { return 0; }
BYTE* DLL_CALLCONV FreeImage_GetTransparencyTable(FIBITMAP*) { return NULL; }
BOOL DLL_CALLCONV FreeImage_CloneMetadata(FIBITMAP*, FIBITMAP*) { return TRUE; }
unsigned DLL_CALLCONV FreeImage_GetRedMask(FIBITMAP*) { return 0; }
unsigned DLL_CALLCONV FreeImage_GetGreenMask(FIBITMAP*) { return 0; }
unsigned DLL_CALLCONV FreeImage_GetBlueMask(FIBITMAP*) { return 0; }

// Not reached for 8-bit greyscale images of different sizes.
FIBITMAP* DLL_CALLCONV FreeImage_Copy(FIBITMAP*, int, int, int, int) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ConvertToGreyscale(FIBITMAP*) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ConvertTo8Bits(FIBITMAP*) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ConvertTo24Bits(FIBITMAP*) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ConvertTo32Bits(FIBITMAP*) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ConvertToRGBF(FIBITMAP*) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ConvertToStandardType(FIBITMAP*, BOOL) { return NULL; }
FIBITMAP* DLL_CALLCONV FreeImage_ToneMapping(FIBITMAP*, FREE_IMAGE_TMO, double, double) { return NULL; }

// Bridge for the fipImage stand-in (FreeImagePlus.h): rescales an 8-bit bottom-up buffer of
// scan width w to nw x nh with the bilinear filter. Returns 0 on success.
extern "C" int pma_shim_rescale8(const unsigned char* bits, unsigned w, unsigned h, unsigned nw, unsigned nh,
                                 unsigned char* out) {
    FIBITMAP* src = FreeImage_AllocateT(FIT_BITMAP, w, h, 8, 0, 0, 0);
    if (!src) return 1;
    for (unsigned r = 0; r < h; ++r) std::memcpy(FreeImage_GetScanLine(src, r), bits + static_cast<size_t>(r) * w, w);
    FIBITMAP* dst = FreeImage_Rescale(src, nw, nh, FILTER_BILINEAR);
    FreeImage_Unload(src);
    if (!dst) return 2;
    for (unsigned r = 0; r < nh; ++r) std::memcpy(out + static_cast<size_t>(r) * nw, FreeImage_GetScanLine(dst, r), nw);
    FreeImage_Unload(dst);
    return 0;
}
