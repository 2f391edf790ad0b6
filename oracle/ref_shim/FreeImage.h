/*
 * Stand-in for the FreeImage C header, used only to compile the reference's own
 * sources into the checker binary oracle/_ref/pma_ref (test infrastructure).
 * The reference includes FreeImage.h only for FreeImage_Initialise under FREEIMAGE_LIB,
 * which this build does not define.
 */
#ifndef PMA_REF_SHIM_FREEIMAGE_H
#define PMA_REF_SHIM_FREEIMAGE_H
typedef unsigned char BYTE;
#endif
