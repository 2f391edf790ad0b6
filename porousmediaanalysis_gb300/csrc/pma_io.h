// Host-side volume and table I/O of the pma library: TIFF stacks, raw volumes,
// config.txt and the reference's text artefacts.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pma {

// One decoded TIFF image: rows x cols samples of 8 or 32 bits.
struct TiffImage {
    int rows = 0;      // TIFF ImageLength; the reference's X extent (Image.h:62-70)
    int cols = 0;      // TIFF ImageWidth;  the reference's Y extent
    int bits = 0;      // 8 (grey) or 32 (4 x 8-bit samples read as one little-endian word)
    std::vector<uint8_t> data;  // rows * cols * bits/8 bytes, file row order
};

// Reads uncompressed or LZW (with or without horizontal predictor) strip TIFFs with
// 8-bit one-sample or 4 x 8-bit samples per pixel. Throws std::runtime_error.
TiffImage read_tiff(const std::string& path);

// Writes an LZW + horizontal-predictor strip TIFF. bits 8 -> grey, 32 -> CMYK
// (the reference's 32-bit format, Image.h:72-83).
void write_tiff(const std::string& path, const TiffImage& img);

// LZW codec of TIFF 6.0 (MSB-first codes, 9..12 bits, early change).
std::vector<uint8_t> lzw_decode(const uint8_t* src, size_t n, size_t expected);
std::vector<uint8_t> lzw_encode(const uint8_t* src, size_t n);

// Sorted list of *.tif / *.tiff files of a folder, ordered by file name without
// extension (Serializer.cpp:254-281).
std::vector<std::string> list_tiff_stack(const std::string& folder);

// Volume helpers. Layout [z][x][y] with y fastest.
struct Dims {
    int sx = 0, sy = 0, sz = 0;
    size_t count() const { return static_cast<size_t>(sx) * sy * sz; }
};

// Reads a stack of slices (one file per z) into [z][x][y] elements of `bytes_per_voxel`.
std::vector<uint8_t> read_stack(const std::string& folder, int bytes_per_voxel, Dims* dims);
// Writes [z][x][y] elements as one TIFF per slice, named after `names` (file names).
void write_stack(const std::string& folder, const std::vector<std::string>& names,
                 const void* data, int bytes_per_voxel, const Dims& dims);

std::vector<uint8_t> read_raw(const std::string& path, size_t bytes);
void write_raw(const std::string& path, const void* data, size_t bytes);

// config.txt (Serializer.cpp:31-64).
struct RunConfig {
    double resolution[3] = {1, 1, 1};
    int available_memory_mb = -1;
    double max_pore_radius_ratio = -1;
    int use_d3q7 = 0;
    int threads = -1;
};
RunConfig read_config(const std::string& path);

bool path_exists(const std::string& p);
void ensure_dir(const std::string& p);
std::string join(const std::string& a, const std::string& b);
// Every folder under base (base included) holding `file`, sorted (CommandLineDispatcher.cpp:62).
std::vector<std::string> folders_with(const std::string& base, const std::string& file);

}  // namespace pma
