// Host-side I/O of the pma library. The TIFF subset matches what the reference reads and
// writes through FreeImage (Image.h:55-83): 8-bit one-sample images in, 8-bit grey and
// 32-bit CMYK (four 8-bit samples holding one little-endian uint32/float) out.
#include "pma_io.h"

#include <dirent.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace pma {

namespace {

struct Reader {
    const std::vector<uint8_t>& b;
    bool le;
    uint16_t u16(size_t o) const {
        if (o + 2 > b.size()) throw std::runtime_error("TIFF: truncated file");
        return le ? static_cast<uint16_t>(b[o] | (b[o + 1] << 8))
                  : static_cast<uint16_t>((b[o] << 8) | b[o + 1]);
    }
    uint32_t u32(size_t o) const {
        if (o + 4 > b.size()) throw std::runtime_error("TIFF: truncated file");
        return le ? (uint32_t(b[o]) | (uint32_t(b[o + 1]) << 8) | (uint32_t(b[o + 2]) << 16) |
                     (uint32_t(b[o + 3]) << 24))
                  : ((uint32_t(b[o]) << 24) | (uint32_t(b[o + 1]) << 16) |
                     (uint32_t(b[o + 2]) << 8) | uint32_t(b[o + 3]));
    }
};

struct Tag {
    uint16_t type = 0;
    uint32_t count = 0;
    uint32_t value_offset = 0;  // raw 4-byte field
    size_t field_pos = 0;       // file position of the 4-byte field
};

size_t type_size(uint16_t t) {
    switch (t) {
        case 1: case 2: case 6: case 7: return 1;
        case 3: case 8: return 2;
        case 4: case 9: case 11: return 4;
        case 5: case 10: case 12: return 8;
        default: return 1;
    }
}

std::vector<uint32_t> tag_values(const Reader& r, const Tag& t) {
    std::vector<uint32_t> out(t.count);
    size_t sz = type_size(t.type);
    size_t base = (sz * t.count <= 4) ? t.field_pos : t.value_offset;
    for (uint32_t i = 0; i < t.count; ++i) {
        if (t.type == 3) out[i] = r.u16(base + 2 * i);
        else if (t.type == 4) out[i] = r.u32(base + 4 * i);
        else if (t.type == 1) {
            if (base + i >= r.b.size()) throw std::runtime_error("TIFF: truncated tag");
            out[i] = r.b[base + i];
        } else throw std::runtime_error("TIFF: unsupported tag type");
    }
    return out;
}

std::vector<uint8_t> slurp(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    return std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

}  // namespace

// TIFF 6.0 LZW: codes are written most significant bit first; 256 clears the table,
// 257 ends the strip, the table grows from 258 and the code width goes from 9 to 12 bits,
// one code earlier than the table size would need ("early change").
std::vector<uint8_t> lzw_decode(const uint8_t* src, size_t n, size_t expected) {
    std::vector<uint8_t> out;
    out.reserve(expected);
    std::vector<uint16_t> prefix(4096);
    std::vector<uint8_t> suffix(4096), first(4096);
    std::vector<uint16_t> length(4096);
    for (int i = 0; i < 256; ++i) {
        prefix[i] = 0xFFFF;
        suffix[i] = static_cast<uint8_t>(i);
        first[i] = static_cast<uint8_t>(i);
        length[i] = 1;
    }
    std::vector<uint8_t> tmp(4096);
    size_t bitpos = 0;
    int width = 9;
    int next = 258;
    int prev = -1;
    auto emit = [&](int code) {
        int len = length[code];
        int c = code;
        for (int i = len - 1; i >= 0; --i) {
            tmp[i] = suffix[c];
            c = prefix[c];
        }
        out.insert(out.end(), tmp.begin(), tmp.begin() + len);
    };
    while (out.size() < expected) {
        if (bitpos + width > n * 8) break;
        uint32_t code = 0;
        for (int i = 0; i < width; ++i) {
            size_t p = bitpos + i;
            code = (code << 1) | ((src[p >> 3] >> (7 - (p & 7))) & 1);
        }
        bitpos += width;
        if (code == 257) break;
        if (code == 256) {
            width = 9;
            next = 258;
            prev = -1;
            continue;
        }
        if (prev < 0) {
            if (code > 255) throw std::runtime_error("TIFF LZW: bad first code");
            emit(code);
            prev = static_cast<int>(code);
            continue;
        }
        if (static_cast<int>(code) > next || next >= 4096)
            throw std::runtime_error("TIFF LZW: corrupt code stream");
        uint8_t head = (static_cast<int>(code) < next) ? first[code] : first[prev];
        prefix[next] = static_cast<uint16_t>(prev);
        suffix[next] = head;
        first[next] = first[prev];
        length[next] = static_cast<uint16_t>(length[prev] + 1);
        ++next;
        emit(code);
        prev = static_cast<int>(code);
        if (next == 511) width = 10;
        else if (next == 1023) width = 11;
        else if (next == 2047) width = 12;
    }
    if (out.size() > expected) out.resize(expected);
    return out;
}

std::vector<uint8_t> lzw_encode(const uint8_t* src, size_t n) {
    std::vector<uint8_t> out;
    uint64_t acc = 0;
    int nacc = 0;
    int width = 9;
    auto put = [&](uint32_t code) {
        acc = (acc << width) | code;
        nacc += width;
        while (nacc >= 8) {
            out.push_back(static_cast<uint8_t>(acc >> (nacc - 8)));
            nacc -= 8;
        }
    };
    // (prefix code, byte) -> code, open-addressed hash.
    const int HS = 1 << 13;
    std::vector<int32_t> hkey(HS, -1);
    std::vector<uint16_t> hval(HS);
    auto reset = [&]() { std::fill(hkey.begin(), hkey.end(), -1); };
    int next = 258;
    put(256);
    if (n == 0) {
        put(257);
        if (nacc > 0) out.push_back(static_cast<uint8_t>(acc << (8 - nacc)));
        return out;
    }
    int cur = src[0];
    for (size_t i = 1; i < n; ++i) {
        uint8_t c = src[i];
        int32_t key = (cur << 8) | c;
        uint32_t h = (static_cast<uint32_t>(key) * 2654435761u) >> 19;
        bool found = false;
        while (hkey[h] != -1) {
            if (hkey[h] == key) {
                found = true;
                break;
            }
            h = (h + 1) & (HS - 1);
        }
        if (found) {
            cur = hval[h];
            continue;
        }
        put(static_cast<uint32_t>(cur));
        hkey[h] = key;
        hval[h] = static_cast<uint16_t>(next);
        ++next;
        cur = c;
        if (next == 4094) {  // table full: clear with the current width
            put(256);
            reset();
            next = 258;
            width = 9;
        } else if (next == 512) width = 10;
        else if (next == 1024) width = 11;
        else if (next == 2048) width = 12;
    }
    put(static_cast<uint32_t>(cur));
    // The decoder adds an entry for this code too; the width must follow it.
    ++next;
    if (next == 4094) {
        put(256);
        width = 9;
    } else if (next == 512) width = 10;
    else if (next == 1024) width = 11;
    else if (next == 2048) width = 12;
    put(257);
    if (nacc > 0) out.push_back(static_cast<uint8_t>(acc << (8 - nacc)));
    return out;
}

TiffImage read_tiff(const std::string& path) {
    std::vector<uint8_t> b = slurp(path);
    if (b.size() < 8) throw std::runtime_error("TIFF: too short: " + path);
    bool le;
    if (b[0] == 'I' && b[1] == 'I') le = true;
    else if (b[0] == 'M' && b[1] == 'M') le = false;
    else throw std::runtime_error("not a TIFF file: " + path);
    Reader r{b, le};
    if (r.u16(2) != 42) throw std::runtime_error("TIFF: bad magic: " + path);
    size_t ifd = r.u32(4);
    uint16_t ntags = r.u16(ifd);
    std::vector<std::pair<uint16_t, Tag>> tags;
    for (uint16_t i = 0; i < ntags; ++i) {
        size_t e = ifd + 2 + 12 * static_cast<size_t>(i);
        Tag t;
        t.type = r.u16(e + 2);
        t.count = r.u32(e + 4);
        t.value_offset = r.u32(e + 8);
        t.field_pos = e + 8;
        tags.push_back({r.u16(e), t});
    }
    auto find = [&](uint16_t id) -> const Tag* {
        for (auto& kv : tags)
            if (kv.first == id) return &kv.second;
        return nullptr;
    };
    auto scalar = [&](uint16_t id, uint32_t dflt) -> uint32_t {
        const Tag* t = find(id);
        if (!t) return dflt;
        return tag_values(r, *t)[0];
    };
    TiffImage img;
    img.cols = static_cast<int>(scalar(256, 0));
    img.rows = static_cast<int>(scalar(257, 0));
    uint32_t spp = scalar(277, 1);
    uint32_t compression = scalar(259, 1);
    uint32_t predictor = scalar(317, 1);
    uint32_t planar = scalar(284, 1);
    const Tag* bps_tag = find(258);
    uint32_t bps = bps_tag ? tag_values(r, *bps_tag)[0] : 1;
    if (bps != 8) throw std::runtime_error("TIFF: only 8-bit samples are supported: " + path);
    if (spp != 1 && spp != 4) throw std::runtime_error("TIFF: only 1 or 4 samples per pixel: " + path);
    if (planar != 1 && spp > 1) throw std::runtime_error("TIFF: planar images unsupported: " + path);
    if (compression != 1 && compression != 5)
        throw std::runtime_error("TIFF: only uncompressed or LZW images: " + path);
    if (img.rows <= 0 || img.cols <= 0) throw std::runtime_error("TIFF: empty image: " + path);
    img.bits = static_cast<int>(8 * spp);
    uint32_t rps = scalar(278, static_cast<uint32_t>(img.rows));
    if (rps == 0 || rps > static_cast<uint32_t>(img.rows)) rps = static_cast<uint32_t>(img.rows);
    const Tag* off_tag = find(273);
    const Tag* cnt_tag = find(279);
    if (!off_tag || !cnt_tag) throw std::runtime_error("TIFF: no strips: " + path);
    std::vector<uint32_t> offs = tag_values(r, *off_tag);
    std::vector<uint32_t> cnts = tag_values(r, *cnt_tag);
    const size_t row_bytes = static_cast<size_t>(img.cols) * spp;
    img.data.assign(row_bytes * img.rows, 0);
    size_t row = 0;
    for (size_t s = 0; s < offs.size() && row < static_cast<size_t>(img.rows); ++s) {
        size_t nrows = std::min<size_t>(rps, img.rows - row);
        size_t want = nrows * row_bytes;
        if (static_cast<size_t>(offs[s]) + cnts[s] > b.size())
            throw std::runtime_error("TIFF: strip beyond end of file: " + path);
        std::vector<uint8_t> strip;
        if (compression == 5) strip = lzw_decode(b.data() + offs[s], cnts[s], want);
        else strip.assign(b.begin() + offs[s], b.begin() + offs[s] + std::min<size_t>(cnts[s], want));
        if (strip.size() < want) throw std::runtime_error("TIFF: short strip: " + path);
        if (predictor == 2) {
            for (size_t rr = 0; rr < nrows; ++rr) {
                uint8_t* p = strip.data() + rr * row_bytes;
                for (size_t i = spp; i < row_bytes; ++i) p[i] = static_cast<uint8_t>(p[i] + p[i - spp]);
            }
        }
        std::memcpy(img.data.data() + row * row_bytes, strip.data(), want);
        row += nrows;
    }
    if (row < static_cast<size_t>(img.rows)) throw std::runtime_error("TIFF: missing strips: " + path);
    return img;
}

void write_tiff(const std::string& path, const TiffImage& img) {
    if (img.bits != 8 && img.bits != 32) throw std::runtime_error("TIFF: only 8 or 32 bits are written");
    const uint32_t spp = img.bits / 8;
    const size_t row_bytes = static_cast<size_t>(img.cols) * spp;
    const uint32_t rps = std::max<uint32_t>(1, static_cast<uint32_t>(8192 / std::max<size_t>(row_bytes, 1)));
    std::vector<std::vector<uint8_t>> strips;
    for (int r0 = 0; r0 < img.rows; r0 += static_cast<int>(rps)) {
        int nr = std::min<int>(static_cast<int>(rps), img.rows - r0);
        std::vector<uint8_t> raw(img.data.begin() + r0 * row_bytes, img.data.begin() + (r0 + nr) * row_bytes);
        for (int rr = 0; rr < nr; ++rr) {  // horizontal differencing, right to left
            uint8_t* p = raw.data() + rr * row_bytes;
            for (size_t i = row_bytes; i-- > spp;) p[i] = static_cast<uint8_t>(p[i] - p[i - spp]);
        }
        strips.push_back(lzw_encode(raw.data(), raw.size()));
    }
    std::vector<uint8_t> f;
    auto p16 = [&](uint16_t v) { f.push_back(v & 0xFF); f.push_back(v >> 8); };
    auto p32 = [&](uint32_t v) { for (int i = 0; i < 4; ++i) f.push_back((v >> (8 * i)) & 0xFF); };
    f.insert(f.end(), {'I', 'I', 42, 0});
    p32(0);  // IFD offset patched below
    std::vector<uint32_t> offsets;
    for (auto& s : strips) {
        offsets.push_back(static_cast<uint32_t>(f.size()));
        f.insert(f.end(), s.begin(), s.end());
        if (f.size() & 1) f.push_back(0);
    }
    // Out-of-line arrays.
    uint32_t off_arr = static_cast<uint32_t>(f.size());
    for (uint32_t o : offsets) p32(o);
    uint32_t cnt_arr = static_cast<uint32_t>(f.size());
    for (auto& s : strips) p32(static_cast<uint32_t>(s.size()));
    uint32_t bps_arr = static_cast<uint32_t>(f.size());
    for (uint32_t i = 0; i < spp; ++i) p16(8);
    if (f.size() & 1) f.push_back(0);
    uint32_t ifd = static_cast<uint32_t>(f.size());
    f[4] = ifd & 0xFF; f[5] = (ifd >> 8) & 0xFF; f[6] = (ifd >> 16) & 0xFF; f[7] = ifd >> 24;
    struct E { uint16_t tag, type; uint32_t count, value; };
    std::vector<E> es;
    es.push_back({256, 4, 1, static_cast<uint32_t>(img.cols)});
    es.push_back({257, 4, 1, static_cast<uint32_t>(img.rows)});
    if (spp == 1) es.push_back({258, 3, 1, 8});
    else es.push_back({258, 3, spp, bps_arr});
    es.push_back({259, 3, 1, 5});
    es.push_back({262, 3, 1, spp == 1 ? 1u : 5u});
    es.push_back({273, 4, static_cast<uint32_t>(offsets.size()),
                  offsets.size() == 1 ? offsets[0] : off_arr});
    es.push_back({277, 3, 1, spp});
    es.push_back({278, 4, 1, rps});
    es.push_back({279, 4, static_cast<uint32_t>(strips.size()),
                  strips.size() == 1 ? static_cast<uint32_t>(strips[0].size()) : cnt_arr});
    es.push_back({284, 3, 1, 1});
    es.push_back({317, 3, 1, 2});
    if (spp == 4) es.push_back({332, 3, 1, 1});
    p16(static_cast<uint16_t>(es.size()));
    for (const E& e : es) {
        p16(e.tag);
        p16(e.type);
        p32(e.count);
        if (e.type == 3 && e.count == 1) { p16(static_cast<uint16_t>(e.value)); p16(0); }
        else p32(e.value);
    }
    p32(0);
    std::ofstream o(path, std::ios::binary | std::ios::trunc);
    if (!o) throw std::runtime_error("cannot write " + path);
    o.write(reinterpret_cast<const char*>(f.data()), static_cast<std::streamsize>(f.size()));
    if (!o) throw std::runtime_error("write failed: " + path);
}

bool path_exists(const std::string& p) {
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

void ensure_dir(const std::string& p) {
    if (p.empty() || path_exists(p)) return;
    size_t slash = p.find_last_of('/');
    if (slash != std::string::npos && slash > 0) ensure_dir(p.substr(0, slash));
    if (::mkdir(p.c_str(), 0755) != 0 && errno != EEXIST)
        throw std::runtime_error("cannot create folder " + p);
}

std::string join(const std::string& a, const std::string& b) {  // Path.cpp Append
    if (a.empty()) return b;
    if (b.empty()) return a;
    if (a.back() == '/' || b.front() == '/') return a + b;
    return a + "/" + b;
}

static std::vector<std::string> list_dir(const std::string& folder, bool want_dirs) {
    std::vector<std::string> out;
    DIR* d = ::opendir(folder.c_str());
    if (!d) return out;
    while (dirent* e = ::readdir(d)) {
        std::string n = e->d_name;
        if (n == "." || n == "..") continue;
        struct stat st;
        if (::stat(join(folder, n).c_str(), &st) != 0) continue;
        bool is_dir = S_ISDIR(st.st_mode);
        if (is_dir == want_dirs) out.push_back(n);
    }
    ::closedir(d);
    std::sort(out.begin(), out.end());
    return out;
}

std::vector<std::string> list_tiff_stack(const std::string& folder) {
    std::vector<std::pair<std::string, std::string>> named;
    for (const std::string& n : list_dir(folder, false)) {
        size_t dot = n.find_last_of('.');
        if (dot == std::string::npos) continue;
        std::string ext = n.substr(dot);
        if (ext == ".tif" || ext == ".tiff") named.push_back({n.substr(0, dot), n});
    }
    std::stable_sort(named.begin(), named.end(),
                     [](const std::pair<std::string, std::string>& a,
                        const std::pair<std::string, std::string>& b) { return a.first < b.first; });
    std::vector<std::string> out;
    for (auto& kv : named) out.push_back(join(folder, kv.second));
    return out;
}

std::vector<uint8_t> read_stack(const std::string& folder, int bpv, Dims* dims) {
    std::vector<std::string> files = list_tiff_stack(folder);
    if (files.empty()) throw std::runtime_error("no TIFF slices in " + folder);
    std::vector<uint8_t> vol;
    for (size_t z = 0; z < files.size(); ++z) {
        TiffImage im = read_tiff(files[z]);
        if (im.bits != 8 * bpv)
            throw std::runtime_error("Bits per pixel in the images are not equal to the size of the data element: " + files[z]);
        if (z == 0) {
            dims->sx = im.rows;
            dims->sy = im.cols;
            dims->sz = static_cast<int>(files.size());
            vol.resize(dims->count() * bpv);
        } else if (im.rows != dims->sx || im.cols != dims->sy) {
            throw std::runtime_error("Image size is incorrect: " + files[z]);
        }
        std::memcpy(vol.data() + z * im.data.size(), im.data.data(), im.data.size());
    }
    return vol;
}

void write_stack(const std::string& folder, const std::vector<std::string>& names, const void* data,
                 int bpv, const Dims& dims) {
    ensure_dir(folder);
    const size_t slice = static_cast<size_t>(dims.sx) * dims.sy * bpv;
    for (int z = 0; z < dims.sz; ++z) {
        TiffImage im;
        im.rows = dims.sx;
        im.cols = dims.sy;
        im.bits = 8 * bpv;
        const uint8_t* p = static_cast<const uint8_t*>(data) + z * slice;
        im.data.assign(p, p + slice);
        std::string name = (static_cast<size_t>(z) < names.size()) ? names[z] : (std::to_string(z + 1) + ".tif");
        write_tiff(join(folder, name), im);
    }
}

std::vector<uint8_t> read_raw(const std::string& path, size_t bytes) {
    std::vector<uint8_t> b = slurp(path);
    if (b.size() != bytes)
        throw std::runtime_error("raw volume " + path + " has " + std::to_string(b.size()) +
                                 " bytes, expected " + std::to_string(bytes));
    return b;
}

void write_raw(const std::string& path, const void* data, size_t bytes) {
    std::ofstream o(path, std::ios::binary | std::ios::trunc);
    if (!o) throw std::runtime_error("cannot write " + path);
    o.write(static_cast<const char*>(data), static_cast<std::streamsize>(bytes));
    if (!o) throw std::runtime_error("write failed: " + path);
}

RunConfig read_config(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) throw std::runtime_error("cannot open " + path);
    RunConfig c;
    // Same fscanf format as Serializer.cpp:40-52; fields that do not parse keep -1.
    int n = std::fscanf(f,
                        "Resolution of initial images: %lf %lf %lf\n"
                        "Available memory in megabytes: %d\n"
                        "Max ratio of pore radius to seed radius: %lf\n"
                        "Use D3Q7 stencil: %d\n"
                        "Number of threads: %d\n",
                        &c.resolution[0], &c.resolution[1], &c.resolution[2], &c.available_memory_mb,
                        &c.max_pore_radius_ratio, &c.use_d3q7, &c.threads);
    std::fclose(f);
    if (n < 6) throw std::runtime_error("config.txt does not follow the expected format: " + path);
    double mn = std::min(c.resolution[0], std::min(c.resolution[1], c.resolution[2]));
    if (!(mn > 0)) throw std::runtime_error("config.txt: resolution must be positive: " + path);
    for (double& r : c.resolution) r /= mn;  // Serializer.cpp:61-63
    return c;
}

static void collect(const std::string& base, const std::string& file, std::vector<std::string>* out) {
    if (path_exists(join(base, file))) out->push_back(base);
    for (const std::string& sub : list_dir(base, true)) collect(join(base, sub), file, out);
}

std::vector<std::string> folders_with(const std::string& base, const std::string& file) {
    std::vector<std::string> out;
    collect(base, file, &out);
    return out;
}

}  // namespace pma
