// Whole-pipeline entry points: host-buffer pipeline and the folder-level drop-in for the
// reference's command-line modes (CommandLineDispatcher.cpp:34-72,
// ImageProcessingManager.cpp:63-108).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "pma_internal.h"
#include "pma_io.h"

using pma::Error;
using pma::guarded;

namespace pma {
namespace {

// Device buffers of one volume, cached in the context under "pipe.*".
struct Fields {
    uint8_t* solid = nullptr;
    uint32_t* edt2 = nullptr;
    uint32_t* crad2 = nullptr;
    uint32_t *cx = nullptr, *cy = nullptr, *cz = nullptr;
    uint8_t* mask = nullptr;
    uint32_t* labels = nullptr;
    uint32_t* labels_ws = nullptr;
    float* dist32 = nullptr;
    double* dist64 = nullptr;
    uint32_t* cavity = nullptr;
};

Fields alloc_fields(pma_ctx* ctx, size_t n, bool pores, bool geo, bool geo64) {
    Fields f;
    f.solid = static_cast<uint8_t*>(ctx->scratch("pipe.solid", n));
    if (pores) {
        f.edt2 = static_cast<uint32_t*>(ctx->scratch("pipe.edt2", n * 4));
        f.crad2 = static_cast<uint32_t*>(ctx->scratch("pipe.crad2", n * 4));
        f.cx = static_cast<uint32_t*>(ctx->scratch("pipe.cx", n * 4));
        f.cy = static_cast<uint32_t*>(ctx->scratch("pipe.cy", n * 4));
        f.cz = static_cast<uint32_t*>(ctx->scratch("pipe.cz", n * 4));
        f.mask = static_cast<uint8_t*>(ctx->scratch("pipe.mask", n));
        f.labels = static_cast<uint32_t*>(ctx->scratch("pipe.labels", n * 4));
        f.labels_ws = static_cast<uint32_t*>(ctx->scratch("pipe.labels_ws", n * 4));
    }
    if (geo) {
        f.dist32 = static_cast<float*>(ctx->scratch("pipe.dist32", n * 4));
        f.cavity = static_cast<uint32_t*>(ctx->scratch("pipe.cavity", n * 4));
    }
    if (geo64) f.dist64 = static_cast<double*>(ctx->scratch("pipe.dist64", n * 8));
    return f;
}

template <class T>
void d2h(pma_ctx* ctx, T* host, const T* dev, size_t n) {
    if (host && dev) copy_to_host(ctx, host, dev, n * sizeof(T));
}

}  // namespace
}  // namespace pma

namespace pma {

// The chain on device fields of one volume (f.solid filled); tables and statistics go to out.
static void run_pore_chain(pma_ctx* ctx, const Fields& f, pma_dims dims, const pma_options& o, pma_outputs* out) {
    out->pores = nullptr;
    out->watershed = nullptr;
    out->n_cavities = 0;
    if (o.run_pores) {
        edt(ctx, f.solid, dims, f.edt2, &out->edt_stats, nullptr, 0);
        containing_balls(ctx, f.edt2, dims, out->edt_stats.max_edt2, f.crad2, f.cx, f.cy, f.cz, f.mask,
                         &out->maximum_balls_count);
        out->pores = pores(ctx, f.mask, f.edt2, f.crad2, dims, o.stencil, f.labels);
        remove_empty_pores(ctx, out->pores, f.labels, dims);
        out->watershed = watershed(ctx, out->pores, f.crad2, dims, o.stencil, out->edt_stats.max_edt2,
                                   f.labels_ws);
    }
}

static void run_geo_chain(pma_ctx* ctx, const Fields& f, pma_dims dims, const pma_options& o, pma_outputs* out) {
    if (!o.run_geodesic) return;
    const std::vector<pma_cavity> rows =
        o.geodesic_fp64 ? geodesic<double>(ctx, f.solid, dims, o.stencil, f.dist64, f.cavity)
                        : geodesic<float>(ctx, f.solid, dims, o.stencil, f.dist32, f.cavity);
    copy_cavities(rows, out->cavities, 16, &out->n_cavities);
    if (out->cavity_rows) copy_cavities(rows, out->cavity_rows, out->cavity_rows_cap, nullptr);
}

static pma_options options_or_default(const pma_options* opts) {
    pma_options o{PMA_D3Q27, 1, 1, 0};
    if (opts) o = *opts;
    return o;
}

void run_pipeline_host(pma_ctx* ctx, const uint8_t* h_solid, pma_dims dims, const pma_options& o,
                       pma_outputs* out) {
    PMA_REQUIRE(h_solid && out, PMA_ERR_ARGUMENT, "pma_pipeline_host: null argument");
    check_dims(dims);
    const size_t n = voxels(dims);
    const bool geo64 = o.run_geodesic && o.geodesic_fp64;
    Fields f = alloc_fields(ctx, n, o.run_pores != 0, o.run_geodesic != 0 && !geo64, geo64);
    if (geo64) f.cavity = static_cast<uint32_t*>(ctx->scratch("pipe.cavity", n * 4));
    copy_from_host(ctx, f.solid, h_solid, n);
    run_pore_chain(ctx, f, dims, o, out);
    run_geo_chain(ctx, f, dims, o, out);
    // Results go back after the whole chain. (Copying the pore-stage fields with the copy
    // engine on a second stream while the geodesics ran made the geodesic kernels slower,
    // 337 -> 754 ms at 1024^3, by more than the copy itself costs.)
    if (o.run_pores) {
        d2h(ctx, out->edt2, f.edt2, n);
        d2h(ctx, out->crad2, f.crad2, n);
        d2h(ctx, out->cx, f.cx, n);
        d2h(ctx, out->cy, f.cy, n);
        d2h(ctx, out->cz, f.cz, n);
        d2h(ctx, out->maxball_mask, f.mask, n);
        d2h(ctx, out->pore_labels, f.labels, n);
        d2h(ctx, out->watershed_labels, f.labels_ws, n);
    }
    if (o.run_geodesic) {
        d2h(ctx, out->dist_f32, f.dist32, n);
        d2h(ctx, out->dist_f64, f.dist64, n);
        d2h(ctx, out->cavity, f.cavity, n);
    }
    ctx->sync();
}

void run_pipeline_device(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, const pma_options& o,
                         pma_outputs* out) {
    PMA_REQUIRE(d_solid && out, PMA_ERR_ARGUMENT, "pma_pipeline_batch: null argument");
    check_dims(dims);
    const size_t n = voxels(dims);
    const bool geo64 = o.run_geodesic && o.geodesic_fp64;
    // caller's device buffers where given, scratch of the context for the rest
    Fields f;
    f.solid = const_cast<uint8_t*>(d_solid);  // only read
    auto pick = [&](auto* given, const char* tag, size_t bytes) {
        using T = std::remove_pointer_t<decltype(given)>;
        return given ? given : static_cast<T*>(ctx->scratch(tag, bytes));
    };
    if (o.run_pores) {
        f.edt2 = pick(out->edt2, "pipe.edt2", n * 4);
        f.crad2 = pick(out->crad2, "pipe.crad2", n * 4);
        f.cx = pick(out->cx, "pipe.cx", n * 4);
        f.cy = pick(out->cy, "pipe.cy", n * 4);
        f.cz = pick(out->cz, "pipe.cz", n * 4);
        f.mask = pick(out->maxball_mask, "pipe.mask", n);
        f.labels = pick(out->pore_labels, "pipe.labels", n * 4);
        f.labels_ws = pick(out->watershed_labels, "pipe.labels_ws", n * 4);
    }
    if (o.run_geodesic) {
        f.cavity = pick(out->cavity, "pipe.cavity", n * 4);
        if (geo64) f.dist64 = pick(out->dist_f64, "pipe.dist64", n * 8);
        else f.dist32 = pick(out->dist_f32, "pipe.dist32", n * 4);
    }
    run_pore_chain(ctx, f, dims, o, out);
    run_geo_chain(ctx, f, dims, o, out);
    ctx->sync();
}

}  // namespace pma

extern "C" int pma_pipeline_host(pma_ctx* ctx, const uint8_t* h_solid, pma_dims dims,
                                 const pma_options* opts, pma_outputs* out) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "pma_pipeline_host: null context");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma::run_pipeline_host(ctx, h_solid, dims, pma::options_or_default(opts), out);
    });
}

// ---------------------------------------------------------------------------------------
// Folder-level drop-in.
// ---------------------------------------------------------------------------------------
namespace pma {
namespace {

const char* kImages = "Images";  // Constants.h:243-254
const char* kEdt = "EuclideanDistanceSquares";
const char* kCrad = "ContainingBallRadiiSquares";
const char* kCx = "ContainingBallCoordinatesX";
const char* kCy = "ContainingBallCoordinatesY";
const char* kCz = "ContainingBallCoordinatesZ";
const char* kMask = "IsMaximumBall";
const char* kPores = "PoreThroatIds";
const char* kWs = "PoreThroatIdsWatershed";
const char* kDist = "ShortestPathDistances";
const char* kCav = "CavityIds";

struct Folder {
    std::string base;
    RunConfig cfg;
    Dims dims;
    std::vector<std::string> slice_names;
    pma_dims pd() const { return pma_dims{dims.sx, dims.sy, dims.sz}; }
};

std::vector<std::string> basenames(const std::vector<std::string>& paths) {
    std::vector<std::string> out;
    for (const std::string& p : paths) {
        size_t s = p.find_last_of('/');
        out.push_back(s == std::string::npos ? p : p.substr(s + 1));
    }
    return out;
}

template <class T>
std::vector<T> read_field(const Folder& f, const char* name) {
    Dims d;
    std::vector<uint8_t> raw = read_stack(join(f.base, name), sizeof(T), &d);
    PMA_REQUIRE(d.sx == f.dims.sx && d.sy == f.dims.sy && d.sz == f.dims.sz, PMA_ERR_IO,
                std::string("Image size is incorrect in ") + name);
    std::vector<T> v(d.count());
    std::memcpy(v.data(), raw.data(), raw.size());
    return v;
}

template <class T>
void write_field(const Folder& f, const char* name, const T* dev, pma_ctx* ctx) {
    std::vector<T> h(f.dims.count());
    PMA_CUDA(cudaMemcpyAsync(h.data(), dev, h.size() * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    write_stack(join(f.base, name), f.slice_names, h.data(), sizeof(T), f.dims);
}

template <class T>
T* upload(pma_ctx* ctx, const std::string& tag, const std::vector<T>& h) {
    T* d = static_cast<T*>(ctx->scratch(tag, h.size() * sizeof(T)));
    PMA_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return d;
}

void write_stats(const Folder& f, uint32_t max_edt2, uint64_t balls) {  // Serializer.cpp:139-146
    FILE* o = std::fopen(join(f.base, "intermediateStatistics.txt").c_str(), "w");
    PMA_REQUIRE(o, PMA_ERR_IO, "cannot write intermediateStatistics.txt");
    std::fprintf(o, "Max Euclidean distance square: %u\nMaximum balls count: %llu\n", max_edt2,
                 static_cast<unsigned long long>(balls));
    std::fclose(o);
}

void read_stats(const Folder& f, uint32_t* max_edt2, uint64_t* balls) {  // Serializer.cpp:130-137
    FILE* i = std::fopen(join(f.base, "intermediateStatistics.txt").c_str(), "r");
    PMA_REQUIRE(i, PMA_ERR_IO, "cannot open intermediateStatistics.txt in " + f.base);
    unsigned long long b = 0;
    unsigned m = 0;
    int k = std::fscanf(i, "Max Euclidean distance square: %u\nMaximum balls count: %llu\n", &m, &b);
    std::fclose(i);
    PMA_REQUIRE(k >= 1, PMA_ERR_IO, "malformed intermediateStatistics.txt in " + f.base);
    *max_edt2 = m;
    *balls = b;
}

void write_hist(const Folder& f, const std::vector<uint64_t>& hist) {  // EDC.cpp:83-110
    size_t last = hist.size();
    for (size_t i = hist.size(); i-- > 0;)
        if (hist[i] != 0) {
            last = i;
            break;
        }
    size_t len = (last == hist.size()) ? 1 : last + 2;
    FILE* o = std::fopen(join(f.base, "euclideanDistanceSquareCounts.txt").c_str(), "w");
    PMA_REQUIRE(o, PMA_ERR_IO, "cannot write euclideanDistanceSquareCounts.txt");
    std::fprintf(o, "EuclideanDistanceSquaresCount (line index is EuclideanDistanceSquare, the next line has index one)\n");
    for (size_t i = 1; i < len; ++i)
        std::fprintf(o, "%llu\n", static_cast<unsigned long long>(i < hist.size() ? hist[i] : 0));
    std::fclose(o);
}

void write_pores(const std::string& path, const pma_table* t) {  // Serializer.cpp:187-201
    FILE* o = std::fopen(path.c_str(), "w");
    PMA_REQUIRE(o, PMA_ERR_IO, "cannot write " + path);
    std::fprintf(o, "PoreId SeedX SeedY SeedZ SeedRadiusSquare IsBoundaryPore Volume\n");
    for (const pma_pore& p : t->pores)
        std::fprintf(o, "%u %d %d %d %d %d %llu\n", p.id, p.seed_x, p.seed_y, p.seed_z,
                     static_cast<int>(p.seed_r2), p.is_boundary ? 1 : 0,
                     static_cast<unsigned long long>(p.volume));
    std::fclose(o);
}

void write_throats(const std::string& path, const pma_table* t) {  // Serializer.cpp:203-221
    FILE* o = std::fopen(path.c_str(), "w");
    PMA_REQUIRE(o, PMA_ERR_IO, "cannot write " + path);
    std::fprintf(o, "SharedPixelTypeId; Volume; PoreId1 PoreId2 ... \n");
    for (const pma_throat& th : t->throats) {
        std::fprintf(o, "%u; %llu;", th.id, static_cast<unsigned long long>(th.volume));
        for (uint32_t i = 0; i < th.n_pores; ++i) std::fprintf(o, " %u", t->pool[th.pool_offset + i]);
        std::fprintf(o, "\n");
    }
    std::fclose(o);
}

pma_table* read_pores(const std::string& path) {  // Serializer.cpp:104-128
    FILE* i = std::fopen(path.c_str(), "r");
    PMA_REQUIRE(i, PMA_ERR_IO, "cannot open " + path);
    int rc = std::fscanf(i, "PoreId SeedX SeedY SeedZ SeedRadiusSquare IsBoundaryPore Volume\n");
    (void)rc;
    pma_table* t = new pma_table;
    while (true) {
        pma_pore p;
        std::memset(&p, 0, sizeof(p));
        int b = 0, r2 = 0;
        unsigned long long vol = 0;
        int k = std::fscanf(i, "%u %d %d %d %d %d %llu\n", &p.id, &p.seed_x, &p.seed_y, &p.seed_z, &r2,
                            &b, &vol);
        if (k != 7) break;
        p.seed_r2 = static_cast<uint32_t>(r2);
        p.is_boundary = b != 0;
        p.volume = vol;
        bool replaced = false;
        for (pma_pore& q : t->pores)
            if (q.id == p.id) {
                q = p;
                replaced = true;
            }
        if (!replaced) t->pores.push_back(p);
    }
    std::fclose(i);
    std::sort(t->pores.begin(), t->pores.end(),
              [](const pma_pore& a, const pma_pore& b) { return a.id < b.id; });
    return t;
}

void write_cavities(const Folder& f, const pma_cavity* c, int n) {  // Serializer.cpp:161-185
    FILE* o = std::fopen(join(f.base, "cavityDescriptions.txt").c_str(), "w");
    PMA_REQUIRE(o, PMA_ERR_IO, "cannot write cavityDescriptions.txt");
    std::fprintf(o, "CavityId SeedX SeedY SeedZ DistanceToCenter VoidPixelsCount ReachedWallsCount IsReachingAllWalls\n");
    for (int i = 0; i < n; ++i)
        std::fprintf(o, "%u %d %d %d %f %llu %d %d\n", c[i].id, c[i].seed_x, c[i].seed_y, c[i].seed_z,
                     static_cast<double>(c[i].distance_to_center),
                     static_cast<unsigned long long>(c[i].void_count), c[i].reached_walls,
                     c[i].reaches_all_walls ? 1 : 0);
    std::fclose(o);
}

std::string file_name(const std::string& path) {
    const size_t s = path.find_last_of('/');
    return s == std::string::npos ? path : path.substr(s + 1);
}

void copy_file(const std::string& from, const std::string& to) {
    FILE* i = std::fopen(from.c_str(), "rb");
    PMA_REQUIRE(i, PMA_ERR_IO, "cannot open " + from);
    FILE* o = std::fopen(to.c_str(), "wb");
    if (!o) {
        std::fclose(i);
        throw Error(PMA_ERR_IO, "cannot write " + to);
    }
    char b[1 << 16];
    size_t k;
    bool ok = true;
    while ((k = std::fread(b, 1, sizeof(b), i)) > 0) ok = ok && std::fwrite(b, 1, k, o) == k;
    std::fclose(i);
    ok = (std::fclose(o) == 0) && ok;
    PMA_REQUIRE(ok, PMA_ERR_IO, "cannot write " + to);
}

// ImageResampler::ResampleImages (ImageResampler.cpp:28-67): when the configured resolution
// makes the image size differ from the slices', the slices move to Original/ and Images/
// receives the resampled ones: slice i of the new stack copies original slice
// (int)(i / resolution_z) (repeated names get "_1", "_2", ... before the extension,
// :184-207), and, when the in-plane size changes too, each is upsampled in plane
// (resample.cu). Runs once: an existing Original/ folder means it already ran.
void resample_images(pma_ctx* ctx, const std::string& base, const RunConfig& cfg) {
    const std::string images = join(base, kImages), original = join(base, "Original");
    if (path_exists(original)) return;
    const std::vector<std::string> paths = list_tiff_stack(images);
    PMA_REQUIRE(!paths.empty(), PMA_ERR_IO,
                "Initial images folder, \"Images\", which shall be near the config.txt file, is empty: " + base);
    const TiffImage first = read_tiff(paths[0]);
    const int actual[3] = {first.rows, first.cols, static_cast<int>(paths.size())};
    int target[3];
    for (int a = 0; a < 3; ++a)  // Serializer.cpp:247-251 (Math::Round)
        target[a] = static_cast<int>(std::floor(actual[a] * cfg.resolution[a] + 0.5));
    if (target[0] == actual[0] && target[1] == actual[1] && target[2] == actual[2]) return;
    PMA_REQUIRE(std::rename(images.c_str(), original.c_str()) == 0, PMA_ERR_IO, "cannot rename " + images);
    ensure_dir(images);
    const std::vector<std::string> before = list_tiff_stack(original);
    std::vector<int> source(target[2]);
    std::vector<std::string> names(target[2]);
    std::string previous;
    int dup = 0;
    for (int i = 0; i < target[2]; ++i) {  // :209-218, :184-207
        source[i] = static_cast<int>(i / cfg.resolution[2]);
        PMA_REQUIRE(source[i] < static_cast<int>(before.size()), PMA_ERR_INTERNAL, "resample: slice index");
        std::string name = file_name(before[source[i]]);
        if (name == previous) {
            ++dup;
            const size_t dot = name.find_last_of('.');
            name = name.substr(0, dot) + "_" + std::to_string(dup) + name.substr(dot);
        } else {
            dup = 0;
            previous = name;
        }
        names[i] = name;
        copy_file(before[source[i]], join(images, name));  // :152-160
    }
    if (target[0] == actual[0] && target[1] == actual[1]) return;
    // in-plane upsampling of every original slice, written under each of its names
    const size_t plane = static_cast<size_t>(actual[0]) * actual[1];
    std::vector<uint8_t> src(plane * before.size());
    for (size_t k = 0; k < before.size(); ++k) {
        const TiffImage im = read_tiff(before[k]);
        PMA_REQUIRE(im.rows == actual[0] && im.cols == actual[1] && im.bits == 8, PMA_ERR_IO,
                    "Image size is incorrect in " + before[k]);
        std::memcpy(src.data() + k * plane, im.data.data(), plane);
    }
    const std::vector<uint8_t> out = resample_slices(ctx, src, static_cast<int>(before.size()), actual[0],
                                                     actual[1], target[0], target[1]);
    const size_t plane2 = static_cast<size_t>(target[0]) * target[1];
    for (int i = 0; i < target[2]; ++i) {
        TiffImage im;
        im.rows = target[0];
        im.cols = target[1];
        im.bits = 8;
        im.data.assign(out.begin() + source[i] * plane2, out.begin() + (source[i] + 1) * plane2);
        write_tiff(join(images, names[i]), im);
    }
}

struct TableGuard {
    pma_table* t = nullptr;
    ~TableGuard() { delete t; }
};

void run_one(pma_ctx* ctx, const std::string& base, pma_mode mode) {
    Folder f;
    f.base = base;
    f.cfg = read_config(join(base, "config.txt"));
    // -edt (and -all) and -spd resample first (ImageProcessingManager.cpp:76-80, 101-105)
    if (mode == PMA_MODE_ALL || mode == PMA_MODE_EDT || mode == PMA_MODE_SPD) resample_images(ctx, base, f.cfg);
    std::vector<std::string> slices = list_tiff_stack(join(base, kImages));
    PMA_REQUIRE(!slices.empty(), PMA_ERR_IO,
                "Initial images folder, \"Images\", which shall be near the config.txt file, is empty: " + base);
    f.slice_names = basenames(slices);
    std::vector<uint8_t> solid = read_stack(join(base, kImages), 1, &f.dims);
    const pma_dims dims = f.pd();
    check_dims(dims);
    const size_t n = f.dims.count();
    const pma_stencil st = f.cfg.use_d3q7 ? PMA_D3Q7 : PMA_D3Q27;

    if (mode == PMA_MODE_SPD) {
        uint8_t* d_solid = upload(ctx, "pipe.solid", solid);
        float* dist = static_cast<float*>(ctx->scratch("pipe.dist32", n * 4));
        uint32_t* cav = static_cast<uint32_t*>(ctx->scratch("pipe.cavity", n * 4));
        const std::vector<pma_cavity> c = geodesic<float>(ctx, d_solid, dims, st, dist, cav);
        write_field(f, kDist, dist, ctx);
        write_field(f, kCav, cav, ctx);
        write_cavities(f, c.data(), static_cast<int>(c.size()));
        return;
    }

    uint32_t* edt2 = static_cast<uint32_t*>(ctx->scratch("pipe.edt2", n * 4));
    uint32_t max_edt2 = 0;
    uint64_t balls = 0;
    if (mode == PMA_MODE_ALL || mode == PMA_MODE_EDT) {
        uint8_t* d_solid = upload(ctx, "pipe.solid", solid);
        pma_edt_stats stats;
        int minext = std::min(f.dims.sx, std::min(f.dims.sy, f.dims.sz));
        std::vector<uint64_t> hist(static_cast<size_t>((minext - 1) / 2) * ((minext - 1) / 2) + 2);
        edt(ctx, d_solid, dims, edt2, &stats, hist.data(), hist.size());
        max_edt2 = stats.max_edt2;
        hist.resize(std::min<size_t>(hist.size(), static_cast<size_t>(max_edt2) + 1));
        write_field(f, kEdt, edt2, ctx);
        write_stats(f, max_edt2, 0);
        write_hist(f, hist);
        if (mode == PMA_MODE_EDT) return;
    } else {
        read_stats(f, &max_edt2, &balls);
    }

    uint32_t* crad2 = static_cast<uint32_t*>(ctx->scratch("pipe.crad2", n * 4));
    uint8_t* mask = static_cast<uint8_t*>(ctx->scratch("pipe.mask", n));
    if (mode == PMA_MODE_ALL || mode == PMA_MODE_RIB) {
        if (mode == PMA_MODE_RIB) {
            std::vector<uint32_t> e = read_field<uint32_t>(f, kEdt);
            edt2 = upload(ctx, "pipe.edt2", e);
        }
        uint32_t* cx = static_cast<uint32_t*>(ctx->scratch("pipe.cx", n * 4));
        uint32_t* cy = static_cast<uint32_t*>(ctx->scratch("pipe.cy", n * 4));
        uint32_t* cz = static_cast<uint32_t*>(ctx->scratch("pipe.cz", n * 4));
        containing_balls(ctx, edt2, dims, max_edt2, crad2, cx, cy, cz, mask, &balls);
        write_field(f, kCrad, crad2, ctx);
        write_field(f, kCx, cx, ctx);
        write_field(f, kCy, cy, ctx);
        write_field(f, kCz, cz, ctx);
        write_field(f, kMask, mask, ctx);
        write_stats(f, max_edt2, balls);
        if (mode == PMA_MODE_RIB) return;
    } else {  // -apt reads the earlier stages' folders
        std::vector<uint32_t> e = read_field<uint32_t>(f, kEdt);
        edt2 = upload(ctx, "pipe.edt2", e);
        std::vector<uint32_t> c = read_field<uint32_t>(f, kCrad);
        crad2 = upload(ctx, "pipe.crad2", c);
        std::vector<uint8_t> m = read_field<uint8_t>(f, kMask);
        mask = upload(ctx, "pipe.mask", m);
    }

    // -apt part (ImageProcessingManager.cpp:89-99)
    uint32_t* labels = static_cast<uint32_t*>(ctx->scratch("pipe.labels", n * 4));
    uint32_t* labels_ws = static_cast<uint32_t*>(ctx->scratch("pipe.labels_ws", n * 4));
    TableGuard pores_t, ws_t;
    pores_t.t = pores(ctx, mask, edt2, crad2, dims, st, labels);
    write_pores(join(base, "pores.txt"), pores_t.t);
    write_throats(join(base, "sharedPixelTypes.txt"), pores_t.t);
    remove_empty_pores(ctx, pores_t.t, labels, dims);
    write_pores(join(base, "pores.txt"), pores_t.t);
    write_throats(join(base, "sharedPixelTypes.txt"), pores_t.t);
    write_field(f, kPores, labels, ctx);
    // The watershed reads the pores back from pores.txt (WatershedComputer.cpp:45).
    TableGuard reread;
    reread.t = read_pores(join(base, "pores.txt"));
    ws_t.t = watershed(ctx, reread.t, crad2, dims, st, max_edt2, labels_ws);
    write_field(f, kWs, labels_ws, ctx);
    write_pores(join(base, "poresWatershed.txt"), ws_t.t);
    write_throats(join(base, "sharedPixelTypesWatershed.txt"), ws_t.t);
}

}  // namespace
}  // namespace pma

extern "C" int pma_run_folder(pma_ctx* ctx, const char* base_folder, pma_mode mode) {
    return guarded([&] {
        PMA_REQUIRE(ctx && base_folder, PMA_ERR_ARGUMENT, "pma_run_folder: null argument");
        PMA_REQUIRE(mode >= PMA_MODE_ALL && mode <= PMA_MODE_SPD, PMA_ERR_ARGUMENT,
                    "pma_run_folder: unknown mode");
        PMA_CUDA(cudaSetDevice(ctx->device));
        std::vector<std::string> folders = pma::folders_with(base_folder, "config.txt");
        // the files written hold the shared-type ids, so they are numbered as the reference does
        const bool numbering = ctx->reference_throat_ids;
        ctx->reference_throat_ids = true;
        try {
            for (const std::string& f : folders) pma::run_one(ctx, f, mode);
        } catch (...) {
            ctx->reference_throat_ids = numbering;
            throw;
        }
        ctx->reference_throat_ids = numbering;
    });
}
