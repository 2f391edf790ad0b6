// In-plane resampling of the input slices (ImageResampler.cpp:93-150).
//
// The reference upsamples each slice to the configured X x Y size with FreeImage's rescale
// and its bilinear filter (Image.h:120-131, ResizeIfNecessary), and saves that image: its own
// nearest-neighbour loop (ImageResampler.cpp:137-150) writes into a copy that is never put
// back into the image. So the slices it writes are FreeImage's two-pass filtered zoom
// (P. Heckbert, "Zoom" 1989; E. Yariv, "Two pass scaling using filters" 1999) with a triangle
// filter of width 1, restated here:
//  * per output position u of a line: centre c = u / s + 0.5 / s (s = dst / src), source
//    window [max(0, (int)(c - w + 0.5)), min((int)(c + w + 0.5), src)) with w = 1 (w = 1 / s
//    and the filter argument scaled by s when s < 1), weights f(i + 0.5 - c), f(t) =
//    max(0, 1 - |t|), normalised when their sum is not 1, zero weights trimmed at the right;
//  * value = sum of weight * sample in double, in window order, stored as (int)(value + 0.5)
//    clamped to 0..255 (an 8-bit image after each pass);
//  * lines are filtered along the rows first (FreeImage's "vertical" pass, over bottom-up
//    scanlines: scanline k is image row H - 1 - k) when the row count changes, then along the
//    columns when the column count changes: for the magnifications the configuration gives
//    (normalised resolutions are >= 1) this is the order FreeImage chooses.
// The device passes add products in the same order with explicitly rounded double
// operations, so they match the reference's x86 build (no fused multiply-add) bit for bit.
#include <cmath>
#include <vector>

#include "devutil.cuh"

namespace pma {
namespace {

struct LineWeights {
    std::vector<int> left, count;  // per output position: first source index, taps
    std::vector<double> w;         // [dst][window]
    int window = 0;
};

// CWeightsTable of FreeImage's resize engine for its bilinear filter (width 1).
LineWeights bilinear_weights(unsigned dst, unsigned src) {
    const double filter_width = 1.0;
    const double scale = static_cast<double>(dst) / static_cast<double>(src);
    double width, fscale;
    if (scale < 1.0) {
        width = filter_width / scale;
        fscale = scale;
    } else {
        width = filter_width;
        fscale = 1.0;
    }
    LineWeights lw;
    lw.window = 2 * static_cast<int>(std::ceil(width)) + 1;
    lw.left.resize(dst);
    lw.count.resize(dst);
    lw.w.assign(static_cast<size_t>(dst) * lw.window, 0.0);
    const double offset = 0.5 / scale;
    for (unsigned u = 0; u < dst; ++u) {
        const double center = static_cast<double>(u) / scale + offset;
        const int il = std::max(0, static_cast<int>(center - width + 0.5));
        const int ir = std::min(static_cast<int>(center + width + 0.5), static_cast<int>(src));
        double* wt = lw.w.data() + static_cast<size_t>(u) * lw.window;
        double total = 0;
        for (int i = il; i < ir; ++i) {
            double t = fscale * ((static_cast<double>(i) + 0.5) - center);
            t = std::fabs(t);
            const double f = t < filter_width ? filter_width - t : 0.0;
            const double weight = fscale * f;
            wt[i - il] = weight;
            total += weight;
        }
        if (total > 0 && total != 1)
            for (int i = il; i < ir; ++i) wt[i - il] /= total;
        int right = ir, trailing = ir - il - 1;
        while (trailing >= 0 && wt[trailing] == 0) {
            --right;
            --trailing;
            if (right == il) break;
        }
        lw.left[u] = il;
        lw.count[u] = right - il;
    }
    return lw;
}

__device__ __forceinline__ uint8_t round_byte(double value) {
    const int r = __double2int_rz(__dadd_rn(value, 0.5));
    return static_cast<uint8_t>(r < 0 ? 0 : (r > 255 ? 255 : r));
}

// Along the rows (FreeImage's vertical pass over bottom-up scanlines): out[z][x'][y] from
// in[z][x][y], x counted from the top, scanline k = rows - 1 - x.
__global__ void resample_rows(const uint8_t* __restrict__ in, int nz, int sx, int sy, int dx,
                              const int* __restrict__ left, const int* __restrict__ count,
                              const double* __restrict__ w, int window, uint8_t* __restrict__ out) {
    const size_t n = static_cast<size_t>(nz) * dx * sy;
    PMA_GRID_STRIDE(i, n) {
        const int y = static_cast<int>(i % sy);
        const size_t zx = i / sy;
        const int x = static_cast<int>(zx % dx);
        const int z = static_cast<int>(zx / dx);
        const int u = dx - 1 - x;  // output scanline
        const uint8_t* col = in + static_cast<size_t>(z) * sx * sy + y;
        double value = 0;
        for (int k = 0; k < count[u]; ++k) {
            const int src_row = sx - 1 - (left[u] + k);
            value = __dadd_rn(value, __dmul_rn(w[static_cast<size_t>(u) * window + k],
                                               static_cast<double>(col[static_cast<size_t>(src_row) * sy])));
        }
        out[i] = round_byte(value);
    }
}

// Along the columns (FreeImage's horizontal pass): out[z][x][y'] from in[z][x][y].
__global__ void resample_cols(const uint8_t* __restrict__ in, size_t lines, int sy, int dy,
                              const int* __restrict__ left, const int* __restrict__ count,
                              const double* __restrict__ w, int window, uint8_t* __restrict__ out) {
    const size_t n = lines * dy;
    PMA_GRID_STRIDE(i, n) {
        const int u = static_cast<int>(i % dy);
        const uint8_t* row = in + (i / dy) * sy + left[u];
        double value = 0;
        for (int k = 0; k < count[u]; ++k)
            value = __dadd_rn(value, __dmul_rn(w[static_cast<size_t>(u) * window + k], static_cast<double>(row[k])));
        out[i] = round_byte(value);
    }
}

}  // namespace

// Slices [nz][sx][sy] (8-bit, host) -> [nz][dx][dy] (host), dx >= sx, dy >= sy.
std::vector<uint8_t> resample_slices(pma_ctx* ctx, const std::vector<uint8_t>& src, int nz, int sx, int sy, int dx,
                                     int dy) {
    PMA_REQUIRE(dx >= sx && dy >= sy && sx > 0 && sy > 0 && nz > 0, PMA_ERR_ARGUMENT,
                "resample: the target size must not be smaller than the images");
    cudaStream_t s = ctx->stream;
    const size_t n_in = static_cast<size_t>(nz) * sx * sy, n_mid = static_cast<size_t>(nz) * dx * sy,
                 n_out = static_cast<size_t>(nz) * dx * dy;
    uint8_t* a = static_cast<uint8_t*>(ctx->scratch("resample.in", n_in));
    uint8_t* b = static_cast<uint8_t*>(ctx->scratch("resample.mid", n_mid));
    uint8_t* c = static_cast<uint8_t*>(ctx->scratch("resample.out", n_out));
    PMA_CUDA(cudaMemcpyAsync(a, src.data(), n_in, cudaMemcpyHostToDevice, s));
    auto upload = [&](const LineWeights& lw, const char* tag, int** dl, int** dc, double** dw) {
        const size_t m = lw.left.size();
        *dl = static_cast<int*>(ctx->scratch(std::string(tag) + ".l", m * 4));
        *dc = static_cast<int*>(ctx->scratch(std::string(tag) + ".c", m * 4));
        *dw = static_cast<double*>(ctx->scratch(std::string(tag) + ".w", lw.w.size() * 8));
        PMA_CUDA(cudaMemcpyAsync(*dl, lw.left.data(), m * 4, cudaMemcpyHostToDevice, s));
        PMA_CUDA(cudaMemcpyAsync(*dc, lw.count.data(), m * 4, cudaMemcpyHostToDevice, s));
        PMA_CUDA(cudaMemcpyAsync(*dw, lw.w.data(), lw.w.size() * 8, cudaMemcpyHostToDevice, s));
    };
    const uint8_t* cur = a;
    LineWeights rows_w, cols_w;  // kept alive until the copies above have run (synchronised below)
    if (dx != sx) {
        rows_w = bilinear_weights(static_cast<unsigned>(dx), static_cast<unsigned>(sx));
        int *l, *cn;
        double* w;
        upload(rows_w, "resample.rows", &l, &cn, &w);
        resample_rows<<<grid_for(ctx, n_mid), 256, 0, s>>>(cur, nz, sx, sy, dx, l, cn, w, rows_w.window, b);
        ctx->check_launch("resample_rows");
        cur = b;
    }
    if (dy != sy) {
        cols_w = bilinear_weights(static_cast<unsigned>(dy), static_cast<unsigned>(sy));
        int *l, *cn;
        double* w;
        upload(cols_w, "resample.cols", &l, &cn, &w);
        resample_cols<<<grid_for(ctx, n_out), 256, 0, s>>>(cur, static_cast<size_t>(nz) * dx, sy, dy, l, cn, w,
                                                          cols_w.window, c);
        ctx->check_launch("resample_cols");
        cur = c;
    }
    std::vector<uint8_t> out(n_out);
    PMA_CUDA(cudaMemcpyAsync(out.data(), cur, n_out, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    return out;
}

}  // namespace pma
