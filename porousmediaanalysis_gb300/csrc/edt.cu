// Squared Euclidean distance transform (EuclideanDistanceComputer.cpp:149-343).
//
// The reference runs a two-scan along X with virtual solids at x = -SX and x = 2SX-1
// (BOUNDARIES_ARE_SOLID = false), then brute-force windowed minima along Y and along Z.
// Both windowed minima compute exactly h(y) = min_{y'} g(y') + (y - y')^2, so any exact
// 1-D minimisation gives identical integers. Here:
//   pass X: one thread per (y, z) column. A forward read of the mask packs the column into
//           a bitmask in shared memory; a backward sweep finds the nearest solid on both
//           sides from the bits. HBM: 1 B read + 4 B written per voxel.
//   pass Y: one warp per contiguous row, staged in shared memory; each output scans
//           outward from its own position and stops once d^2 reaches the best value.
//   pass Z: tiles of 16 consecutive y by all z staged in shared memory, same exact scan,
//           fused with the running maximum and the histogram of balls that do not cross
//           the image boundary (EDC.cpp:310-327).
#include <algorithm>
#include <mutex>
#include <vector>

#include "pma_internal.h"

namespace pma {
namespace {

constexpr int kHistSmall = 2048;  // histogram bins kept in shared memory per block

// ---------------------------------------------------------------------------------------
// Pass X
// ---------------------------------------------------------------------------------------
__global__ void edt_pass_x(const uint8_t* __restrict__ solid, uint32_t* __restrict__ g, int SX,
                           int SY, int SZ, int words) {
    extern __shared__ uint32_t bits[];  // [words][blockDim.x]
    const int col = blockIdx.x * blockDim.x + threadIdx.x;  // over SY * SZ columns
    const int ncols = SY * SZ;
    const bool active = col < ncols;
    const int y = active ? col % SY : 0;
    const int z = active ? col / SY : 0;
    const size_t base = static_cast<size_t>(z) * SX * SY + y;
    const int T = blockDim.x;
    uint32_t* mybits = bits + threadIdx.x;

    // Forward: pack solid flags, 32 rows per word. Loads of a word are independent.
    for (int w = 0; w < words; ++w) {
        uint32_t word = 0;
        if (active) {
            const int x0 = w * 32;
            const int n = min(32, SX - x0);
            uint8_t v[32];
#pragma unroll
            for (int i = 0; i < 32; ++i)
                v[i] = (i < n) ? __ldg(solid + base + static_cast<size_t>(x0 + i) * SY) : 0;
#pragma unroll
            for (int i = 0; i < 32; ++i) word |= (v[i] != 0 ? 1u : 0u) << i;
        }
        mybits[w * T] = word;
    }
    if (!active) return;

    // Backward: nearest solid at or after x (running) and at or before x (bit search).
    int next_solid = -1;  // -1: none yet (virtual solid at 2SX-1)
    int prev_solid = -2;  // -2: not searched yet
    for (int x = SX - 1; x >= 0; --x) {
        const uint32_t word = mybits[(x >> 5) * T];
        const bool s = (word >> (x & 31)) & 1u;
        uint32_t out;
        if (s) {
            next_solid = x;
            prev_solid = x;
            out = 0;
        } else {
            if (prev_solid == -2 || prev_solid > x) {
                // highest set bit at index <= x
                int wi = x >> 5;
                uint32_t m = word & (0xFFFFFFFFu >> (31 - (x & 31)));
                prev_solid = -1;
                while (true) {
                    if (m) {
                        prev_solid = wi * 32 + 31 - __clz(m);
                        break;
                    }
                    if (--wi < 0) break;
                    m = mybits[wi * T];
                }
            }
            const uint32_t dl = prev_solid >= 0 ? static_cast<uint32_t>(x - prev_solid)
                                                : static_cast<uint32_t>(x + SX);
            const uint32_t dr = next_solid >= 0 ? static_cast<uint32_t>(next_solid - x)
                                                : static_cast<uint32_t>(2 * SX - 1 - x);
            const uint32_t dmin = dl < dr ? dl : dr;
            out = dmin * dmin;
        }
        g[base + static_cast<size_t>(x) * SY] = out;
    }
}

// Exact 1-D lower envelope at position i of a staged line: min_j f[j] + (i-j)^2.
__device__ __forceinline__ uint32_t scan_line(const uint32_t* f, int stride, int n, int i) {
    uint32_t best = f[i * stride];
    if (best == 0) return 0;
    for (int d = 1;; ++d) {
        const uint32_t dd = static_cast<uint32_t>(d) * static_cast<uint32_t>(d);
        if (dd >= best) break;
        if (i - d >= 0) {
            const uint32_t c = f[(i - d) * stride] + dd;
            best = c < best ? c : best;
        }
        if (i + d < n) {
            const uint32_t c = f[(i + d) * stride] + dd;
            best = c < best ? c : best;
        }
        if (i - d < 0 && i + d >= n) break;
    }
    return best;
}

// ---------------------------------------------------------------------------------------
// Pass Y: one warp per row of SY elements.
// ---------------------------------------------------------------------------------------
__global__ void edt_pass_y(uint32_t* __restrict__ g, int SY, size_t nrows) {
    extern __shared__ uint32_t rows[];  // [warps][SY]
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int warps = blockDim.x >> 5;
    uint32_t* line = rows + static_cast<size_t>(warp) * SY;
    for (size_t r = static_cast<size_t>(blockIdx.x) * warps + warp; r < nrows;
         r += static_cast<size_t>(gridDim.x) * warps) {
        uint32_t* p = g + r * SY;
        for (int i = lane; i < SY; i += 32) line[i] = p[i];
        __syncwarp();
        for (int i = lane; i < SY; i += 32) p[i] = scan_line(line, 1, SY, i);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------
// Pass Z with maximum and histogram.
// ---------------------------------------------------------------------------------------
constexpr int kTileY = 16;

__global__ void edt_pass_z(uint32_t* __restrict__ g, int SX, int SY, int SZ,
                           unsigned long long* __restrict__ hist, size_t hist_len,
                           unsigned int* __restrict__ max_out) {
    extern __shared__ uint32_t smem[];
    uint32_t* tile = smem;                                  // [SZ][kTileY]
    unsigned int* h_small = smem + static_cast<size_t>(SZ) * kTileY;  // [kHistSmall]
    const int tiles_y = (SY + kTileY - 1) / kTileY;
    const int x = blockIdx.x / tiles_y;
    const int y0 = (blockIdx.x % tiles_y) * kTileY;
    const int ny = min(kTileY, SY - y0);
    const size_t plane = static_cast<size_t>(SX) * SY;
    const size_t base = static_cast<size_t>(x) * SY + y0;

    for (int i = threadIdx.x; i < kHistSmall; i += blockDim.x) h_small[i] = 0;
    for (int i = threadIdx.x; i < SZ * kTileY; i += blockDim.x) {
        const int z = i / kTileY, yy = i % kTileY;
        tile[i] = (yy < ny) ? g[base + z * plane + yy] : 0;
    }
    __syncthreads();

    unsigned int local_max = 0;
    const int mx = min(x, SX - 1 - x);
    for (int i = threadIdx.x; i < SZ * kTileY; i += blockDim.x) {
        const int z = i / kTileY, yy = i % kTileY;
        if (yy >= ny) continue;
        const uint32_t e = scan_line(tile + yy, kTileY, SZ, z);
        g[base + z * plane + yy] = e;
        if (e == 0) continue;
        local_max = e > local_max ? e : local_max;
        const int y = y0 + yy;
        int m = min(mx, min(min(y, SY - 1 - y), min(z, SZ - 1 - z)));
        // e <= m^2 <=> the ball of radius sqrt(e) stays inside the image (EDC.cpp:316-327).
        if (static_cast<unsigned long long>(e) <= static_cast<unsigned long long>(m) * m) {
            if (e < kHistSmall) atomicAdd(&h_small[e], 1u);
            else if (e < hist_len) atomicAdd(&hist[e], 1ull);
        }
    }
    // block maximum
    for (int o = 16; o > 0; o >>= 1) {
        unsigned int v = __shfl_xor_sync(0xFFFFFFFFu, local_max, o);
        local_max = v > local_max ? v : local_max;
    }
    if ((threadIdx.x & 31) == 0 && local_max) atomicMax(max_out, local_max);
    __syncthreads();
    for (int i = threadIdx.x; i < kHistSmall && i < static_cast<int>(hist_len); i += blockDim.x)
        if (h_small[i]) atomicAdd(&hist[i], static_cast<unsigned long long>(h_small[i]));
}

// The dynamic shared-memory limit is a process-wide attribute of each kernel, so it is set
// once per device to the device's opt-in maximum: lowering it per call would race with
// calls on other host threads (batch lanes) that launch with more.
std::mutex g_attr_mutex;
std::vector<int> g_attr_devices;

void edt_smem_attributes(size_t optin) {
    int dev = 0;
    PMA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    if (std::find(g_attr_devices.begin(), g_attr_devices.end(), dev) != g_attr_devices.end()) return;
    const int bytes = static_cast<int>(optin);
    PMA_CUDA(cudaFuncSetAttribute(edt_pass_x, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    PMA_CUDA(cudaFuncSetAttribute(edt_pass_y, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    PMA_CUDA(cudaFuncSetAttribute(edt_pass_z, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    g_attr_devices.push_back(dev);
}

}  // namespace

void edt(pma_ctx* ctx, const uint8_t* solid, pma_dims d, uint32_t* edt2, pma_edt_stats* stats,
         uint64_t* h_hist, size_t hist_cap) {
    KernelTimer kt_stage(ctx, "stage_edt");  // the whole stage, for the untimed remainder
    check_dims(d);
    edt_smem_attributes(ctx->smem_optin);
    PMA_REQUIRE(solid && edt2, PMA_ERR_ARGUMENT, "pma_edt: null device pointer");
    const int SX = d.sx, SY = d.sy, SZ = d.sz;
    cudaStream_t s = ctx->stream;

    // Pass X
    {
        const int words = (SX + 31) / 32;
        int threads = 256;
        while (threads > 32 && static_cast<size_t>(words) * 4 * threads > 96 * 1024) threads >>= 1;
        const size_t smem = static_cast<size_t>(words) * 4 * threads;
        PMA_REQUIRE(smem <= ctx->smem_optin, PMA_ERR_ARGUMENT, "pma_edt: X extent too large");
        const size_t cols = static_cast<size_t>(SY) * SZ;
        KernelTimer kt(ctx, "edt_pass_x");
        edt_pass_x<<<div_up(cols, threads), threads, smem, s>>>(solid, edt2, SX, SY, SZ, words);
        ctx->check_launch("edt_pass_x");
    }
    // Pass Y
    {
        int warps = 8;
        while (warps > 1 && static_cast<size_t>(warps) * SY * 4 > 96 * 1024) warps >>= 1;
        const size_t smem = static_cast<size_t>(warps) * SY * 4;
        PMA_REQUIRE(smem <= ctx->smem_optin, PMA_ERR_ARGUMENT, "pma_edt: Y extent too large");
        const size_t rows = static_cast<size_t>(SX) * SZ;
        size_t blocks = std::min<size_t>((rows + warps - 1) / warps, static_cast<size_t>(ctx->num_sms) * 64);
        KernelTimer kt(ctx, "edt_pass_y");
        edt_pass_y<<<static_cast<unsigned>(blocks), warps * 32, smem, s>>>(edt2, SY, rows);
        ctx->check_launch("edt_pass_y");
    }
    // Pass Z with statistics. Non-crossing balls have e <= ((min extent - 1) / 2)^2.
    int minext = std::min(SX, std::min(SY, SZ));
    size_t hist_len = static_cast<size_t>((minext - 1) / 2) * ((minext - 1) / 2) + 1;
    hist_len = std::max<size_t>(hist_len, kHistSmall);
    auto* d_hist = static_cast<unsigned long long*>(ctx->scratch("edt.hist", hist_len * 8 + 16));
    auto* d_max = reinterpret_cast<unsigned int*>(d_hist + hist_len);
    PMA_CUDA(cudaMemsetAsync(d_hist, 0, hist_len * 8 + 16, s));
    {
        const size_t smem = static_cast<size_t>(SZ) * kTileY * 4 + kHistSmall * 4;
        PMA_REQUIRE(smem <= ctx->smem_optin, PMA_ERR_ARGUMENT, "pma_edt: Z extent too large");
        const size_t tiles = static_cast<size_t>(SX) * ((SY + kTileY - 1) / kTileY);
        KernelTimer kt(ctx, "edt_pass_z");
        edt_pass_z<<<static_cast<unsigned>(tiles), 256, smem, s>>>(edt2, SX, SY, SZ, d_hist,
                                                                  hist_len, d_max);
        ctx->check_launch("edt_pass_z");
    }
    unsigned int maxv = 0;
    PMA_CUDA(cudaMemcpyAsync(&maxv, d_max, 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    if (stats) {
        stats->max_edt2 = maxv;
        stats->pad_ = 0;
        stats->hist_len = static_cast<uint64_t>(maxv) + 1;
    }
    if (h_hist && hist_cap) {
        size_t want = std::min<size_t>(hist_cap, static_cast<size_t>(maxv) + 1);
        size_t have = std::min(want, hist_len);
        PMA_CUDA(cudaMemcpy(h_hist, d_hist, have * 8, cudaMemcpyDeviceToHost));
        for (size_t i = have; i < want; ++i) h_hist[i] = 0;
    }
}

// ---------------------------------------------------------------------------------------
// Allocation-free variant (pma_edt_noalloc)
//
// Some callers cannot let the library allocate device memory: an application whose own
// memory pool already holds the device's memory, or one that must not call cudaMalloc and
// cudaFree while it runs because both can synchronise the whole device and stall its other
// streams (a service answering requests on streams it owns, an interactive viewer stepping
// through volumes). Such callers also hold no pma_ctx, whose scratch cache allocates on
// first use. This variant writes its results into the caller's buffers and keeps its only
// scratch - the histogram bins and the running maximum of pass Z - in a fixed array in the
// module's global memory. Its size bounds the volumes it accepts: a 2^18-bin histogram
// covers balls up to e = 511^2, i.e. volumes whose smallest extent is at most 1024.
// ---------------------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocHistBins = size_t(1) << 18;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocDevice {
    unsigned long long* scratch = nullptr;  // address of the static array on that device
    size_t smem_optin = 0;
    int num_sms = 0;
};

std::mutex g_noalloc_mutex;
NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];

}  // namespace

// Bins [0, kNoAllocHistBins) followed by two words; the maximum sits in the first word
// after the bins in use (hist_len), as in the context-based path.
static __device__ __align__(256) unsigned long long g_edt_noalloc_scratch[kNoAllocHistBins + 2];

// Once per device, with that device current: the scratch address, the shared-memory limit
// and the SM count. Later calls read the cached values.
static NoAllocDevice noalloc_device() {
    int dev = 0;
    PMA_CUDA(cudaGetDevice(&dev));
    PMA_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, PMA_ERR_ARGUMENT,
                "pma_edt_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoAllocDevice& e = g_noalloc_devices[dev];
    if (!e.scratch) {
        void* p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_edt_noalloc_scratch);
        PMA_REQUIRE(rc == cudaSuccess && p, PMA_ERR_CUDA,
                    std::string("pma_edt_noalloc: cudaGetSymbolAddress of the scratch array failed: ") +
                        cudaGetErrorString(rc));
        int optin = 0;
        PMA_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        PMA_CUDA(cudaDeviceGetAttribute(&e.num_sms, cudaDevAttrMultiProcessorCount, dev));
        e.smem_optin = static_cast<size_t>(optin);
        e.scratch = static_cast<unsigned long long*>(p);
    }
    return e;
}

void edt_noalloc(const uint8_t* solid, pma_dims d, uint32_t* edt2, pma_edt_stats* stats,
                 uint64_t* h_hist, size_t hist_cap, cudaStream_t s) {
    check_dims(d);
    PMA_REQUIRE(solid && edt2, PMA_ERR_ARGUMENT, "pma_edt_noalloc: null device pointer");
    const int SX = d.sx, SY = d.sy, SZ = d.sz;
    const int minext = std::min(SX, std::min(SY, SZ));
    size_t hist_len = static_cast<size_t>((minext - 1) / 2) * ((minext - 1) / 2) + 1;
    hist_len = std::max<size_t>(hist_len, kHistSmall);
    PMA_REQUIRE(hist_len <= kNoAllocHistBins, PMA_ERR_LIMIT,
                "pma_edt_noalloc: smallest volume extent " + std::to_string(minext) +
                    " is above 1024, the largest its fixed 2 MiB histogram scratch covers; use pma_edt");
    const NoAllocDevice dev = noalloc_device();
    edt_smem_attributes(dev.smem_optin);

    {
        const int words = (SX + 31) / 32;
        int threads = 256;
        while (threads > 32 && static_cast<size_t>(words) * 4 * threads > 96 * 1024) threads >>= 1;
        const size_t smem = static_cast<size_t>(words) * 4 * threads;
        PMA_REQUIRE(smem <= dev.smem_optin, PMA_ERR_ARGUMENT, "pma_edt_noalloc: X extent too large");
        const size_t cols = static_cast<size_t>(SY) * SZ;
        edt_pass_x<<<div_up(cols, threads), threads, smem, s>>>(solid, edt2, SX, SY, SZ, words);
        PMA_CUDA(cudaGetLastError());
    }
    {
        int warps = 8;
        while (warps > 1 && static_cast<size_t>(warps) * SY * 4 > 96 * 1024) warps >>= 1;
        const size_t smem = static_cast<size_t>(warps) * SY * 4;
        PMA_REQUIRE(smem <= dev.smem_optin, PMA_ERR_ARGUMENT, "pma_edt_noalloc: Y extent too large");
        const size_t rows = static_cast<size_t>(SX) * SZ;
        const size_t blocks = std::min<size_t>((rows + warps - 1) / warps, static_cast<size_t>(dev.num_sms) * 64);
        edt_pass_y<<<static_cast<unsigned>(blocks), warps * 32, smem, s>>>(edt2, SY, rows);
        PMA_CUDA(cudaGetLastError());
    }
    // The bins in use and the maximum word must start at zero on every call.
    unsigned long long* d_hist = dev.scratch;
    auto* d_max = reinterpret_cast<unsigned int*>(d_hist + hist_len);
    PMA_CUDA(cudaMemsetAsync(d_hist, 0, hist_len * 8 + 16, s));
    {
        const size_t smem = static_cast<size_t>(SZ) * kTileY * 4 + kHistSmall * 4;
        PMA_REQUIRE(smem <= dev.smem_optin, PMA_ERR_ARGUMENT, "pma_edt_noalloc: Z extent too large");
        const size_t tiles = static_cast<size_t>(SX) * ((SY + kTileY - 1) / kTileY);
        edt_pass_z<<<static_cast<unsigned>(tiles), 256, smem, s>>>(edt2, SX, SY, SZ, d_hist, hist_len, d_max);
        PMA_CUDA(cudaGetLastError());
    }
    unsigned int maxv = 0;
    PMA_CUDA(cudaMemcpyAsync(&maxv, d_max, 4, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaStreamSynchronize(s));
    if (stats) {
        stats->max_edt2 = maxv;
        stats->pad_ = 0;
        stats->hist_len = static_cast<uint64_t>(maxv) + 1;
    }
    if (h_hist && hist_cap) {
        const size_t want = std::min<size_t>(hist_cap, static_cast<size_t>(maxv) + 1);
        const size_t have = std::min(want, hist_len);
        PMA_CUDA(cudaMemcpyAsync(h_hist, d_hist, have * 8, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaStreamSynchronize(s));
        for (size_t i = have; i < want; ++i) h_hist[i] = 0;
    }
}

}  // namespace pma
