// Device helpers shared by the pore and watershed stages: volume geometry, the reference's
// neighbour order and thin wrappers over CUB's order-preserving select, scan and sort.
#pragma once

#include <cub/cub.cuh>

#include "pma_internal.h"

namespace pma {

// Division of 32-bit values by a divisor fixed in advance, as a multiply-high, an add and a
// shift (the "round-up" magic-number method of Granlund and Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(m, n) + n) >> l for every n < 2^32.
struct FastDiv {
    uint32_t d = 1, m = 1, l = 0;
    FastDiv() = default;
    __host__ __device__ explicit FastDiv(uint32_t divisor) : d(divisor) {
        l = 0;
        while (l < 32 && (1ull << l) < divisor) ++l;
        m = static_cast<uint32_t>(((1ull << 32) * ((1ull << l) - divisor)) / divisor + 1);
    }
    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
        const uint32_t t = __umulhi(m, n);
#else
        const uint32_t t = static_cast<uint32_t>((static_cast<unsigned long long>(m) * n) >> 32);
#endif
        return static_cast<uint32_t>((static_cast<unsigned long long>(t) + n) >> l);
    }
};

struct Grid {
    int SX, SY, SZ;
    FastDiv fy, fx;  // division by SY and by SX
    Grid() = default;
    __host__ __device__ Grid(int sx, int sy, int sz)
        : SX(sx), SY(sy), SZ(sz), fy(static_cast<uint32_t>(sy)), fx(static_cast<uint32_t>(sx)) {}
    __host__ __device__ __forceinline__ size_t idx(int x, int y, int z) const {
        return (static_cast<size_t>(z) * SX + x) * SY + y;
    }
    // Volumes hold fewer than 2^32 voxels, so the divisions run in 32 bits, by multiplication
    // (the index-heavy kernels spend most of their instructions here otherwise).
    __host__ __device__ __forceinline__ void coords(size_t v, int& x, int& y, int& z) const {
        const uint32_t v32 = static_cast<uint32_t>(v);
        const uint32_t zx = fy.div(v32);
        y = static_cast<int>(v32 - zx * static_cast<uint32_t>(SY));
        const uint32_t zz = fx.div(zx);
        x = static_cast<int>(zx - zz * static_cast<uint32_t>(SX));
        z = static_cast<int>(zz);
    }
    __host__ __device__ __forceinline__ bool inside(int x, int y, int z) const {
        return x >= 0 && x < SX && y >= 0 && y < SY && z >= 0 && z < SZ;
    }
    __host__ __device__ __forceinline__ bool on_face(int x, int y, int z) const {
        return x == 0 || y == 0 || z == 0 || x == SX - 1 || y == SY - 1 || z == SZ - 1;
    }
};

// Neighbour j in 0..26 in the reference's loop order (x outer, then y, then z, each -1..1;
// e.g. PoreAndThroatComputer.cpp:228-234). Returns false for the centre and, with D3Q7,
// for diagonal offsets (ModelUtilities.h:295-302).
__device__ __forceinline__ bool stencil_offset(int j, bool d3q7, int& dx, int& dy, int& dz) {
    dx = j / 9 - 1;
    dy = (j / 3) % 3 - 1;
    dz = j % 3 - 1;
    if (j == 13) return false;
    if (d3q7 && (dx != 0) + (dy != 0) + (dz != 0) > 1) return false;
    return true;
}

// Two independent 64-bit hashes of an id sequence (FNV-1a and a multiply-xorshift stream).
// Sets are compared by both hashes and then verified element by element.
__device__ __forceinline__ void list_hash(const uint32_t* a, uint32_t n, unsigned long long& h1,
                                          unsigned long long& h2) {
    h1 = 1469598103934665603ull ^ n;
    h2 = 0x9E3779B97F4A7C15ull + n;
    for (uint32_t i = 0; i < n; ++i) {
        h1 = (h1 ^ a[i]) * 1099511628211ull;
        h2 = (h2 + a[i] + 0x632BE59BD9B4E019ull) * 0xD6E8FEB86659FD93ull;
        h2 ^= h2 >> 32;
    }
}

// --- CUB wrappers (all on ctx->stream; temporary storage cached in the context) ----------

template <class InIt, class T>
inline int64_t select_flagged(pma_ctx* ctx, InIt in, const uint8_t* flags, T* out, int64_t n,
                              int64_t* d_count) {
    size_t bytes = 0;
    PMA_CUDA(cub::DeviceSelect::Flagged(nullptr, bytes, in, flags, out, d_count, n, ctx->stream));
    void* tmp = ctx->scratch("cub.tmp", bytes);
    PMA_CUDA(cub::DeviceSelect::Flagged(tmp, bytes, in, flags, out, d_count, n, ctx->stream));
    int64_t* h = ctx->pinned_count();
    PMA_CUDA(cudaMemcpyAsync(h, d_count, sizeof(*h), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->count_launch(1);
    return *h;
}

template <class T>
inline void exclusive_sum(pma_ctx* ctx, const T* in, T* out, int64_t n) {
    size_t bytes = 0;
    PMA_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, ctx->stream));
    void* tmp = ctx->scratch("cub.tmp", bytes);
    PMA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, n, ctx->stream));
    ctx->count_launch(1);
}

template <class K, class V>
inline void sort_pairs(pma_ctx* ctx, const K* kin, K* kout, const V* vin, V* vout, int64_t n,
                       int end_bit = sizeof(K) * 8) {
    size_t bytes = 0;
    PMA_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, n, 0, end_bit,
                                             ctx->stream));
    void* tmp = ctx->scratch("cub.tmp", bytes);
    PMA_CUDA(cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, n, 0, end_bit,
                                             ctx->stream));
    ctx->count_launch(1);
}

template <class K>
inline void sort_keys(pma_ctx* ctx, const K* kin, K* kout, int64_t n, int end_bit = sizeof(K) * 8) {
    size_t bytes = 0;
    PMA_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, bytes, kin, kout, n, 0, end_bit, ctx->stream));
    void* tmp = ctx->scratch("cub.tmp", bytes);
    PMA_CUDA(cub::DeviceRadixSort::SortKeys(tmp, bytes, kin, kout, n, 0, end_bit, ctx->stream));
    ctx->count_launch(1);
}

template <class T>
inline int64_t unique(pma_ctx* ctx, const T* in, T* out, int64_t n, int64_t* d_count) {
    size_t bytes = 0;
    PMA_CUDA(cub::DeviceSelect::Unique(nullptr, bytes, in, out, d_count, n, ctx->stream));
    void* tmp = ctx->scratch("cub.tmp", bytes);
    PMA_CUDA(cub::DeviceSelect::Unique(tmp, bytes, in, out, d_count, n, ctx->stream));
    int64_t* h = ctx->pinned_count();
    PMA_CUDA(cudaMemcpyAsync(h, d_count, sizeof(*h), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->count_launch(1);
    return *h;
}

inline unsigned grid_for(pma_ctx* ctx, size_t n, int threads = 256) {
    size_t b = (n + threads - 1) / threads;
    size_t cap = static_cast<size_t>(ctx->num_sms) * 32;
    if (b > cap) b = cap;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

#define PMA_GRID_STRIDE(i, n)                                                             \
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < (n); \
         i += static_cast<size_t>(gridDim.x) * blockDim.x)

// Pore-id sequence of the reference: 127, 128, ... skipping past multiples of 255
// (PoreAndThroatComputer.cpp:60, 149-153).
inline std::vector<uint32_t> pore_id_sequence(size_t n) {
    std::vector<uint32_t> ids(n);
    uint32_t id = 127;
    for (size_t i = 0; i < n; ++i) {
        ids[i] = id;
        id += (id % 255 == 0) ? 127 : 1;
    }
    return ids;
}

// Small device-to-host reads of loop counters: a one-block kernel stores the words straight
// into pinned (mapped) host memory, then the stream is synchronised. Unlike cudaMemcpyAsync,
// the read does not queue on a copy engine behind large transfers of other streams (the
// pipeline's side-stream result copies), and one launch covers several sources.
struct ReadBack {
    const void* src[4] = {};
    void* dst[4] = {};
    unsigned words[4] = {};  // 4-byte words
    int n = 0;
    void add(void* host_dst, const void* dev_src, size_t bytes) {
        PMA_REQUIRE(n < 4, PMA_ERR_INTERNAL, "read-back of more than four arrays");
        src[n] = dev_src;
        dst[n] = host_dst;
        words[n] = static_cast<unsigned>(bytes / 4);
        ++n;
    }
};

namespace {  // one copy per translation unit

__global__ void read_back_kernel(ReadBack rb) {
    for (int k = 0; k < rb.n; ++k)
        for (unsigned i = threadIdx.x; i < rb.words[k]; i += blockDim.x)
            static_cast<volatile uint32_t*>(rb.dst[k])[i] = __ldcg(static_cast<const uint32_t*>(rb.src[k]) + i);
    __threadfence_system();
}

inline void read_back(pma_ctx* ctx, ReadBack rb) {
    for (int k = 0; k < rb.n; ++k) {
        void* d = nullptr;
        PMA_CUDA(cudaHostGetDevicePointer(&d, rb.dst[k], 0));
        rb.dst[k] = d;
    }
    read_back_kernel<<<1, 64, 0, ctx->stream>>>(rb);
    ctx->count_launch();
    ctx->check_launch("read_back");
    ctx->sync();
}

}  // namespace

}  // namespace pma
