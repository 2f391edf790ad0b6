// Geodesic (shortest-path) distances, cavity ids and cavity restarts
// (ShortestPathComputer.cpp:39-511).
//
// The reference settles voxels with Dijkstra over an indexed heap (HeapUtilities.h).
// Every settled distance equals min over void neighbours u of fl(d(u) + w(u, v)); this
// system has one greatest fixed point below the initial values and any monotone
// relaxation that runs until nothing improves reaches it, so the parallel form below is
// bit-identical in float32 (and in float64 against the float64 restatement).
//
// Bucketing: all step weights w are >= 1 (1, sqrt 2, sqrt 3, or 1 for D3Q7) and in
// round-to-nearest fl(d + w) >= floor(d) + 1, so relaxing a voxel of bucket floor(d) = k
// only reaches buckets k+1 and k+2. Bucket k is therefore final when it is processed and
// one parallel sweep per bucket suffices (Dial's algorithm). Buckets are a ring of four
// bitmaps over the voxels (a voxel is set in bucket b's bitmap when its distance drops into
// b); before its sweep, bucket k's bitmap is compacted into a list in voxel order (per block
// of 8192 voxels), which is also cleared for bucket k + 4. A voxel whose distance dropped to a
// lower bucket after being set is skipped as stale.
#include "devutil.cuh"

#include <cfloat>
#include <cmath>
#include <cstring>

namespace pma {
namespace {

template <class T> struct Bits;
template <> struct Bits<float> {
    typedef unsigned int U;
    static __device__ __forceinline__ U to(float f) { return __float_as_uint(f); }
    static __device__ __forceinline__ float from(U u) { return __uint_as_float(u); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __host__ __device__ float unknown() { return FLT_MAX; }
    static __device__ __forceinline__ int bucket(float d) { return static_cast<int>(floorf(d)); }
};
template <> struct Bits<double> {
    typedef unsigned long long U;
    static __device__ __forceinline__ U to(double f) { return static_cast<U>(__double_as_longlong(f)); }
    static __device__ __forceinline__ double from(U u) { return __longlong_as_double(static_cast<long long>(u)); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __host__ __device__ double unknown() { return DBL_MAX; }
    static __device__ __forceinline__ int bucket(double d) { return static_cast<int>(floor(d)); }
};

struct Geo {
    int SX, SY, SZ;
    FastDiv fy, fx;  // division by SY and by SX (multiply-high)
    Geo() = default;
    Geo(int sx, int sy, int sz) : SX(sx), SY(sy), SZ(sz), fy(static_cast<uint32_t>(sy)), fx(static_cast<uint32_t>(sx)) {}
    __device__ __forceinline__ size_t idx(int x, int y, int z) const {
        return (static_cast<size_t>(z) * SX + x) * SY + y;
    }
};

// Compaction chunks: 256 bitmap words (8192 voxels), one block step of geo_compact.
constexpr int kChunkWords = 256;
constexpr int kChunkShift = 13;  // voxel index -> chunk

struct Frontier {
    uint32_t* bits;        // four bitmaps of nwords words: bucket b uses bitmap b & 3
    size_t nwords;
    uint8_t* dirty;        // four flag arrays of nchunks bytes: a bit was set in the chunk
    size_t nchunks;
    unsigned int* count;   // [4] non-zero when a voxel was marked in that bitmap
    uint32_t* list;        // the compacted bucket being swept
    unsigned int* list_n;  // its length
    uint32_t cap;          // list capacity
    unsigned int* overflow;
    unsigned long long* settled;  // voxels settled in this cavity
    unsigned int* walls;          // bit 2i: plane axis i at 0, bit 2i+1: at size-1
};

template <class T>
__global__ void geo_init(const uint8_t* __restrict__ solid, size_t n, T* __restrict__ dist,
                         uint32_t* __restrict__ cavity) {
    for (size_t v = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; v < n;
         v += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const bool s = solid[v] != 0;  // SPC.cpp:354-372
        dist[v] = s ? static_cast<T>(-1) : Bits<T>::unknown();
        cavity[v] = s ? 0u : 0xFFFFFFFFu;
    }
}

template <class T>
__global__ void geo_start(Frontier f, T* dist, uint32_t v) {
    dist[v] = static_cast<T>(0);
    f.bits[v >> 5] |= 1u << (v & 31);  // bucket 0
    f.dirty[v >> kChunkShift] = 1;
    f.count[0] = 1;
}

// Bucket k's bitmap -> list (voxel order within each block's 8192 voxels), cleared behind.
// Only chunks whose flag is set are read: a bucket is a thin shell of the volume, and reading
// the whole bitmap for each bucket took a quarter of the geodesic kernels' time at 512^3.
__global__ void __launch_bounds__(kChunkWords) geo_compact(Frontier f, int k) {
    __shared__ unsigned int wsum[kChunkWords / 32];
    __shared__ unsigned int base;
    uint32_t* bm = f.bits + static_cast<size_t>(k & 3) * f.nwords;
    uint8_t* dirty = f.dirty + static_cast<size_t>(k & 3) * f.nchunks;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (size_t ch = blockIdx.x; ch < f.nchunks; ch += gridDim.x) {
        if (!dirty[ch]) continue;  // the same byte for the whole block: a uniform skip
        const size_t w = ch * kChunkWords + threadIdx.x;
        uint32_t word = 0;
        if (w < f.nwords) {
            word = bm[w];
            if (word) bm[w] = 0;
        }
        const unsigned c = __popc(word);
        unsigned incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<unsigned>(o)) incl += t;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();  // every thread has read the flag
        if (threadIdx.x == 0) {
            dirty[ch] = 0;
            unsigned tot = 0;
            for (int i = 0; i < kChunkWords / 32; ++i) {
                const unsigned v = wsum[i];
                wsum[i] = tot;
                tot += v;
            }
            base = tot ? atomicAdd(f.list_n, tot) : 0u;
        }
        __syncthreads();
        unsigned pos = base + wsum[warp] + incl - c;
        while (word) {
            const int bit = __ffs(word) - 1;
            word &= word - 1;
            if (pos < f.cap) f.list[pos] = static_cast<uint32_t>(w * 32 + bit);
            else atomicExch(f.overflow, 1u);
            ++pos;
        }
        __syncthreads();
    }
}

// Processes bucket k: settle its voxels and relax their neighbours. One thread per list
// entry: it reads its own distance, then issues the loads of all its neighbours' distances at
// once (26 independent loads in flight per thread hide their latency; the list is in voxel
// order, so a warp's loads of one stencil position fall on neighbouring addresses), then
// lowers the neighbours it improves. Each voxel is in the list once, so a live entry
// (bucket(dist) == k) is settled exactly once. Steps are in [1, 2), so pushes go to buckets
// k + 1 and k + 2 only; whether a bucket got any is flagged per warp at the end (the host
// only asks whether the next buckets are empty).
// Four blocks per SM (64 registers; the float64 form spills about 100 bytes to L1): more
// warps hide more of the neighbour loads' latency than the spilled registers cost (the float64
// bucket loop of the 1024^3 spinodal: 338 ms at 120 registers, 299 ms at three blocks per SM,
// 294 ms at four).
template <class T, bool D3Q7>
__global__ void __launch_bounds__(256, 4) geo_bucket(Geo g, T w1, T w2, T w3, T* __restrict__ dist,
                                                  uint32_t* __restrict__ cavity, Frontier f, int k,
                                                  uint32_t cavity_id) {
    typedef typename Bits<T>::U U;
    const unsigned n = min(*f.list_n, f.cap);
    const uint32_t* list = f.list;
    const long long sy = g.SY, sxy = static_cast<long long>(g.SX) * g.SY;
    unsigned long long my_settled = 0;
    unsigned my_walls = 0, c1 = 0, c2 = 0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = list[i];
        const T dv = dist[v];
        if (Bits<T>::bucket(dv) != k) continue;  // stale: the voxel moved to a lower bucket
        const uint32_t zx = g.fy.div(v);
        const int y = static_cast<int>(v - zx * static_cast<uint32_t>(g.SY));
        const uint32_t zz = g.fx.div(zx);
        const int x = static_cast<int>(zx - zz * static_cast<uint32_t>(g.SX));
        const int z = static_cast<int>(zz);
        cavity[v] = cavity_id;
        ++my_settled;
        const bool xl = x > 0, xh = x < g.SX - 1, yl = y > 0, yh = y < g.SY - 1, zl = z > 0, zh = z < g.SZ - 1;
        if (!xl) my_walls |= 1u;
        if (!xh && g.SX > 1) my_walls |= 2u;
        if (!yl) my_walls |= 4u;
        if (!yh && g.SY > 1) my_walls |= 8u;
        if (!zl) my_walls |= 16u;
        if (!zh && g.SZ > 1) my_walls |= 32u;
        const T nd1 = Bits<T>::add(dv, D3Q7 ? static_cast<T>(1) : w1);
        const T nd2 = Bits<T>::add(dv, w2), nd3 = Bits<T>::add(dv, w3);
        T nb[27];
#pragma unroll
        for (int j = 0; j < 27; ++j) {
            const int dx = j / 9 - 1, dy = (j / 3) % 3 - 1, dz = j % 3 - 1;
            const int kk = dx * dx + dy * dy + dz * dz;
            if (kk == 0 || (D3Q7 && kk != 1)) continue;
            const bool ok = (dx < 0 ? xl : (dx > 0 ? xh : true)) && (dy < 0 ? yl : (dy > 0 ? yh : true)) &&
                            (dz < 0 ? zl : (dz > 0 ? zh : true));
            // out of the box reads as -1, like a solid voxel: never improved
            nb[j] = ok ? dist[static_cast<long long>(v) + dz * sxy + dx * sy + dy] : static_cast<T>(-1);
        }
#pragma unroll
        for (int j = 0; j < 27; ++j) {
            const int dx = j / 9 - 1, dy = (j / 3) % 3 - 1, dz = j % 3 - 1;
            const int kk = dx * dx + dy * dy + dz * dz;
            if (kk == 0 || (D3Q7 && kk != 1)) continue;
            const T nd = kk == 1 ? nd1 : (kk == 2 ? nd2 : nd3);
            if (nd < nb[j]) {
                // Neither update waits for its old value (reductions, no round trip): the bit
                // marks the voxel in nd's bucket even when another thread has lowered it further
                // meanwhile, and such an entry is skipped as stale when its bucket comes (the
                // lowest value's bucket has its bit from the thread that wrote that value).
                const size_t w = static_cast<size_t>(static_cast<long long>(v) + dz * sxy + dx * sy + dy);
                atomicMin(reinterpret_cast<U*>(dist + w), Bits<T>::to(nd));
                const int pb = Bits<T>::bucket(nd);
                const uint32_t bit = 1u << (w & 31);
                atomicOr(&f.bits[static_cast<size_t>(pb & 3) * f.nwords + (w >> 5)], bit);
                f.dirty[static_cast<size_t>(pb & 3) * f.nchunks + (w >> kChunkShift)] = 1;
                if (pb == k + 1) c1 = 1;
                else if (pb == k + 2) c2 = 1;
                else atomicOr(&f.count[pb & 3], 1u);  // not reachable with steps in [1, 2)
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        my_settled += __shfl_xor_sync(0xFFFFFFFFu, my_settled, o);
        my_walls |= __shfl_xor_sync(0xFFFFFFFFu, my_walls, o);
        c1 |= __shfl_xor_sync(0xFFFFFFFFu, c1, o);
        c2 |= __shfl_xor_sync(0xFFFFFFFFu, c2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (my_settled) atomicAdd(f.settled, my_settled);
        if (my_walls) atomicOr(f.walls, my_walls);
        if (c1) atomicOr(&f.count[(k + 1) & 3], 1u);
        if (c2) atomicOr(&f.count[(k + 2) & 3], 1u);
    }
}

// Before bucket k is compacted: empty the list and its bitmap count.
__global__ void geo_next(Frontier f, int k) {
    *f.list_n = 0;
    f.count[k & 3] = 0;
}

// Start-voxel search on box shells h0 .. h0+nh-1 around the centre, in the reference's
// visiting order (SPC.cpp:460-511). Writes the smallest (shell, order) key of a void,
// unreached voxel.
template <class T>
__global__ void geo_shell_search(const uint8_t* __restrict__ solid, const T* __restrict__ dist,
                                 Geo g, int cx, int cy, int cz, int h0, int nh,
                                 unsigned long long* __restrict__ best) {
    const int s[3] = {g.SX, g.SY, g.SZ};
    const int c[3] = {cx, cy, cz};
    const int h = h0 + blockIdx.y;
    if (blockIdx.y >= nh) return;
    // segment sizes in order (k, f)
    unsigned long long off = 0;
    unsigned long long t = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    for (int k = 0; k < 3; ++k) {
        const int a = (k == 0) ? 1 : 0, b = (k == 2) ? 1 : 2;
        const int a0 = max(c[a] - h, 0), a1 = min(c[a] + h, s[a] - 1);
        const int b0 = max(c[b] - h, 0), b1 = min(c[b] + h, s[b] - 1);
        const int f0 = max(c[k] - h, 0), f1 = min(c[k] + h, s[k] - 1);
        const int nf = (f0 == f1) ? 1 : 2;
        const unsigned long long na = a1 - a0 + 1, nb = b1 - b0 + 1;
        const unsigned long long seg = static_cast<unsigned long long>(nf) * na * nb;
        for (unsigned long long i = t; i < seg; i += gridDim.x * static_cast<unsigned long long>(blockDim.x)) {
            const int f = static_cast<int>(i / (na * nb));
            const unsigned long long r = i % (na * nb);
            int p[3];
            p[a] = a0 + static_cast<int>(r / nb);
            p[b] = b0 + static_cast<int>(r % nb);
            p[k] = f == 0 ? f0 : f1;
            const size_t v = g.idx(p[0], p[1], p[2]);
            if (solid[v] == 0 && dist[v] == Bits<T>::unknown())
                atomicMin(best, (static_cast<unsigned long long>(blockIdx.y) << 40) | (off + i));
        }
        off += seg;
    }
}

}  // namespace

template <class T>
std::vector<pma_cavity> geodesic(pma_ctx* ctx, const uint8_t* solid, pma_dims d, pma_stencil st, T* dist,
                                 uint32_t* cavity) {
    KernelTimer kt_stage(ctx, "stage_geodesic");  // the whole stage, for the untimed remainder
    check_dims(d);
    PMA_REQUIRE(solid && dist && cavity, PMA_ERR_ARGUMENT, "pma_geodesic: null device pointer");
    cudaStream_t s = ctx->stream;
    const size_t n = voxels(d);
    const Geo g{d.sx, d.sy, d.sz};
    const int d3q7 = st == PMA_D3Q7 ? 1 : 0;
    const T w1 = std::sqrt(static_cast<T>(1)), w2 = std::sqrt(static_cast<T>(2)),
            w3 = std::sqrt(static_cast<T>(3));  // SPC.cpp:31-36
    const unsigned grid = static_cast<unsigned>(std::min<size_t>(div_up(n, 256), ctx->num_sms * 16ull));

    const uint32_t cap = static_cast<uint32_t>(std::min<size_t>(n, size_t(1) << 28));
    const size_t nwords = (n + 31) / 32;
    auto* bits = static_cast<uint32_t*>(ctx->scratch("geo.bits", 4 * nwords * 4));
    const size_t nchunks = (nwords + kChunkWords - 1) / kChunkWords;
    auto* dirty = static_cast<uint8_t*>(ctx->scratch("geo.dirty", 4 * nchunks));
    auto* list = static_cast<uint32_t*>(ctx->scratch("geo.list", static_cast<size_t>(cap) * 4));
    auto* misc = static_cast<unsigned long long*>(ctx->scratch("geo.misc", 64));
    Frontier f;
    f.bits = bits;
    f.nwords = nwords;
    f.dirty = dirty;
    f.nchunks = nchunks;
    f.list = list;
    f.count = reinterpret_cast<unsigned int*>(misc);          // 4 x u32 = misc[0..1]
    f.overflow = reinterpret_cast<unsigned int*>(misc + 2);   // misc[2] low
    f.walls = reinterpret_cast<unsigned int*>(misc + 3);      // misc[3] low
    f.settled = misc + 4;
    unsigned long long* best = misc + 5;
    f.list_n = reinterpret_cast<unsigned int*>(misc + 6);     // misc[6] low
    f.cap = cap;
    PMA_CUDA(cudaMemsetAsync(bits, 0, 4 * nwords * 4, s));
    PMA_CUDA(cudaMemsetAsync(dirty, 0, 4 * nchunks, s));

    geo_init<T><<<grid, 256, 0, s>>>(solid, n, dist, cavity);
    ctx->check_launch("geo_init");

    // SPC.cpp:443-458: centre = round(size * 0.5) clipped to size - 1.
    int sz3[3] = {d.sx, d.sy, d.sz}, c[3];
    for (int i = 0; i < 3; ++i) c[i] = std::min(static_cast<int>(sz3[i] * 0.5 + 0.5), sz3[i] - 1);
    int maxh = 0;
    for (int i = 0; i < 3; ++i) maxh = std::max(maxh, std::max(sz3[i] - 1 - c[i], c[i]));
    int walls_total = 0;
    for (int i = 0; i < 3; ++i) walls_total += (sz3[i] == 1) ? 1 : 2;
    const size_t center_idx = (static_cast<size_t>(c[2]) * d.sx + c[0]) * d.sy + c[1];

    auto* h = static_cast<unsigned long long*>(ctx->host_staging(64));
    int half = 0;
    uint32_t cavity_id = 0;
    std::vector<pma_cavity> rows;
    const int max_buckets_per_sync = 32;
    const uint64_t bucket_limit = ctx->limits.geodesic_buckets ? ctx->limits.geodesic_buckets : 2ull * n + 64;
    const unsigned bucket_grid = static_cast<unsigned>(ctx->num_sms * 8);
    const unsigned compact_grid = static_cast<unsigned>(std::min<size_t>(nchunks, ctx->num_sms * 8ull));
    while (true) {  // SPC.cpp:94-140
        ++half;
        // SelectStartingPosition (SPC.cpp:396-426)
        bool found = false;
        int start[3] = {0, 0, 0};
        {
            uint8_t sv = 1;
            T dv = 0;
            PMA_CUDA(cudaMemcpyAsync(&sv, solid + center_idx, 1, cudaMemcpyDeviceToHost, s));
            PMA_CUDA(cudaMemcpyAsync(&dv, dist + center_idx, sizeof(T), cudaMemcpyDeviceToHost, s));
            ctx->sync();
            if (sv == 0 && dv == Bits<T>::unknown()) {
                found = true;
                for (int i = 0; i < 3; ++i) start[i] = c[i];
            }
        }
        while (!found && half < maxh) {
            const int nh = std::min(16, maxh - half);
            PMA_CUDA(cudaMemsetAsync(best, 0xFF, 8, s));
            unsigned long long face = 2ull * std::max(d.sx, std::max(d.sy, d.sz)) *
                                      std::max(d.sx, std::max(d.sy, d.sz));
            unsigned gx = static_cast<unsigned>(std::min<unsigned long long>((face + 255) / 256, 4096));
            geo_shell_search<T><<<dim3(gx, nh), 256, 0, s>>>(solid, dist, g, c[0], c[1], c[2], half, nh, best);
            ctx->check_launch("geo_shell_search");
            PMA_CUDA(cudaMemcpyAsync(h, best, 8, cudaMemcpyDeviceToHost, s));
            ctx->sync();
            const unsigned long long b = h[0];
            if (b == ~0ull) {
                half += nh;
                continue;
            }
            half += static_cast<int>(b >> 40);
            unsigned long long flat = b & ((1ull << 40) - 1);
            // decode in the same segment order as the kernel
            for (int k = 0; k < 3 && !found; ++k) {
                const int a = (k == 0) ? 1 : 0, bb = (k == 2) ? 1 : 2;
                const int a0 = std::max(c[a] - half, 0), a1 = std::min(c[a] + half, sz3[a] - 1);
                const int b0 = std::max(c[bb] - half, 0), b1 = std::min(c[bb] + half, sz3[bb] - 1);
                const int f0 = std::max(c[k] - half, 0), f1 = std::min(c[k] + half, sz3[k] - 1);
                const int nf = (f0 == f1) ? 1 : 2;
                const unsigned long long na = a1 - a0 + 1, nb = b1 - b0 + 1, seg = nf * na * nb;
                if (flat < seg) {
                    const int fi = static_cast<int>(flat / (na * nb));
                    const unsigned long long r = flat % (na * nb);
                    start[a] = a0 + static_cast<int>(r / nb);
                    start[bb] = b0 + static_cast<int>(r % nb);
                    start[k] = fi == 0 ? f0 : f1;
                    found = true;
                } else {
                    flat -= seg;
                }
            }
            PMA_REQUIRE(found, PMA_ERR_INTERNAL, "geodesic: shell search decode failed");
        }
        if (!found) break;

        cavity_id += 127;
        PMA_CUDA(cudaMemsetAsync(misc, 0, 5 * 8, s));  // counts, overflow, walls, settled
        const size_t sidx = (static_cast<size_t>(start[2]) * d.sx + start[0]) * d.sy + start[1];
        geo_start<T><<<1, 1, 0, s>>>(f, dist, static_cast<uint32_t>(sidx));
        ctx->check_launch("geo_start");
        int k = 0;
        while (true) {
            KernelTimer kt(ctx, "geo_bucket");
            for (int i = 0; i < max_buckets_per_sync; ++i, ++k) {
                geo_next<<<1, 1, 0, s>>>(f, k);
                geo_compact<<<compact_grid, kChunkWords, 0, s>>>(f, k);
                if (d3q7) geo_bucket<T, true><<<bucket_grid, 256, 0, s>>>(g, w1, w2, w3, dist, cavity, f, k, cavity_id);
                else geo_bucket<T, false><<<bucket_grid, 256, 0, s>>>(g, w1, w2, w3, dist, cavity, f, k, cavity_id);
            }
            ctx->count_launch(3 * max_buckets_per_sync - 1);
            ctx->check_launch("geo_bucket");
            {
                ReadBack rb;
                rb.add(h, misc, 3 * 8);
                read_back(ctx, rb);
            }
            const unsigned* cnt = reinterpret_cast<const unsigned*>(h);
            PMA_REQUIRE(reinterpret_cast<const unsigned*>(h)[4] == 0, PMA_ERR_LIMIT,
                        "geodesic: frontier list overflow");
            // after bucket k-1: lists of buckets k and k+1 hold all pending work
            if (cnt[k & 3] == 0 && cnt[(k + 1) & 3] == 0) break;
            // Distances are below 2 per voxel step, so no bucket index can exceed 2n.
            PMA_REQUIRE(static_cast<uint64_t>(k) <= bucket_limit, PMA_ERR_LIMIT,
                        "geodesic: bucket sweep did not terminate");
        }
        {
            ReadBack rb;
            rb.add(h, misc, 5 * 8);
            read_back(ctx, rb);
        }
        ctx->count("geo.buckets", k);
        const unsigned walls_bits = static_cast<unsigned>(h[3]);
        const unsigned long long settled = h[4];
        const int reached = __builtin_popcount(walls_bits);
        {  // SPC.cpp:143-164: one row per cavity, however many there are
            pma_cavity o;
            std::memset(&o, 0, sizeof(o));
            o.id = cavity_id;
            o.seed_x = start[0];
            o.seed_y = start[1];
            o.seed_z = start[2];
            o.reached_walls = reached;
            o.reaches_all_walls = reached == walls_total ? 1 : 0;
            o.void_count = settled;
            const int dx = start[0] - c[0], dy = start[1] - c[1], dz = start[2] - c[2];
            o.distance_to_center = static_cast<float>(std::sqrt(static_cast<double>(dx * dx + dy * dy + dz * dz)));
            rows.push_back(o);
        }
        if (reached == walls_total) break;
    }
    return rows;
}

template std::vector<pma_cavity> geodesic<float>(pma_ctx*, const uint8_t*, pma_dims, pma_stencil, float*,
                                                 uint32_t*);
template std::vector<pma_cavity> geodesic<double>(pma_ctx*, const uint8_t*, pma_dims, pma_stencil, double*,
                                                  uint32_t*);

}  // namespace pma
