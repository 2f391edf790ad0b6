// Containing-ball radii, winning centres and the maximum-ball mask
// (ContainingBallsAssigner.cpp:101-250).
//
// Single-thread semantics of the reference: centres are visited in x, y, z order and a
// voxel takes a new centre only on a strictly larger squared radius, so each void voxel
// ends with the largest r^2 covering it and, among those, the lexicographically smallest
// (x, y, z) centre. Both orders fit one 64-bit key,
//     key = (r^2 << 32) | (0xFFFFFFFF - ((x * SY + y) * SZ + z)),
// and the result is the atomicMax of keys over covering balls, whatever the order.
//
// Work reduction: a centre whose discrete ball lies inside the ball of one of its 26
// neighbours can never win a voxel (the neighbour covers the same voxels with a strictly
// larger radius), so it is not scattered. Containment B(c, R) in B(c + e, R') holds iff
// R' >= M_k(R) = max over lattice v with |v|^2 <= R of |v + e|^2, k = |e|^2; the table
// M_k is computed exactly for R <= kExactTable and replaced above it by the continuous
// sufficient condition (sqrt(R) + sqrt(k))^2 <= R'. Surviving centres are bucketed by
// r^2 and scattered largest first, so most reads find a larger key already in place and
// skip the atomic.
#include "pma_internal.h"

namespace pma {
namespace {

constexpr uint32_t kExactTable = 1u << 16;

__device__ __forceinline__ uint32_t isqrt_u32(uint32_t n) {
    uint32_t r = static_cast<uint32_t>(sqrtf(static_cast<float>(n)));
    while (r * r > n) --r;
    while ((r + 1) * (r + 1) <= n) ++r;
    return r;
}

// M_k(R) for k = 1, 2, 3, one thread per R.
__global__ void balls_containment_table(uint32_t* __restrict__ m1, uint32_t* __restrict__ m2,
                                        uint32_t* __restrict__ m3, uint32_t nR) {
    const uint32_t R = blockIdx.x * blockDim.x + threadIdx.x;
    if (R >= nR) return;
    uint32_t b1 = 0, b2 = 0, b3 = 0;
    const uint32_t amax = isqrt_u32(R);
    for (uint32_t a = 0; a <= amax; ++a) {
        const uint32_t ra = R - a * a;
        const uint32_t bmax = isqrt_u32(ra);
        for (uint32_t b = 0; b <= bmax; ++b) {
            const uint32_t c = isqrt_u32(ra - b * b);
            const uint32_t a1 = (a + 1) * (a + 1), bb = b * b, b1s = (b + 1) * (b + 1);
            const uint32_t cc = c * c, c1 = (c + 1) * (c + 1);
            const uint32_t v1 = a1 + bb + cc, v2 = a1 + b1s + cc, v3 = a1 + b1s + c1;
            b1 = v1 > b1 ? v1 : b1;
            b2 = v2 > b2 ? v2 : b2;
            b3 = v3 > b3 ? v3 : b3;
        }
    }
    m1[R] = b1;
    m2[R] = b2;
    m3[R] = b3;
}

struct Geo {
    int SX, SY, SZ;
    __device__ __forceinline__ size_t idx(int x, int y, int z) const {
        return (static_cast<size_t>(z) * SX + x) * SY + y;
    }
};

__device__ __forceinline__ bool dominated(const uint32_t* __restrict__ edt2, Geo g, int x, int y,
                                          int z, uint32_t R, const uint32_t* __restrict__ mtab,
                                          uint32_t ntab) {
    for (int dz = -1; dz <= 1; ++dz) {
        const int nz = z + dz;
        if (nz < 0 || nz >= g.SZ) continue;
        for (int dx = -1; dx <= 1; ++dx) {
            const int nx = x + dx;
            if (nx < 0 || nx >= g.SX) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int ny = y + dy;
                if (ny < 0 || ny >= g.SY) continue;
                const int k = dx * dx + dy * dy + dz * dz;
                if (k == 0) continue;
                const uint32_t Rn = __ldg(edt2 + g.idx(nx, ny, nz));
                if (Rn <= R) continue;
                if (R < ntab) {
                    if (Rn >= __ldg(mtab + (k - 1) * ntab + R)) return true;
                } else {
                    // (sqrt(R) + sqrt(k))^2 <= Rn  <=>  t >= 0 and t^2 >= 4kR, t = Rn - R - k
                    const long long t = static_cast<long long>(Rn) - R - k;
                    if (t >= 0 && static_cast<unsigned long long>(t) * t >=
                                      4ull * static_cast<unsigned long long>(k) * R)
                        return true;
                }
            }
        }
    }
    return false;
}

// Pass 1 (count) and pass 2 (place) of the counting sort of surviving centres by r^2.
template <bool kPlace>
__global__ void balls_candidates(const uint32_t* __restrict__ edt2, Geo g, size_t n,
                                 const uint32_t* __restrict__ mtab, uint32_t ntab, uint32_t nR,
                                 uint32_t* __restrict__ counts, uint32_t* __restrict__ cursor,
                                 uint32_t* __restrict__ list, unsigned long long* __restrict__ keys,
                                 unsigned int* __restrict__ err) {
    for (size_t v = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; v < n;
         v += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const uint32_t R = edt2[v];
        if (!kPlace) keys[v] = (R == 0) ? ~0ull : 0ull;  // solid voxels never change
        if (R == 0) continue;
        if (R >= nR) {  // max_edt2 below the data: refuse rather than index past counts
            atomicOr(err, 1u);
            continue;
        }
        const int y = static_cast<int>(v % g.SY);
        const size_t zx = v / g.SY;
        const int x = static_cast<int>(zx % g.SX);
        const int z = static_cast<int>(zx / g.SX);
        if (dominated(edt2, g, x, y, z, R, mtab, ntab)) continue;
        if (kPlace) list[atomicAdd(&cursor[R], 1u)] = static_cast<uint32_t>(v);
        else atomicAdd(&counts[R], 1u);
    }
}

// Exclusive scan of counts in descending r^2 order: cursor[R] = sum of counts[R' > R].
// One block; nR is at most max_edt2 + 1.
__global__ void balls_bucket_offsets(const uint32_t* __restrict__ counts, uint32_t* __restrict__ cursor,
                                     uint32_t nR, uint32_t* __restrict__ total) {
    __shared__ unsigned long long part[1024];
    const uint32_t per = (nR + blockDim.x - 1) / blockDim.x;
    // thread t owns the descending range [nR-1 - t*per, ...)
    unsigned long long s = 0;
    for (uint32_t i = 0; i < per; ++i) {
        long long R = static_cast<long long>(nR) - 1 - (static_cast<long long>(threadIdx.x) * per + i);
        if (R >= 0) s += counts[R];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (unsigned t = 0; t < blockDim.x; ++t) {
            unsigned long long c = part[t];
            part[t] = run;
            run += c;
        }
        *total = static_cast<uint32_t>(run);
    }
    __syncthreads();
    unsigned long long run = part[threadIdx.x];
    for (uint32_t i = 0; i < per; ++i) {
        long long R = static_cast<long long>(nR) - 1 - (static_cast<long long>(threadIdx.x) * per + i);
        if (R >= 0) {
            cursor[R] = static_cast<uint32_t>(run);
            run += counts[R];
        }
    }
}

// Scatter: warps take centres in list order (largest r^2 first). Lanes split into groups
// of G; a group walks one y-span of the ball at a time.
__global__ void balls_scatter(const uint32_t* __restrict__ edt2, Geo g,
                              const uint32_t* __restrict__ list, uint32_t total,
                              unsigned int* __restrict__ next, unsigned long long* __restrict__ keys) {
    const int lane = threadIdx.x & 31;
    while (true) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(next, 1u);
        item = __shfl_sync(0xFFFFFFFFu, item, 0);
        if (item >= total) return;
        const uint32_t v = list[item];
        const uint32_t R = edt2[v];
        const int cy = static_cast<int>(v % g.SY);
        const size_t zx = v / g.SY;
        const int cx = static_cast<int>(zx % g.SX);
        const int cz = static_cast<int>(zx / g.SX);
        const uint32_t lex = (static_cast<uint32_t>(cx) * g.SY + cy) * static_cast<uint32_t>(g.SZ) + cz;
        const unsigned long long key = (static_cast<unsigned long long>(R) << 32) | (0xFFFFFFFFu - lex);
        const int r = static_cast<int>(isqrt_u32(R));
        const int G = r >= 12 ? 32 : (r >= 6 ? 16 : (r >= 3 ? 8 : 4));
        const int groups = 32 / G;
        const int grp = lane / G, gl = lane % G;
        const int x0 = max(cx - r, 0), x1 = min(cx + r, g.SX - 1);
        const int z0 = max(cz - r, 0), z1 = min(cz + r, g.SZ - 1);
        const int nxs = x1 - x0 + 1;
        const int nspans = nxs * (z1 - z0 + 1);
        for (int s = grp; s < nspans; s += groups) {
            const int z = z0 + s / nxs;
            const int x = x0 + s % nxs;
            const int ddx = x - cx, ddz = z - cz;
            const int rem = static_cast<int>(R) - ddx * ddx - ddz * ddz;
            if (rem < 0) continue;
            const int w = static_cast<int>(isqrt_u32(static_cast<uint32_t>(rem)));
            const int ya = max(cy - w, 0), yb = min(cy + w, g.SY - 1);
            unsigned long long* row = keys + g.idx(x, 0, z);
            for (int y = ya + gl; y <= yb; y += G) {
                const unsigned long long cur = __ldcg(row + y);
                if (cur < key) atomicMax(row + y, key);
            }
        }
    }
}

__global__ void balls_unpack(const unsigned long long* __restrict__ keys, Geo g, size_t n,
                             uint32_t* __restrict__ crad2, uint32_t* __restrict__ cxo,
                             uint32_t* __restrict__ cyo, uint32_t* __restrict__ czo,
                             uint8_t* __restrict__ mask, unsigned int* __restrict__ err) {
    const uint32_t syz = static_cast<uint32_t>(g.SY) * g.SZ;
    for (size_t v = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; v < n;
         v += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const unsigned long long k = keys[v];
        if (k == 0) atomicOr(err, 2u);  // a void voxel no kept ball covers: internal error
        if (k == ~0ull || k == 0) {
            crad2[v] = 0;
            cxo[v] = 0xFFFFFFFFu;
            cyo[v] = 0xFFFFFFFFu;
            czo[v] = 0xFFFFFFFFu;
            mask[v] = 0;
        } else {
            const uint32_t lex = 0xFFFFFFFFu - static_cast<uint32_t>(k);
            crad2[v] = static_cast<uint32_t>(k >> 32);
            cxo[v] = lex / syz;
            const uint32_t rem = lex % syz;
            cyo[v] = rem / g.SZ;
            czo[v] = rem % g.SZ;
            mask[v] = 127;
        }
    }
}

// Marks winning centres (OUTER = 255). Reads the packed keys rather than the three
// coordinate arrays.
__global__ void balls_mark(const unsigned long long* __restrict__ keys, Geo g, size_t n,
                           uint8_t* __restrict__ mask) {
    const uint32_t limit = static_cast<uint32_t>(n);
    const uint32_t syz = static_cast<uint32_t>(g.SY) * g.SZ;
    for (size_t v = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; v < n;
         v += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const unsigned long long k = keys[v];
        if (k == ~0ull || k == 0) continue;
        const uint32_t lex = 0xFFFFFFFFu - static_cast<uint32_t>(k);
        if (lex >= limit) continue;
        const uint32_t x = lex / syz, rem = lex % syz;
        mask[g.idx(static_cast<int>(x), static_cast<int>(rem / g.SZ), static_cast<int>(rem % g.SZ))] = 255;
    }
}

__global__ void count_value(const uint8_t* __restrict__ a, size_t n, uint8_t value,
                            unsigned long long* __restrict__ out) {
    unsigned long long c = 0;
    for (size_t v = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; v < n;
         v += static_cast<size_t>(gridDim.x) * blockDim.x)
        c += (a[v] == value);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

}  // namespace

void containing_balls(pma_ctx* ctx, const uint32_t* edt2, pma_dims d, uint32_t max_edt2,
                      uint32_t* crad2, uint32_t* cx, uint32_t* cy, uint32_t* cz, uint8_t* mask,
                      uint64_t* count) {
    check_dims(d);
    PMA_REQUIRE(edt2 && crad2 && cx && cy && cz && mask, PMA_ERR_ARGUMENT,
                "pma_containing_balls: null device pointer");
    cudaStream_t s = ctx->stream;
    const size_t n = voxels(d);
    const Geo g{d.sx, d.sy, d.sz};
    const uint32_t nR = max_edt2 + 1;
    const uint32_t ntab = std::min<uint32_t>(nR, kExactTable);
    const unsigned grid = static_cast<unsigned>(std::min<size_t>(div_up(n, 256), ctx->num_sms * 16ull));

    auto* keys = static_cast<unsigned long long*>(ctx->scratch("balls.keys", n * 8));
    auto* mtab = static_cast<uint32_t*>(ctx->scratch("balls.mtab", 3ull * ntab * 4));
    auto* counts = static_cast<uint32_t*>(ctx->scratch("balls.counts", (2ull * nR + 6) * 4));
    uint32_t* cursor = counts + nR;
    uint32_t* misc = cursor + nR;  // [0] total, [1] next, [2..3] count, [4] error flags
    auto* list = static_cast<uint32_t*>(ctx->scratch("balls.list", n * 4));

    balls_containment_table<<<div_up(ntab, 128), 128, 0, s>>>(mtab, mtab + ntab, mtab + 2 * ntab, ntab);
    ctx->check_launch("balls_containment_table");
    PMA_CUDA(cudaMemsetAsync(counts, 0, (2ull * nR + 6) * 4, s));
    unsigned int* err = misc + 4;
    {
    KernelTimer kt(ctx, "balls_candidates");
    balls_candidates<false><<<grid, 256, 0, s>>>(edt2, g, n, mtab, ntab, nR, counts, nullptr, nullptr,
                                                 keys, err);
    ctx->check_launch("balls_candidates(count)");
    balls_bucket_offsets<<<1, 1024, 0, s>>>(counts, cursor, nR, misc);
    ctx->check_launch("balls_bucket_offsets");
    balls_candidates<true><<<grid, 256, 0, s>>>(edt2, g, n, mtab, ntab, nR, counts, cursor, list,
                                                keys, err);
    ctx->check_launch("balls_candidates(place)");
    }
    uint32_t hm[5] = {0, 0, 0, 0, 0};
    PMA_CUDA(cudaMemcpyAsync(hm, misc, sizeof(hm), cudaMemcpyDeviceToHost, s));
    ctx->sync();
    PMA_REQUIRE(!(hm[4] & 1u), PMA_ERR_ARGUMENT,
                "pma_containing_balls: max_edt2 is smaller than the largest squared distance");
    const uint32_t total = hm[0];
    if (total) {
        KernelTimer kt(ctx, "balls_scatter");
        balls_scatter<<<ctx->num_sms * 8, 256, 0, s>>>(edt2, g, list, total, misc + 1, keys);
        ctx->check_launch("balls_scatter");
    }
    balls_unpack<<<grid, 256, 0, s>>>(keys, g, n, crad2, cx, cy, cz, mask, err);
    ctx->check_launch("balls_unpack");
    balls_mark<<<grid, 256, 0, s>>>(keys, g, n, mask);
    ctx->check_launch("balls_mark");
    auto* d_count = reinterpret_cast<unsigned long long*>(misc + 2);
    PMA_CUDA(cudaMemsetAsync(d_count, 0, 8, s));
    count_value<<<grid, 256, 0, s>>>(mask, n, 255, d_count);
    ctx->check_launch("count_value");
    unsigned long long c = 0;
    PMA_CUDA(cudaMemcpyAsync(&c, d_count, 8, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(hm, misc, sizeof(hm), cudaMemcpyDeviceToHost, s));
    ctx->sync();
    PMA_REQUIRE(!(hm[4] & 2u), PMA_ERR_INTERNAL, "pma_containing_balls: uncovered void voxel");
    if (count) *count = c;
}

}  // namespace pma
