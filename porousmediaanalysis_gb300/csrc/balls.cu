// Containing-ball radii, winning centres and the maximum-ball mask
// (ContainingBallsAssigner.cpp:101-250).
//
// Single-thread semantics of the reference: centres are visited in x, y, z order and a
// voxel takes a new centre only on a strictly larger squared radius, so each void voxel
// ends with the largest r^2 covering it and, among those, the lexicographically smallest
// (x, y, z) centre. Both orders fit one 64-bit key,
//     key = (r^2 << 32) | (0xFFFFFFFF - ((x * SY + y) * SZ + z)),
// and the winner of a voxel is the covering centre of largest key.
//
// Work reduction: a centre whose discrete ball lies inside the ball of one of its 26
// neighbours can never win a voxel (the neighbour covers the same voxels with a strictly
// larger radius), so it is dropped. Containment B(c, R) in B(c + e, R') holds iff
// R' >= M_k(R) = max over lattice v with |v|^2 <= R of |v + e|^2, k = |e|^2; M_k is computed
// exactly for R < kExactTable and replaced above it by the continuous sufficient condition
// (sqrt(R) + sqrt(k))^2 <= R'.
//
// Gather: the volume is cut into 8^3 tiles; every kept centre is listed in each tile its
// ball reaches, unless its key is below the tile's floor (the largest key of a ball covering
// the whole tile, which every voxel of the tile is covered by). One CTA per tile orders its
// list by radius in shared memory, and each warp of voxels takes, per voxel, the largest key
// among the entries whose ball covers it: the reference's winner. A warp only tests entries
// that reach its 1 x 4 x 8 box and beat its lanes' smallest key so far, and stops where the
// radius order shows that no later entry can, so the work is close to the winners' ranks in
// the list rather than the ball volumes a scatter would touch.
#include <thrust/iterator/counting_iterator.h>

#include <vector>

#include "devutil.cuh"

namespace pma {
namespace {

constexpr uint32_t kExactTable = 1u << 16;
constexpr int kTile = 8;          // tile edge
constexpr int kTileVox = 512;     // voxels (and threads) per tile
constexpr int kListCap = 2048;    // entries ordered in shared memory at a time; longer lists go in chunks

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

__device__ __forceinline__ bool dominated(const uint32_t* __restrict__ edt2, Grid g, int x, int y,
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

__global__ void balls_candidate_flags(const uint32_t* __restrict__ edt2, Grid g, size_t n,
                                      const uint32_t* __restrict__ mtab, uint32_t ntab, uint32_t nR,
                                      uint8_t* __restrict__ flags, unsigned int* __restrict__ err) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t R = edt2[v];
        uint8_t f = 0;
        if (R != 0) {
            if (R >= nR) {  // max_edt2 below the data: refuse rather than index past the table
                atomicOr(err, 1u);
            } else {
                int x, y, z;
                g.coords(v, x, y, z);
                f = dominated(edt2, g, x, y, z, R, mtab, ntab) ? 0 : 1;
            }
        }
        flags[v] = f;
    }
}

struct Tiles {
    int TX, TY, TZ;  // tiles per axis
    __device__ __forceinline__ size_t id(int tx, int ty, int tz) const {
        return (static_cast<size_t>(tz) * TX + tx) * TY + ty;
    }
};

// Visits the tiles whose box is within sqrt(R) of centre (x, y, z), restricted to tile
// z-range [tz0, tz1). f(tile, full): full = the ball covers the whole tile (clipped to the
// volume), i.e. its farthest corner - a ball is convex, so covering the eight corners of a
// box covers every lattice point in it.
template <class F>
__device__ __forceinline__ void for_each_tile(Grid g, Tiles t, int x, int y, int z, uint32_t R,
                                              int tz0, int tz1, F f) {
    const int r = static_cast<int>(isqrt_u32(R));
    const int ax = max(x - r, 0) / kTile, bx = min(x + r, g.SX - 1) / kTile;
    const int ay = max(y - r, 0) / kTile, by = min(y + r, g.SY - 1) / kTile;
    const int az = max(max(z - r, 0) / kTile, tz0), bz = min(min(z + r, g.SZ - 1) / kTile, tz1 - 1);
    for (int tz = az; tz <= bz; ++tz) {
        const int lz = tz * kTile, hz = min(lz + kTile - 1, g.SZ - 1);
        const int dz = z < lz ? lz - z : (z > hz ? z - hz : 0);
        const int fz = max(abs(z - lz), abs(hz - z));
        for (int tx = ax; tx <= bx; ++tx) {
            const int lx = tx * kTile, hx = min(lx + kTile - 1, g.SX - 1);
            const int dx = x < lx ? lx - x : (x > hx ? x - hx : 0);
            const int dxz = dx * dx + dz * dz;
            if (static_cast<uint32_t>(dxz) > R) continue;
            const int fx = max(abs(x - lx), abs(hx - x));
            const int fxz = fx * fx + fz * fz;
            for (int ty = ay; ty <= by; ++ty) {
                const int ly = ty * kTile, hy = min(ly + kTile - 1, g.SY - 1);
                const int dy = y < ly ? ly - y : (y > hy ? y - hy : 0);
                if (static_cast<uint32_t>(dxz + dy * dy) > R) continue;
                const int fy = max(abs(y - ly), abs(hy - y));
                f(t.id(tx, ty, tz), static_cast<uint32_t>(fxz + fy * fy) <= R);
            }
        }
    }
}

// Floor of a tile: the largest key among balls covering the whole tile. Every voxel of the
// tile is covered by that ball, so its winner's key is at least the floor, and list entries
// below it can be left out.
struct FloorTile {
    unsigned long long* floor;
    unsigned long long key;
    __device__ void operator()(size_t tid, bool full) const {
        if (full) atomicMax(&floor[tid], key);
    }
};

struct CountTile {
    const unsigned long long* floor;
    unsigned int* tcount;
    unsigned long long key;
    __device__ void operator()(size_t tid, bool) const {
        if (key >= __ldg(floor + tid)) atomicAdd(&tcount[tid], 1u);
    }
};

struct FillTile {
    const unsigned long long* floor;
    const unsigned long long* toff;
    unsigned long long base;
    unsigned int* tcursor;
    unsigned long long* entries;
    unsigned long long key;
    __device__ void operator()(size_t tid, bool) const {
        if (key < __ldg(floor + tid)) return;
        const unsigned pos = atomicAdd(&tcursor[tid], 1u);
        entries[toff[tid] - base + pos] = key;
    }
};

__device__ __forceinline__ unsigned long long ball_key(Grid g, int x, int y, int z, uint32_t R) {
    const uint32_t lex = (static_cast<uint32_t>(x) * g.SY + y) * static_cast<uint32_t>(g.SZ) + z;
    return (static_cast<unsigned long long>(R) << 32) | (0xFFFFFFFFu - lex);
}

__global__ void balls_tile_floor(const uint32_t* __restrict__ edt2, const uint32_t* __restrict__ cand,
                                 size_t nc, Grid g, Tiles t, unsigned long long* __restrict__ floor) {
    PMA_GRID_STRIDE(i, nc) {
        const uint32_t v = cand[i];
        int x, y, z;
        g.coords(v, x, y, z);
        const uint32_t R = edt2[v];
        for_each_tile(g, t, x, y, z, R, 0, t.TZ, FloorTile{floor, ball_key(g, x, y, z, R)});
    }
}

__global__ void balls_tile_count(const uint32_t* __restrict__ edt2, const uint32_t* __restrict__ cand,
                                 size_t nc, Grid g, Tiles t, const unsigned long long* __restrict__ floor,
                                 unsigned int* __restrict__ tcount) {
    PMA_GRID_STRIDE(i, nc) {
        const uint32_t v = cand[i];
        int x, y, z;
        g.coords(v, x, y, z);
        const uint32_t R = edt2[v];
        for_each_tile(g, t, x, y, z, R, 0, t.TZ, CountTile{floor, tcount, ball_key(g, x, y, z, R)});
    }
}

__global__ void balls_tile_fill(const uint32_t* __restrict__ edt2, const uint32_t* __restrict__ cand,
                                size_t nc, Grid g, Tiles t, int tz0, int tz1,
                                const unsigned long long* __restrict__ floor,
                                const unsigned long long* __restrict__ toff, unsigned long long base,
                                unsigned int* __restrict__ tcursor, unsigned long long* __restrict__ entries) {
    PMA_GRID_STRIDE(i, nc) {
        const uint32_t v = cand[i];
        int x, y, z;
        g.coords(v, x, y, z);
        const uint32_t R = edt2[v];
        for_each_tile(g, t, x, y, z, R, tz0, tz1,
                      FillTile{floor, toff, base, tcursor, entries, ball_key(g, x, y, z, R)});
    }
}

__device__ __forceinline__ int4 decode_key(unsigned long long key, Grid g) {
    const uint32_t lex = 0xFFFFFFFFu - static_cast<uint32_t>(key);
    const uint32_t syz = static_cast<uint32_t>(g.SY) * g.SZ;
    const uint32_t x = lex / syz, rem = lex % syz;
    return make_int4(static_cast<int>(x), static_cast<int>(rem / g.SZ), static_cast<int>(rem % g.SZ),
                     static_cast<int>(key >> 32));
}

// 32-bit arithmetic while every offset is below 2^15 (the squared sum then fits), 64-bit
// otherwise (only balls of radius >= 2^15, e.g. the virtual-solid distances of a long empty
// volume).
__device__ __forceinline__ bool covers(int4 c, int vx, int vy, int vz) {
    const unsigned dx = static_cast<unsigned>(abs(vx - c.x)), dy = static_cast<unsigned>(abs(vy - c.y));
    const unsigned dz = static_cast<unsigned>(abs(vz - c.z));
    if ((dx | dy | dz) < (1u << 15)) return dx * dx + dy * dy + dz * dz <= static_cast<uint32_t>(c.w);
    const unsigned long long d2 = static_cast<unsigned long long>(dx) * dx +
                                  static_cast<unsigned long long>(dy) * dy + static_cast<unsigned long long>(dz) * dz;
    return d2 <= static_cast<uint32_t>(c.w);
}

__device__ __forceinline__ unsigned long long pos_key(int4 c, Grid g) {
    const uint32_t lex = (static_cast<uint32_t>(c.x) * g.SY + static_cast<uint32_t>(c.y)) * static_cast<uint32_t>(g.SZ) +
                         static_cast<uint32_t>(c.z);
    return (static_cast<unsigned long long>(static_cast<uint32_t>(c.w)) << 32) | (0xFFFFFFFFu - lex);
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = t < v ? t : v;
    }
    return v;
}

// One CTA per tile of the z-range starting at tz0: winner key of each voxel.
//
// The tile's list is taken in chunks of up to kListCap entries. Each chunk is decoded into
// shared memory ordered by radius, largest first (a counting sort on r^2 when the chunk's r^2
// span fits kSortBins, else left in list order). A warp covers a 1 x 4 x 8 box of voxels and
// keeps, per lane, the largest covering key so far (best). It reads the chunk 32 entries at a
// time: an entry can matter only if its ball reaches the warp's box and its key exceeds the
// smallest best of the warp's lanes; the lanes test every such entry against their own voxel.
// In a chunk sorted by radius the warp stops once the next entry's r^2 is below the smallest
// best's r^2 (every later entry's key is smaller). The result is the largest covering key over
// the whole list, i.e. the covering centre of largest key.
constexpr int kSortBins = 2048;

__global__ void __launch_bounds__(kTileVox, 3) balls_tile_gather(
    const uint32_t* __restrict__ edt2, Grid g, Tiles t, int tz0,
    const unsigned int* __restrict__ tcount, const unsigned long long* __restrict__ toff,
    unsigned long long base, const unsigned long long* __restrict__ entries,
    unsigned long long* __restrict__ keys, unsigned int* __restrict__ err) {
    __shared__ int4 s_pos[kListCap];
    __shared__ unsigned int s_bin[kSortBins];
    __shared__ unsigned int s_rmin, s_rmax, s_wsum[kTileVox / 32];
    const size_t tile = static_cast<size_t>(tz0) * t.TX * t.TY + blockIdx.x;
    const int ty = static_cast<int>(tile % t.TY);
    const size_t rest = tile / t.TY;
    const int tx = static_cast<int>(rest % t.TX);
    const int tz = static_cast<int>(rest / t.TX);
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // voxel of this thread: y fastest, then x, then z (a warp covers a 1 x 4 x 8 box)
    const int vy = ty * kTile + (threadIdx.x & 7);
    const int vx = tx * kTile + ((threadIdx.x >> 3) & 7);
    const int vz = tz * kTile + (threadIdx.x >> 6);
    const bool inside = vx < g.SX && vy < g.SY && vz < g.SZ;
    const size_t v = inside ? g.idx(vx, vy, vz) : 0;
    const bool void_voxel = inside && edt2[v] != 0;
    // the warp's box
    const int bx0 = tx * kTile + (warp & 1) * 4, by0 = ty * kTile, bz = vz;
    const unsigned int L = tcount[tile];
    const unsigned long long* list = entries + (toff[tile] - base);
    unsigned long long best = void_voxel ? 0ull : ~0ull;
    for (unsigned int c0 = 0; c0 < L; c0 += kListCap) {
        const unsigned int m = min(static_cast<unsigned int>(kListCap), L - c0);
        // radius span of the chunk; up to four entries per thread stay in registers
        constexpr int kPer = kListCap / kTileVox;
        unsigned long long k[kPer];
        if (threadIdx.x == 0) {
            s_rmin = 0xFFFFFFFFu;
            s_rmax = 0;
        }
        for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) s_bin[i] = 0;
        __syncthreads();
        unsigned int rmin = 0xFFFFFFFFu, rmax = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const unsigned int i = threadIdx.x + q * kTileVox;
            k[q] = i < m ? list[c0 + i] : 0ull;
            if (i < m) {
                rmin = min(rmin, static_cast<unsigned int>(k[q] >> 32));
                rmax = max(rmax, static_cast<unsigned int>(k[q] >> 32));
            }
        }
        rmin = __reduce_min_sync(0xFFFFFFFFu, rmin);
        rmax = __reduce_max_sync(0xFFFFFFFFu, rmax);
        if (lane == 0) {
            atomicMin(&s_rmin, rmin);
            atomicMax(&s_rmax, rmax);
        }
        __syncthreads();
        const unsigned int r_hi = s_rmax;
        const bool sorted = r_hi - s_rmin < static_cast<unsigned int>(kSortBins);
        unsigned int rank[kPer];
        if (sorted) {  // counting sort, descending r^2: bin = r_hi - r^2
            // equal radii are common: lanes with the same bin take their ranks with one atomic
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const unsigned int i = threadIdx.x + q * kTileVox;
                const unsigned int bin = i < m ? r_hi - static_cast<unsigned int>(k[q] >> 32) : 0xFFFFFFFFu;
                const unsigned int peers = __match_any_sync(0xFFFFFFFFu, bin);
                const int leader = __ffs(peers) - 1;
                unsigned int at = 0;
                if (bin != 0xFFFFFFFFu && static_cast<int>(lane) == leader) at = atomicAdd(&s_bin[bin], __popc(peers));
                at = __shfl_sync(0xFFFFFFFFu, at, leader);
                rank[q] = at + __popc(peers & ((1u << lane) - 1u));
            }
            __syncthreads();
            // exclusive scan of the bins, four per thread
            unsigned int b4[kSortBins / kTileVox], sum = 0;
#pragma unroll
            for (int q = 0; q < kSortBins / kTileVox; ++q) {
                b4[q] = s_bin[threadIdx.x * (kSortBins / kTileVox) + q];
                sum += b4[q];
            }
            unsigned int incl = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int t2 = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= static_cast<unsigned>(o)) incl += t2;
            }
            if (lane == 31) s_wsum[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                unsigned int w = lane < kTileVox / 32 ? s_wsum[lane] : 0u;
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned int t2 = __shfl_up_sync(0xFFFFFFFFu, w, o);
                    if (lane >= static_cast<unsigned>(o)) w += t2;
                }
                if (lane < kTileVox / 32) s_wsum[lane] = w;
            }
            __syncthreads();
            unsigned int run = (warp ? s_wsum[warp - 1] : 0u) + incl - sum;
#pragma unroll
            for (int q = 0; q < kSortBins / kTileVox; ++q) {
                s_bin[threadIdx.x * (kSortBins / kTileVox) + q] = run;
                run += b4[q];
            }
            __syncthreads();
        }
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const unsigned int i = threadIdx.x + q * kTileVox;
            if (i < m) {
                const unsigned int at = sorted ? s_bin[r_hi - static_cast<unsigned int>(k[q] >> 32)] + rank[q] : i;
                s_pos[at] = decode_key(k[q], g);
            }
        }
        __syncthreads();
        // the warp's pass over the chunk
        for (unsigned int e0 = 0; e0 < m; e0 += 32) {
            const unsigned long long mb = warp_min_u64(best);
            if (mb == ~0ull) break;  // no void voxel left to improve
            if (sorted && static_cast<uint32_t>(s_pos[e0].w) < static_cast<uint32_t>(mb >> 32)) break;
            bool cand = false;
            if (e0 + lane < m) {
                const int4 c = s_pos[e0 + lane];
                if (pos_key(c, g) > mb) {  // can beat some lane; does the ball reach the box?
                    const int dx = c.x < bx0 ? bx0 - c.x : (c.x > bx0 + 3 ? c.x - bx0 - 3 : 0);
                    const int dy = c.y < by0 ? by0 - c.y : (c.y > by0 + 7 ? c.y - by0 - 7 : 0);
                    const int dz = c.z < bz ? bz - c.z : (c.z > bz ? c.z - bz : 0);
                    cand = covers(make_int4(dx, dy, dz, c.w), 0, 0, 0);
                }
            }
            unsigned int mask = __ballot_sync(0xFFFFFFFFu, cand);
            while (mask) {
                const int b = __ffs(mask) - 1;
                mask &= mask - 1;
                const int4 c = s_pos[e0 + b];
                const unsigned long long kc = pos_key(c, g);
                if (kc > best && void_voxel && covers(c, vx, vy, vz)) best = kc;
            }
        }
        if (c0 + kListCap < L) __syncthreads();  // before the next chunk replaces s_pos
    }
    if (inside) {
        if (void_voxel && best == 0) atomicOr(err, 2u);  // no kept ball covers a void voxel
        keys[v] = void_voxel ? best : ~0ull;
    }
}

__global__ void balls_unpack(const unsigned long long* __restrict__ keys, Grid g, size_t n,
                             uint32_t* __restrict__ crad2, uint32_t* __restrict__ cxo,
                             uint32_t* __restrict__ cyo, uint32_t* __restrict__ czo,
                             uint8_t* __restrict__ mask) {
    const uint32_t syz = static_cast<uint32_t>(g.SY) * g.SZ;
    PMA_GRID_STRIDE(v, n) {
        const unsigned long long k = keys[v];
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

// Marks winning centres (OUTER = 255) from the packed keys.
__global__ void balls_mark(const unsigned long long* __restrict__ keys, Grid g, size_t n,
                           uint8_t* __restrict__ mask) {
    const uint32_t syz = static_cast<uint32_t>(g.SY) * g.SZ;
    const uint32_t limit = static_cast<uint32_t>(n);
    PMA_GRID_STRIDE(v, n) {
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
    PMA_GRID_STRIDE(v, n) c += (a[v] == value);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

template <class T>
T* buf(pma_ctx* ctx, const char* tag, size_t count) {
    return static_cast<T*>(ctx->scratch(tag, std::max<size_t>(count, 1) * sizeof(T)));
}

// Tile counts as 64-bit values, with a zero past the end (the scan then gives the total).
__global__ void widen_counts(const unsigned int* __restrict__ c, size_t n, unsigned long long* __restrict__ out) {
    PMA_GRID_STRIDE(i, n + 1) out[i] = i < n ? c[i] : 0ull;
}

// Offsets of the first tile of each z-slab (and the total at tz).
__global__ void slab_offsets(const unsigned long long* __restrict__ toff, size_t per_z, int tz,
                             unsigned long long* __restrict__ zoff) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z <= tz) zoff[z] = toff[static_cast<size_t>(z) * per_z];
}

}  // namespace

void containing_balls(pma_ctx* ctx, const uint32_t* edt2, pma_dims d, uint32_t max_edt2,
                      uint32_t* crad2, uint32_t* cx, uint32_t* cy, uint32_t* cz, uint8_t* mask,
                      uint64_t* count) {
    KernelTimer kt_stage(ctx, "stage_balls");  // the whole stage, for the untimed remainder
    check_dims(d);
    PMA_REQUIRE(edt2 && crad2 && cx && cy && cz && mask, PMA_ERR_ARGUMENT,
                "pma_containing_balls: null device pointer");
    cudaStream_t s = ctx->stream;
    const size_t n = voxels(d);
    const Grid g{d.sx, d.sy, d.sz};
    const uint32_t nR = max_edt2 + 1;
    const uint32_t ntab = std::min<uint32_t>(nR, kExactTable);
    const unsigned G = grid_for(ctx, n);

    auto* keys = buf<unsigned long long>(ctx, "balls.keys", n);
    auto* mtab = buf<uint32_t>(ctx, "balls.mtab", 3ull * ntab);
    auto* misc = buf<unsigned long long>(ctx, "balls.misc", 4);  // [0] count, [1] err, [2] select
    auto* err = reinterpret_cast<unsigned int*>(misc + 1);
    PMA_CUDA(cudaMemsetAsync(misc, 0, 32, s));

    // Kept centres.
    balls_containment_table<<<div_up(ntab, 128), 128, 0, s>>>(mtab, mtab + ntab, mtab + 2 * ntab, ntab);
    ctx->check_launch("balls_containment_table");
    uint8_t* flags = buf<uint8_t>(ctx, "balls.flags", n);
    uint32_t* cand = buf<uint32_t>(ctx, "balls.cand", n);
    int64_t nc = 0;
    {
        KernelTimer kt(ctx, "balls_candidates");
        balls_candidate_flags<<<G, 256, 0, s>>>(edt2, g, n, mtab, ntab, nR, flags, err);
        ctx->check_launch("balls_candidate_flags");
        nc = select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), flags, cand,
                            static_cast<int64_t>(n), reinterpret_cast<int64_t*>(misc + 2));
    }
    unsigned int h_err = 0;
    PMA_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    PMA_REQUIRE(!(h_err & 1u), PMA_ERR_ARGUMENT,
                "pma_containing_balls: max_edt2 is smaller than the largest squared distance");

    // Tile lists: counts, 64-bit offsets (host scan), then fill + gather by tile z-ranges
    // whose entries fit the memory budget.
    Tiles t{(d.sx + kTile - 1) / kTile, (d.sy + kTile - 1) / kTile, (d.sz + kTile - 1) / kTile};
    const size_t per_z = static_cast<size_t>(t.TX) * t.TY;
    const size_t ntiles = per_z * t.TZ;
    unsigned int* tcount = buf<unsigned int>(ctx, "balls.tcount", ntiles);
    unsigned int* tcursor = buf<unsigned int>(ctx, "balls.tcursor", ntiles);
    auto* toff = buf<unsigned long long>(ctx, "balls.toff", ntiles + 1);
    auto* floor = buf<unsigned long long>(ctx, "balls.floor", ntiles);
    PMA_CUDA(cudaMemsetAsync(tcount, 0, ntiles * 4, s));
    PMA_CUDA(cudaMemsetAsync(tcursor, 0, ntiles * 4, s));
    PMA_CUDA(cudaMemsetAsync(floor, 0, ntiles * 8, s));
    if (nc) {
        KernelTimer kt(ctx, "balls_tile_count");
        balls_tile_floor<<<grid_for(ctx, nc), 256, 0, s>>>(edt2, cand, nc, g, t, floor);
        ctx->check_launch("balls_tile_floor");
        balls_tile_count<<<grid_for(ctx, nc), 256, 0, s>>>(edt2, cand, nc, g, t, floor, tcount);
        ctx->check_launch("balls_tile_count");
    }
    // 64-bit list offsets by a device scan; the host reads back only the offsets at the tile
    // z-slab boundaries, which choose the slabs that fit the memory budget
    auto* tc64 = buf<unsigned long long>(ctx, "balls.tc64", ntiles + 1);
    widen_counts<<<grid_for(ctx, ntiles + 1), 256, 0, s>>>(tcount, ntiles, tc64);
    ctx->check_launch("widen_counts");
    exclusive_sum(ctx, tc64, toff, static_cast<int64_t>(ntiles + 1));
    auto* zoff = buf<unsigned long long>(ctx, "balls.zoff", t.TZ + 1);
    slab_offsets<<<div_up(t.TZ + 1, 256), 256, 0, s>>>(toff, per_z, t.TZ, zoff);
    ctx->check_launch("slab_offsets");
    std::vector<unsigned long long> hz(t.TZ + 1);
    PMA_CUDA(cudaMemcpyAsync(hz.data(), zoff, (t.TZ + 1) * 8ull, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    auto ho_at = [&](int z) { return hz[z]; };  // offset of the first tile of slab z
    size_t free_b = 0, total_b = 0;
    PMA_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const unsigned long long budget = std::max<unsigned long long>(
        1ull << 20, std::min<unsigned long long>(free_b / 3, 32ull << 30) / 8);
    for (int z0 = 0; z0 < t.TZ;) {
        int z1 = z0 + 1;
        while (z1 < t.TZ && ho_at(z1 + 1) - ho_at(z0) <= budget) ++z1;
        const unsigned long long base = ho_at(z0);
        const unsigned long long cnt = ho_at(z1) - base;
        auto* entries = buf<unsigned long long>(ctx, "balls.entries", cnt);
        if (nc) {
            KernelTimer kt(ctx, "balls_tile_fill");
            balls_tile_fill<<<grid_for(ctx, nc), 256, 0, s>>>(edt2, cand, nc, g, t, z0, z1, floor, toff,
                                                              base, tcursor, entries);
            ctx->check_launch("balls_tile_fill");
        }
        {
            KernelTimer kt(ctx, "balls_tile_gather");
            balls_tile_gather<<<static_cast<unsigned>((z1 - z0) * per_z), kTileVox, 0, s>>>(
                edt2, g, t, z0, tcount, toff, base, entries, keys, err);
            ctx->check_launch("balls_tile_gather");
        }
        z0 = z1;
    }
    balls_unpack<<<G, 256, 0, s>>>(keys, g, n, crad2, cx, cy, cz, mask);
    ctx->check_launch("balls_unpack");
    balls_mark<<<G, 256, 0, s>>>(keys, g, n, mask);
    ctx->check_launch("balls_mark");
    PMA_CUDA(cudaMemsetAsync(misc, 0, 8, s));
    count_value<<<G, 256, 0, s>>>(mask, n, 255, misc);
    ctx->check_launch("count_value");
    unsigned long long c = 0;
    PMA_CUDA(cudaMemcpyAsync(&c, misc, 8, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    PMA_REQUIRE(!(h_err & 2u), PMA_ERR_INTERNAL, "pma_containing_balls: uncovered void voxel");
    if (count) *count = c;
}

}  // namespace pma
