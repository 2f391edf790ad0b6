// Pore seeds, initial pore propagation and empty-pore removal
// (PoreAndThroatComputer.cpp:93-269, BasePoreAndThroatComputer.cpp:37-133,
// EmptyPoresRemover.cpp:31-244).
//
// The reference runs one depth-first search per pore: from the seed it follows u -> v when
// v is a void stencil neighbour with crad(v) <= crad(u). Restated exactly:
//  * Plateaus. Voxels of one connected set of equal crad ("plateau") all reach each other,
//    so the set S of seeds reaching a voxel is constant on its plateau, and
//    S(p) = union of S(q) over plateaus q with an edge into p, plus p's own seed.
//  * Seeds. Maximum balls are visited in std::sort order and a ball starts a pore unless an
//    earlier pore already reached its centre. By induction on that order, a ball is a seed
//    exactly when no ball earlier in the order reaches it (a skipped ball was reached by an
//    earlier seed, which then reaches all it reaches). With m(p) the smallest rank of a ball
//    reaching plateau p, p's smallest-rank ball is a seed iff it beats m of every plateau
//    with an edge into p.
//  * Plateaus are found by a union-find over equal-crad neighbours (from 2^24 voxels:
//    pointer jumping on the initial trees, then unions of the recorded parent pairs).
//  * Both recurrences run plateau by plateau in decreasing crad, a few launches per crad
//    level. The ball order is std::sort's on the host (ordered_sort: libstdc++'s own
//    introsort steps on several threads) applied to the same sequence (z, x, y scan order)
//    with the same comparator, so equal radii tie-break exactly as in the reference.
//  * A voxel's label is its seed's pore id when |S| = 1 and a shared type ("throat") when
//    |S| >= 2. Pore volumes, boundary flags, type volumes and type pore lists are exact.
//    The reference numbers types in its depth-first creation order, which also consumed ids
//    for types deleted later. The types are first numbered by (last pore of the type, first
//    voxel of the type), then renumbered in the reference's order by a host replay of each
//    pore's search order (exact_ids.cpp), unless the context asks for the cheaper numbering.
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <chrono>
#include <thread>
#include <vector>

#include "devutil.cuh"
#include "ordered_sort.h"

namespace pma {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;

__global__ void flag_outer(const uint8_t* __restrict__ mask, size_t n, uint8_t* __restrict__ flags) {
    PMA_GRID_STRIDE(v, n) flags[v] = mask[v] == 255;
}

__global__ void gather_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx,
                           size_t n, uint32_t* __restrict__ out) {
    PMA_GRID_STRIDE(i, n) out[i] = src[idx[i]];
}

__global__ void fill_u32(uint32_t* __restrict__ a, size_t n, uint32_t value) {
    PMA_GRID_STRIDE(i, n) a[i] = value;
}

__global__ void flag_seeds(const uint32_t* __restrict__ seed, size_t np, uint8_t* __restrict__ flags) {
    PMA_GRID_STRIDE(p, np) flags[p] = seed[p] != kNone;
}

// up = [seed ranks (ascending) | their pore ids]
__global__ void scatter_seed_ids(const uint32_t* __restrict__ up, size_t npores, uint32_t* __restrict__ rank2pore,
                                 uint32_t* __restrict__ rank2id) {
    PMA_GRID_STRIDE(k, npores) {
        rank2pore[up[k]] = static_cast<uint32_t>(k);
        rank2id[up[k]] = up[npores + k];
    }
}

__global__ void pack_items(const uint32_t* __restrict__ r2, const uint32_t* __restrict__ idx, size_t n,
                           unsigned long long* __restrict__ items) {
    PMA_GRID_STRIDE(i, n) items[i] = (static_cast<unsigned long long>(r2[i]) << 32) | idx[i];
}

__global__ void scatter_rank(const uint32_t* __restrict__ voxel_of_rank, size_t n,
                             uint32_t* __restrict__ crank) {
    PMA_GRID_STRIDE(r, n) crank[voxel_of_rank[r]] = static_cast<uint32_t>(r);
}

// --- union-find over equal-crad neighbours (parents always point to smaller indices) ---

__device__ __forceinline__ uint32_t uf_root(uint32_t* parent, uint32_t v) {
    uint32_t cur = parent[v];
    if (cur == v) return v;
    uint32_t prev = v, next;
    while (cur > (next = parent[cur])) {
        parent[prev] = next;  // path halving; racing writes only shorten paths
        prev = cur;
        cur = next;
    }
    return cur;
}

// Start every void voxel under its smallest-index equal-crad neighbour (the backward
// offsets, most negative index first), so that most trees exist before any union runs.
__global__ void uf_init(const uint32_t* __restrict__ crad, Grid g, size_t n, int d3q7,
                        uint32_t* __restrict__ parent) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t r = crad[v];
        if (!r) {
            parent[v] = kNone;
            continue;
        }
        int x, y, z;
        g.coords(v, x, y, z);
        uint32_t p = static_cast<uint32_t>(v);
        for (int k = 12; k >= 0 && p == v; --k) {  // the 13 forward offsets, negated, largest first
            int dx, dy, dz;
            if (k < 4) {
                dz = 0;
                dx = (k == 0) ? 0 : 1;
                dy = (k == 0) ? 1 : k - 2;
            } else {
                dz = 1;
                dx = (k - 4) / 3 - 1;
                dy = (k - 4) % 3 - 1;
            }
            if (d3q7 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
            const int nx = x - dx, ny = y - dy, nz = z - dz;
            if (!g.inside(nx, ny, nz)) continue;
            const size_t w = g.idx(nx, ny, nz);
            if (crad[w] == r) p = static_cast<uint32_t>(w);
        }
        parent[v] = p;
    }
}

// Pointer jumping on the initial trees: parent[v] moves up to a few ancestors at a time, in
// place (a value read may already have jumped in this pass, which only shortens paths). The
// initial trees of a large plateau are chains of backward neighbours hundreds of voxels long;
// after a few passes almost every voxel points at its tree's root, so that uf_hook finds
// most neighbour pairs already joined without walking. Each pass skips once a pass changed
// nothing (done[k - 1] == 0).
// Measured: 1024^3 spinodal 408 -> 371 ms for jumps and hooks together; on a 96^3 sphere pack
// the passes cost more (0.5 ms) than they save, so they run from 2^24 voxels up.
constexpr int kJumpPasses = 6;
constexpr size_t kJumpMinVoxels = size_t(1) << 24;

__global__ void uf_jump(size_t n, uint32_t* __restrict__ parent, unsigned int* __restrict__ changed, int pass) {
    if (pass > 0 && *reinterpret_cast<volatile unsigned int*>(changed + pass - 1) == 0) return;
    unsigned int any = 0;
    PMA_GRID_STRIDE(v, n) {
        const uint32_t p = parent[v];
        if (p == kNone || p == v) continue;
        uint32_t cur = p, next = parent[cur];
        for (int k = 0; k < 4 && next != cur; ++k) {
            cur = next;
            next = parent[cur];
        }
        if (cur != p) {
            parent[v] = cur;
            any = 1;
        }
    }
    if (__any_sync(0xFFFFFFFFu, any) && (threadIdx.x & 31) == 0) changed[pass] = 1;
}

__global__ void uf_hook(const uint32_t* __restrict__ crad, Grid g, size_t n, int d3q7,
                        uint32_t* __restrict__ parent, unsigned int* __restrict__ err, int union_limit) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t r = crad[v];
        if (!r) continue;
        int x, y, z;
        g.coords(v, x, y, z);
        // Each unordered pair once: the 13 offsets whose linear index delta
        // dz*SX*SY + dx*SY + dy is positive, i.e. (dz, dx, dy) > 0 lexicographically.
        // rv: a known ancestor of v (its parent after the jumps, then its root after each
        // union), so root walks from v start close to the root.
        uint32_t rv = parent[v];
        for (int k = 0; k < 13; ++k) {
            int dx, dy, dz;
            if (k < 4) {
                dz = 0;
                dx = (k == 0) ? 0 : 1;
                dy = (k == 0) ? 1 : k - 2;
            } else {
                dz = 1;
                dx = (k - 4) / 3 - 1;
                dy = (k - 4) % 3 - 1;
            }
            if (d3q7 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
            const int nx = x + dx, ny = y + dy, nz = z + dz;
            if (!g.inside(nx, ny, nz)) continue;
            const size_t w = g.idx(nx, ny, nz);
            if (crad[w] != r) continue;
            if (parent[w] == rv) continue;  // already joined
            uint32_t a = uf_root(parent, rv);
            uint32_t b = uf_root(parent, static_cast<uint32_t>(w));
            int it = 0;
            while (a != b) {
                if (++it > union_limit) {
                    atomicOr(err, 1u);
                    break;
                }
                if (a < b) {
                    const uint32_t old = atomicCAS(&parent[b], b, a);
                    if (old == b) break;
                    b = old;
                } else {
                    const uint32_t old = atomicCAS(&parent[a], a, b);
                    if (old == a) break;
                    a = old;
                }
            }
            rv = a < b ? a : b;  // the surviving root, an ancestor of v
        }
    }
}

// Large volumes, after the pointer jumps: almost every voxel points at its initial tree's
// root, so a neighbour pair of equal crad whose parents differ is the rare case. uf_pairs
// records those parent pairs (de-duplicated within the block's voxels) instead of walking to
// the roots in line, and uf_union_pairs unions them, one thread per pair, so that the root
// walks (into arrays far larger than L2) run in parallel rather than one neighbour after
// another. The partition and its roots are the same: each plateau's root is its smallest
// voxel index, whatever the union order.
constexpr int kPairTable = 2048;

__global__ void uf_pairs(const uint32_t* __restrict__ crad, Grid g, size_t n, int d3q7,
                         const uint32_t* __restrict__ parent, unsigned long long* __restrict__ pairs,
                         unsigned long long cap, unsigned long long* __restrict__ count) {
    __shared__ unsigned long long table[kPairTable];
    const unsigned lane = threadIdx.x & 31;
    // block-uniform trip count: whole blocks reach the barriers and warps the placement below
    for (size_t base = static_cast<size_t>(blockIdx.x) * blockDim.x; base < n;
         base += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const size_t v = base + threadIdx.x;
        const uint32_t r = v < n ? crad[v] : 0u;
        // shared-memory set of the block's pairs: keep the first copy of each
        for (int i = threadIdx.x; i < kPairTable; i += blockDim.x) table[i] = ~0ull;
        __syncthreads();
        unsigned long long keys[13];
        int kept = 0;
        if (r) {
            int x, y, z;
            g.coords(v, x, y, z);
            const uint32_t rv = parent[v];
            uint32_t seen[13];
            int ns = 0;
            for (int k = 0; k < 13; ++k) {  // the 13 forward offsets, as in uf_hook
                int dx, dy, dz;
                if (k < 4) {
                    dz = 0;
                    dx = (k == 0) ? 0 : 1;
                    dy = (k == 0) ? 1 : k - 2;
                } else {
                    dz = 1;
                    dx = (k - 4) / 3 - 1;
                    dy = (k - 4) % 3 - 1;
                }
                if (d3q7 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
                const int nx = x + dx, ny = y + dy, nz = z + dz;
                if (!g.inside(nx, ny, nz)) continue;
                const size_t w = g.idx(nx, ny, nz);
                if (crad[w] != r) continue;
                const uint32_t pw = parent[w];
                if (pw == rv) continue;  // already in one tree
                bool dup = false;
                for (int i = 0; i < ns; ++i) dup |= seen[i] == pw;
                if (dup) continue;
                seen[ns++] = pw;
                const uint32_t lo = min(rv, pw), hi = max(rv, pw);
                const unsigned long long key = (static_cast<unsigned long long>(lo) << 32) | hi;
                unsigned h = static_cast<unsigned>((key * 0x9E3779B97F4A7C15ull) >> 40) & (kPairTable - 1);
                bool fresh = true;
                for (int probe = 0; probe < 8; ++probe, h = (h + 1) & (kPairTable - 1)) {
                    const unsigned long long prev = atomicCAS(&table[h], ~0ull, key);
                    if (prev == ~0ull) break;
                    if (prev == key) {
                        fresh = false;
                        break;
                    }
                }
                if (fresh) keys[kept++] = key;
            }
        }
        __syncthreads();
        // one atomic per warp; lanes place their pairs by a warp prefix sum
        unsigned incl = static_cast<unsigned>(kept);
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<unsigned>(o)) incl += t;
        }
        unsigned long long pos = 0;
        if (lane == 31 && incl) pos = atomicAdd(count, static_cast<unsigned long long>(incl));
        pos = __shfl_sync(0xFFFFFFFFu, pos, 31) + (incl - static_cast<unsigned>(kept));
        for (int i = 0; i < kept; ++i)
            if (pos + i < cap) pairs[pos + i] = keys[i];
    }
}

__global__ void uf_union_pairs(const unsigned long long* __restrict__ pairs, size_t np,
                               uint32_t* __restrict__ parent, unsigned int* __restrict__ err, int union_limit) {
    PMA_GRID_STRIDE(i, np) {
        uint32_t a = uf_root(parent, static_cast<uint32_t>(pairs[i] >> 32));
        uint32_t b = uf_root(parent, static_cast<uint32_t>(pairs[i]));
        int it = 0;
        while (a != b) {
            if (++it > union_limit) {
                atomicOr(err, 1u);
                break;
            }
            if (a < b) {
                const uint32_t old = atomicCAS(&parent[b], b, a);
                if (old == b) break;
                b = old;
            } else {
                const uint32_t old = atomicCAS(&parent[a], a, b);
                if (old == a) break;
                a = old;
            }
        }
    }
}

// Read-only root walk: flattening must not halve paths, or a racing halving store could
// replace another voxel's final root pointer with an intermediate ancestor.
__device__ __forceinline__ uint32_t uf_root_readonly(const uint32_t* parent, uint32_t v) {
    uint32_t cur = v, next;
    while ((next = parent[cur]) != cur) cur = next;
    return cur;
}

__global__ void uf_flatten(size_t n, uint32_t* parent) {
    PMA_GRID_STRIDE(v, n) {
        if (parent[v] != kNone) parent[v] = uf_root_readonly(parent, static_cast<uint32_t>(v));
    }
}

__global__ void flag_roots(const uint32_t* __restrict__ parent, size_t n, uint8_t* __restrict__ flags) {
    PMA_GRID_STRIDE(v, n) flags[v] = parent[v] == v;
}

__global__ void scatter_pid(const uint32_t* __restrict__ roots, size_t np, uint32_t* __restrict__ tmp) {
    PMA_GRID_STRIDE(p, np) tmp[roots[p]] = static_cast<uint32_t>(p);
}

// parent[v] (the root voxel) becomes the dense plateau id.
__global__ void to_pid(const uint32_t* __restrict__ tmp, size_t n, size_t np, uint32_t* __restrict__ parent,
                       unsigned int* __restrict__ err) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t r = parent[v];
        if (r == kNone) continue;
        const uint32_t p = tmp[r];
        if (p < np) {
            parent[v] = p;
        } else {  // not a root: refuse rather than index past the plateau arrays
            parent[v] = kNone;
            atomicOr(err, 8u);
        }
    }
}

__global__ void plateau_stats(const uint32_t* __restrict__ pid, const uint32_t* __restrict__ crad,
                              const uint32_t* __restrict__ crank, Grid g, size_t n,
                              uint32_t* __restrict__ pcrad, unsigned int* __restrict__ psize,
                              unsigned int* __restrict__ pface, uint32_t* __restrict__ pminrank) {
    // Neighbouring voxels mostly share a plateau: lanes of a warp with the same plateau
    // combine their updates (one atomic per plateau and warp).
    const unsigned lane = threadIdx.x & 31;
    PMA_GRID_STRIDE(v, n) {
        const uint32_t p = pid[v];
        int x, y, z;
        g.coords(v, x, y, z);
        const unsigned face = g.on_face(x, y, z) ? 1u : 0u;
        const uint32_t rk = p == kNone ? kNone : crank[v];
        const unsigned peers = __match_any_sync(__activemask(), p);
        const unsigned any_face = __reduce_or_sync(peers, face);
        const uint32_t min_rank = __reduce_min_sync(peers, rk);
        if (p == kNone || static_cast<int>(lane) != __ffs(peers) - 1) continue;
        pcrad[p] = crad[v];
        atomicAdd(&psize[p], static_cast<unsigned>(__popc(peers)));
        if (any_face) pface[p] = 1;
        if (min_rank != kNone) atomicMin(&pminrank[p], min_rank);
    }
}

// Plateau edges q -> p (crad strictly decreasing), deduplicated per tile; count receives the
// number of edges, also those beyond cap (not written). Each unordered voxel pair is visited
// once, from the voxel of smaller index (the 13 forward offsets), and gives the edge from the
// pair's higher-radius plateau to the lower one; the keys stay in registers.
//
// A block takes tiles of 4 (z) x 8 (x) x 32 (y) voxels: warp w covers row x = w of the tile,
// lane l the voxel y = l (coalesced), one z slice after another. Neighbouring voxels mostly
// report the same plateau pairs, and plateaus are 3-D blobs: the first copy of each pair is
// kept per tile (a shared-memory hash set over the tile's four slices; a pair that finds no free
// slot is kept too - the sort and unique that follow are exact). At 1024^3 a set over 256
// consecutive voxels of one row wrote 1.36 G edges for 0.50 G distinct ones.
constexpr int kEdgeTable = 2048;  // shared-memory pair set of plateau_edges (power of two)
constexpr int kEdgeTileY = 32, kEdgeTileX = 8, kEdgeTileZ = 4;

__global__ void __launch_bounds__(256, 4) plateau_edges(const uint32_t* __restrict__ pid, const uint32_t* __restrict__ crad,
                              Grid g, int d3q7, int sb, unsigned long long* __restrict__ count,
                              unsigned long long* __restrict__ edges, unsigned long long cap) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ unsigned long long table[kEdgeTable];
    const unsigned nty = (g.SY + kEdgeTileY - 1) / kEdgeTileY, ntx = (g.SX + kEdgeTileX - 1) / kEdgeTileX;
    const unsigned ntz = (g.SZ + kEdgeTileZ - 1) / kEdgeTileZ;
    const size_t ntiles = static_cast<size_t>(nty) * ntx * ntz;
    // block-uniform trip counts, so whole warps reach the warp-wide placement below
    for (size_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const unsigned ty = static_cast<unsigned>(t % nty);
        const size_t rest = t / nty;
        const unsigned tx = static_cast<unsigned>(rest % ntx), tz = static_cast<unsigned>(rest / ntx);
        for (int i = threadIdx.x; i < kEdgeTable; i += blockDim.x) table[i] = ~0ull;
        __syncthreads();
        const int x = static_cast<int>(tx) * kEdgeTileX + static_cast<int>(warp);
        const int y = static_cast<int>(ty) * kEdgeTileY + static_cast<int>(lane);
        for (int zs = 0; zs < kEdgeTileZ; ++zs) {
            const int z = static_cast<int>(tz) * kEdgeTileZ + zs;
            const bool in = x < g.SX && y < g.SY && z < g.SZ;
            const size_t v = in ? g.idx(x, y, z) : 0;
            unsigned long long key[13];
            bool has[13];
            const uint32_t p = in ? pid[v] : kNone;
            const uint32_t r = p != kNone ? crad[v] : 0u;
#pragma unroll
            for (int k = 0; k < 13; ++k) {  // the forward offsets, as in uf_hook
                int dx, dy, dz;
                if (k < 4) {
                    dz = 0;
                    dx = (k == 0) ? 0 : 1;
                    dy = (k == 0) ? 1 : k - 2;
                } else {
                    dz = 1;
                    dx = (k - 4) / 3 - 1;
                    dy = (k - 4) % 3 - 1;
                }
                has[k] = false;
                key[k] = 0;
                if (p == kNone || (d3q7 && (dx != 0) + (dy != 0) + (dz != 0) > 1)) continue;
                const int nx = x + dx, ny = y + dy, nz = z + dz;
                if (!g.inside(nx, ny, nz)) continue;
                const size_t w = g.idx(nx, ny, nz);
                const uint32_t rw = crad[w];
                if (rw == 0 || rw == r) continue;
                const uint32_t q = pid[w];
                key[k] = rw < r ? (static_cast<unsigned long long>(q) << sb) | p
                                : (static_cast<unsigned long long>(p) << sb) | q;
                has[k] = true;
            }
            unsigned ns = 0;
#pragma unroll
            for (int k = 0; k < 13; ++k) {
                if (!has[k]) continue;
                unsigned h = static_cast<unsigned>((key[k] * 0x9E3779B97F4A7C15ull) >> 40) & (kEdgeTable - 1);
                for (int probe = 0; probe < 8; ++probe, h = (h + 1) & (kEdgeTable - 1)) {
                    const unsigned long long prev = atomicCAS(&table[h], ~0ull, key[k]);
                    if (prev == ~0ull) break;
                    if (prev == key[k]) {
                        has[k] = false;
                        break;
                    }
                }
                ns += has[k] ? 1u : 0u;
            }
            // one atomic per warp; lanes place their edges by a warp prefix sum
            unsigned incl = ns;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned t2 = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= static_cast<unsigned>(o)) incl += t2;
            }
            unsigned long long pos = 0;
            if (lane == 31 && incl) pos = atomicAdd(count, static_cast<unsigned long long>(incl));
            pos = __shfl_sync(0xFFFFFFFFu, pos, 31) + (incl - ns);
#pragma unroll
            for (int k = 0; k < 13; ++k)
                if (has[k]) {
                    if (pos < cap) edges[pos] = key[k];
                    ++pos;
                }
        }
        __syncthreads();  // before the next tile resets the table
    }
}

// CSR offsets of edges sorted by destination (key >> sb), and the sources (the low sb bits) as
// 32-bit words, the form the level sweep reads.
__global__ void edge_offsets(const unsigned long long* __restrict__ edges, size_t ne, size_t np, int sb,
                             unsigned int* __restrict__ eoff, uint32_t* __restrict__ src) {
    PMA_GRID_STRIDE(i, ne + 1) {
        const uint32_t cur = (i < ne) ? static_cast<uint32_t>(edges[i] >> sb) : static_cast<uint32_t>(np);
        const uint32_t prev = (i == 0) ? 0u : static_cast<uint32_t>(edges[i - 1] >> sb) + 1u;
        for (uint32_t p = prev; p <= cur && p <= np; ++p) eoff[p] = static_cast<unsigned int>(i);
        if (i < ne) src[i] = static_cast<uint32_t>(edges[i] & ((1ull << sb) - 1));
    }
}

__global__ void level_starts(const uint32_t* __restrict__ key, size_t np, uint8_t* __restrict__ flags) {
    PMA_GRID_STRIDE(i, np) flags[i] = i == 0 || key[i] != key[i - 1];
}

__global__ void level_keys(const uint32_t* __restrict__ pcrad, size_t np, uint32_t* __restrict__ key,
                           uint32_t* __restrict__ val) {
    PMA_GRID_STRIDE(p, np) {
        key[p] = 0xFFFFFFFFu - pcrad[p];  // ascending key = descending crad
        val[p] = static_cast<uint32_t>(p);
    }
}

constexpr int kSmallSet = 32;            // sets this small are merged by one warp
constexpr unsigned kHeavyDegree = 1024;  // plateaus with more in-edges are reduced by a block
constexpr int kLevelWarps = 4;           // warps per block of the per-plateau kernels

// Level sweep state. Plateaus of one level are addressed by their local index L (position
// in `order` minus the level's first position).
struct PlateauSets {
    const unsigned int* eoff;
    // Read-only path: the edges, and every array entry of a predecessor (m, slen, soff, its
    // pool elements), are read through __ldg. A predecessor has a larger radius, so it belongs
    // to an earlier level and was written by an earlier launch; the loads need not wait for
    // the launch's own stores to the sweep's 32-bit arrays.
    const uint32_t* edges;  // sources, sorted by destination
    const uint32_t* order;            // plateaus in decreasing crad
    const uint32_t* minrank;
    uint32_t* m;       // smallest ball rank reaching the plateau
    uint32_t* seed;    // rank of the plateau's seed or kNone
    unsigned long long* soff;
    uint32_t* slen;
    uint32_t* pool;
    unsigned long long pool_cap;
    unsigned int* err;
    unsigned long long* cnt;     // [L] set size
    unsigned long long* off;     // [L] exclusive scan of cnt
    unsigned long long* first;   // [L] first merged element of a large set
    uint8_t* big;                // [L] 1: merged by the sort path
    uint32_t* heavy;             // local indices of high in-degree plateaus
    uint32_t* big_list;          // local indices of the sort-path plateaus
    unsigned long long* info;    // [0] heavy, [1] big, [2] big elements, [3] expansion fill,
                                 // [4] fill of the medium unions' buffer
    uint32_t* mtmp;              // sorted medium unions of the level, until level_write
    unsigned long long mtmp_cap;
    unsigned long long* mtoff;   // [L] position of plateau L's medium union in mtmp
};

__device__ __forceinline__ uint32_t warp_min_u32(uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Union of the predecessors' sets and the own seed when it has at most kSmallSet elements
// (the caller checked the sum of the sizes). On return the warp holds the union sorted
// ascending: lanes with keep = true hold element `rank`; the return value is its size.
__device__ __forceinline__ int warp_small_union(const PlateauSets& st, unsigned e0, unsigned e1,
                                                uint32_t seed, uint32_t* wbuf, unsigned int* wfill,
                                                unsigned lane, uint32_t& value, bool& keep, int& rank) {
    if (lane == 0) *wfill = 0;
    __syncwarp();
    for (unsigned e = e0 + lane; e < e1; e += 32) {
        const uint32_t q = __ldg(st.edges + e);
        const uint32_t len = __ldg(st.slen + q);
        if (!len) continue;
        const unsigned pos = atomicAdd(wfill, len);
        const uint32_t* src = st.pool + __ldg(st.soff + q);
        for (uint32_t k = 0; k < len; ++k)
            if (pos + k < kSmallSet) wbuf[pos + k] = __ldg(src + k);
    }
    __syncwarp();
    const unsigned total = min(*wfill, static_cast<unsigned>(kSmallSet));
    __syncwarp();
    uint32_t v = lane < total ? wbuf[lane] : kNone;
    if (seed != kNone && lane == total) v = seed;
    // bitonic sort of the 32 lanes, ascending (kNone pads sort last)
    for (int k = 2; k <= 32; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t other = __shfl_xor_sync(0xFFFFFFFFu, v, j);
            const bool ascending = (lane & k) == 0;
            const bool lower = (lane & j) == 0;
            v = (lower == ascending) ? min(v, other) : max(v, other);
        }
    const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, v, 1);
    keep = v != kNone && (lane == 0 || prev != v);
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, keep);
    rank = __popc(mask & ((1u << lane) - 1u));
    value = v;
    return __popc(mask);
}

// Medium unions: predecessors whose sizes add up to at most kMedSum elements but repeat the
// same seeds (a plateau's in-edges mostly come from plateaus reached by the same pores). One
// warp inserts every element into a hash set of its own in shared memory; when at most kMedCap
// distinct elements remain, they are sorted in the warp and the union stays on this path
// instead of the expand-and-sort path of the big sets. One warp streams a union's elements
// serially, so a long one delays its whole level: at 1024^3 the sweep took 269 ms with unions of
// up to 8192 elements here, 261 with 4096, 257 with 2048 (the rest going to the parallel sort
// path).
constexpr unsigned kMedSum = 2048;
constexpr int kMedCap = 128;
constexpr int kMedHash = 256;  // slots (power of two, twice kMedCap)
constexpr unsigned long long kMedSlab = 1024;  // buffer space a warp takes at a time

struct MedBuf {
    uint32_t table[kMedHash];
    uint32_t sorted[kMedCap];
    unsigned int count;
};

// Inserts the predecessors' elements and the seed into the warp's hash set; returns the
// number of distinct elements, or -1 when there are more than kMedCap.
__device__ __forceinline__ int warp_medium_insert(const PlateauSets& st, unsigned e0, unsigned e1, uint32_t seed,
                                                  MedBuf& mb, unsigned lane) {
    for (int i = lane; i < kMedHash; i += 32) mb.table[i] = kNone;
    if (lane == 0) mb.count = 0;
    __syncwarp();
    bool over = false;
    auto insert = [&](uint32_t x) {
        unsigned h = (x * 2654435761u) >> (32 - 8);  // kMedHash = 2^8 slots
        for (int probe = 0; probe < kMedHash; ++probe, h = (h + 1) & (kMedHash - 1)) {
            const uint32_t prev = atomicCAS(&mb.table[h], kNone, x);
            if (prev == x) return;
            if (prev == kNone) {
                if (atomicAdd(&mb.count, 1u) >= static_cast<unsigned>(kMedCap)) over = true;
                return;
            }
        }
        over = true;  // table full (only after more than kMedCap insertions)
    };
    // The warp streams through the predecessors' sets one set at a time, 32 elements a step
    // (lanes take 32 edges' sizes and offsets at once, then broadcast them): a set of
    // thousands of elements costs its length / 32 steps, not its length on one lane.
    bool stop = false;
    for (unsigned eb = e0; eb < e1 && !stop; eb += 32) {
        uint32_t len = 0;
        unsigned long long off = 0;
        if (eb + lane < e1) {
            const uint32_t q = __ldg(st.edges + eb + lane);
            len = __ldg(st.slen + q);
            off = __ldg(st.soff + q);
        }
        const unsigned ne = min(32u, e1 - eb);
        for (unsigned t = 0; t < ne && !stop; ++t) {
            const uint32_t tl = __shfl_sync(0xFFFFFFFFu, len, t);
            const uint32_t* src = st.pool + __shfl_sync(0xFFFFFFFFu, off, t);
            for (uint32_t b = 0; b < tl; b += 32) {  // warp-uniform steps
                if (b + lane < tl) insert(__ldg(src + b + lane));
                // past the cap on any lane: the union takes the sort path
                if (__any_sync(0xFFFFFFFFu, over)) {
                    stop = true;
                    break;
                }
            }
        }
    }
    if (seed != kNone && lane == 0 && !over) insert(seed);
    if (__any_sync(0xFFFFFFFFu, over)) return -1;
    __syncwarp();
    const unsigned n = mb.count;
    return n > static_cast<unsigned>(kMedCap) ? -1 : static_cast<int>(n);
}

// The union gathered by warp_medium_insert (n elements), sorted ascending: up to 32 elements
// in the lanes' registers, more in mb.sorted. Lane l then holds element l (value, keep = l < n)
// when n <= 32.
__device__ __forceinline__ void warp_medium_sort(MedBuf& mb, int n, unsigned lane, uint32_t& value) {
    if (lane == 0) mb.count = 0;
    __syncwarp();
    for (int i = lane; i < kMedHash; i += 32) {
        const uint32_t x = mb.table[i];
        if (x != kNone) mb.sorted[atomicAdd(&mb.count, 1u)] = x;
    }
    __syncwarp();
    if (n <= 32) {
        uint32_t v = static_cast<int>(lane) < n ? mb.sorted[lane] : kNone;
        for (int k = 2; k <= 32; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                const uint32_t other = __shfl_xor_sync(0xFFFFFFFFu, v, j);
                const bool ascending = (lane & k) == 0;
                const bool lower = (lane & j) == 0;
                v = (lower == ascending) ? min(v, other) : max(v, other);
            }
        value = v;
        return;
    }
    int N = 64;
    while (N < n) N <<= 1;
    for (int i = n + lane; i < N; i += 32) mb.sorted[i] = kNone;
    __syncwarp();
    for (int k = 2; k <= N; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < N; i += 32) {
                const int q = i ^ j;
                if (q > i) {
                    const uint32_t a = mb.sorted[i], b = mb.sorted[q];
                    if (((i & k) == 0) ? (a > b) : (a < b)) {
                        mb.sorted[i] = b;
                        mb.sorted[q] = a;
                    }
                }
            }
            __syncwarp();
        }
    value = kNone;
}

// Seeds, m and set sizes of one level, one warp per plateau. Small and medium unions are
// merged here and kept, sorted, in mtmp until level_write copies them to the pool; larger ones
// go to the sort path and plateaus with many in-edges to level_heavy. A union that finds no
// room in mtmp is merged again by level_write (small) or takes the sort path (medium).
__global__ void level_seeds(PlateauSets st, size_t begin, size_t end, unsigned slab) {
    __shared__ uint32_t wbuf[kLevelWarps][kSmallSet];
    __shared__ unsigned int wfill[kLevelWarps];
    __shared__ MedBuf med[kLevelWarps];
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // The warp takes mtmp space in slabs (one atomic per slab, not one per union on a counter
    // every warp of the level shares); returns the start of k elements, or ~0 when full.
    unsigned long long slab_base = 0, slab_left = 0;
    auto take = [&](unsigned long long k) -> unsigned long long {
        if (k > slab_left) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&st.info[4], static_cast<unsigned long long>(slab));
            slab_base = __shfl_sync(0xFFFFFFFFu, b, 0);
            slab_left = slab_base + slab <= st.mtmp_cap ? slab : 0;
        }
        if (k > slab_left) return ~0ull;
        const unsigned long long at = slab_base;
        slab_base += k;
        slab_left -= k;
        return at;
    };
    const size_t stride = static_cast<size_t>(gridDim.x) * kLevelWarps;
    for (size_t i = begin + static_cast<size_t>(blockIdx.x) * kLevelWarps + w; i < end; i += stride) {
        const size_t L = i - begin;
        const uint32_t p = st.order[i];
        const unsigned e0 = st.eoff[p], e1 = st.eoff[p + 1];
        if (e1 - e0 > kHeavyDegree) {
            if (lane == 0) {
                st.big[L] = 1;
                st.cnt[L] = 0;
                st.heavy[atomicAdd(&st.info[0], 1ull)] = static_cast<uint32_t>(L);
            }
            continue;
        }
        uint32_t mp = kNone;
        unsigned long long u = 0;
        for (unsigned e = e0 + lane; e < e1; e += 32) {
            const uint32_t q = __ldg(st.edges + e);
            mp = min(mp, __ldg(st.m + q));
            u += __ldg(st.slen + q);
        }
        mp = warp_min_u32(mp);
        u = warp_sum_u64(u);
        const uint32_t own = st.minrank[p];
        const uint32_t seed = own < mp ? own : kNone;
        if (lane == 0) {
            st.m[p] = min(own, mp);
            st.seed[p] = seed;
        }
        const unsigned long long total = u + (seed != kNone ? 1u : 0u);
        if (total <= kSmallSet) {
            uint32_t v;
            bool keep;
            int rank;
            const int k = warp_small_union(st, e0, e1, seed, wbuf[w], &wfill[w], lane, v, keep, rank);
            const unsigned long long at = k > 0 ? take(static_cast<unsigned long long>(k)) : 0ull;
            if (at != ~0ull) {
                if (keep) st.mtmp[at + rank] = v;
                if (lane == 0) st.mtoff[L] = at;
            }
            if (lane == 0) {
                st.big[L] = at != ~0ull ? 2 : 0;
                st.cnt[L] = static_cast<unsigned long long>(k);
            }
        } else {
            int k = total <= kMedSum ? warp_medium_insert(st, e0, e1, seed, med[w], lane) : -1;
            if (k >= 0) {  // a medium union: sorted now, kept in mtmp until level_write
                uint32_t v;
                warp_medium_sort(med[w], k, lane, v);
                const unsigned long long at = take(static_cast<unsigned long long>(k));
                if (at != ~0ull) {
                    if (k <= 32) {
                        if (static_cast<int>(lane) < k) st.mtmp[at + lane] = v;
                    } else {
                        for (int r = lane; r < k; r += 32) st.mtmp[at + r] = med[w].sorted[r];
                    }
                    if (lane == 0) st.mtoff[L] = at;
                } else {
                    k = -1;  // no room left: the sort path takes it
                }
            }
            if (lane == 0) {
                if (k >= 0) {
                    st.big[L] = 2;
                    st.cnt[L] = static_cast<unsigned long long>(k);
                } else {
                    st.big[L] = 1;
                    st.cnt[L] = 0;
                    st.big_list[atomicAdd(&st.info[1], 1ull)] = static_cast<uint32_t>(L);
                    atomicAdd(&st.info[2], total);
                }
            }
        }
    }
}

// Seeds and m of the high in-degree plateaus, one block each; they all take the sort path.
__global__ void level_heavy(PlateauSets st, size_t begin) {
    __shared__ uint32_t smin[32];
    __shared__ unsigned long long ssum[32];
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned long long nh = st.info[0];
    for (unsigned long long h = blockIdx.x; h < nh; h += gridDim.x) {
        const uint32_t L = st.heavy[h];
        const uint32_t p = st.order[begin + L];
        const unsigned e0 = st.eoff[p], e1 = st.eoff[p + 1];
        uint32_t mp = kNone;
        unsigned long long u = 0;
        for (unsigned e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            const uint32_t q = __ldg(st.edges + e);
            mp = min(mp, __ldg(st.m + q));
            u += __ldg(st.slen + q);
        }
        mp = warp_min_u32(mp);
        u = warp_sum_u64(u);
        if (lane == 0) {
            smin[w] = mp;
            ssum[w] = u;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (unsigned k = 1; k < nw; ++k) {
                mp = min(mp, smin[k]);
                u += ssum[k];
            }
            const uint32_t own = st.minrank[p];
            const uint32_t seed = own < mp ? own : kNone;
            st.m[p] = min(own, mp);
            st.seed[p] = seed;
            st.big_list[atomicAdd(&st.info[1], 1ull)] = L;
            atomicAdd(&st.info[2], u + (seed != kNone ? 1u : 0u));
        }
        __syncthreads();
    }
}

// Sort path: every element of every predecessor set (and the own seed) of the big plateaus
// becomes a key (plateau << shift | rank); sorting and removing duplicates yields each union.
// The plateau of a key is its index in the level's big list, above the rank bits (32 bits
// in the single-block merge); keys are 32-bit whenever ranks and big-list indices fit together,
// else 64-bit, and the radix sort covers the used bits only.
template <class K>
__device__ __forceinline__ uint32_t key_plateau(const PlateauSets& st, K key, int shift) {
    return st.big_list[static_cast<uint32_t>(key >> shift)];
}

// In-degrees of the big plateaus (their edges are spread over the whole grid below).
__global__ void level_big_degrees(PlateauSets st, size_t begin, unsigned long long* __restrict__ deg) {
    const unsigned long long nbig = st.info[1];
    PMA_GRID_STRIDE(b, nbig) {
        const uint32_t p = st.order[begin + st.big_list[b]];
        deg[b] = st.eoff[p + 1] - st.eoff[p];
    }
}

// One thread per in-edge of a big plateau (t over the concatenated edge lists, doff = the
// exclusive scan of the in-degrees): a giant plateau with a million in-edges is spread over
// the whole GPU instead of one block. The in-edges of a block mostly belong to one plateau and
// bring the same seeds many times, so each block keeps only the first copy of a key (shared-
// memory hash set; a key that finds no free slot is emitted anyway, the sort and unique that
// follow are exact). Keys of a warp are placed with one atomic.
constexpr int kMergeTable = 2048;

template <class K>
__global__ void __launch_bounds__(256) level_expand(PlateauSets st, size_t begin,
                                                    const unsigned long long* __restrict__ doff,
                                                    const unsigned long long* __restrict__ deg,
                                                    unsigned long long nbig, K* __restrict__ keys,
                                                    unsigned long long cap, int shift) {
    __shared__ K table[kMergeTable];
    const unsigned lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
    const unsigned long long total = doff[nbig - 1] + deg[nbig - 1];
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    const K empty = ~static_cast<K>(0);
    // block-uniform trip count (the table is cleared between rounds)
    for (unsigned long long tb = blockIdx.x * static_cast<unsigned long long>(blockDim.x); tb < total;
         tb += stride) {
        for (int i = threadIdx.x; i < kMergeTable; i += blockDim.x) table[i] = empty;
        __syncthreads();
        const unsigned long long t = tb + threadIdx.x;
        uint32_t len = 0;
        const uint32_t* src = st.pool;
        K hi = 0;
        if (t < total) {
            unsigned long long lo = 0, up = nbig;  // last b with doff[b] <= t
            while (up - lo > 1) {
                const unsigned long long mid = (lo + up) >> 1;
                if (doff[mid] <= t) lo = mid;
                else up = mid;
            }
            const uint32_t L = st.big_list[lo];
            const uint32_t p = st.order[begin + L];
            const uint32_t q = __ldg(st.edges + st.eoff[p] + (t - doff[lo]));
            len = __ldg(st.slen + q);
            src = st.pool + __ldg(st.soff + q);
            hi = static_cast<K>(lo) << shift;
        }
        // The warp's 32 sets are expanded together, 32 elements per round: element u of the
        // concatenation belongs to the last lane whose exclusive offset is <= u (a shuffle
        // binary search), so one long set does not hold the warp for its whole length.
        uint32_t incl = len;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t2 = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<unsigned>(o)) incl += t2;
        }
        const uint32_t excl = incl - len;
        const uint32_t wtotal = __shfl_sync(0xFFFFFFFFu, incl, 31);
        for (uint32_t u0 = 0; u0 < wtotal; u0 += 32) {
            const uint32_t u = u0 + lane;
            int owner = 0;
            for (int step = 16; step >= 1; step >>= 1) {
                const uint32_t e = __shfl_sync(0xFFFFFFFFu, excl, owner + step);
                if (e <= u) owner += step;
            }
            const uint32_t* osrc = reinterpret_cast<const uint32_t*>(
                __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(src), owner));
            const K ohi = __shfl_sync(0xFFFFFFFFu, hi, owner);
            const uint32_t oexcl = __shfl_sync(0xFFFFFFFFu, excl, owner);
            K key = 0;
            bool emit = false;
            if (u < wtotal) {
                key = ohi | static_cast<K>(__ldg(osrc + (u - oexcl)));
                emit = true;
                unsigned h = static_cast<unsigned>((static_cast<unsigned long long>(key) * 0x9E3779B97F4A7C15ull) >> 40) &
                             (kMergeTable - 1);
                for (int probe = 0; probe < 8; ++probe, h = (h + 1) & (kMergeTable - 1)) {
                    const K prev = atomicCAS(&table[h], empty, key);
                    if (prev == empty) break;
                    if (prev == key) {
                        emit = false;
                        break;
                    }
                }
            }
            const unsigned m = __ballot_sync(0xFFFFFFFFu, emit);
            if (!m) continue;
            const int leader = __ffs(m) - 1;
            unsigned long long pos = 0;
            if (static_cast<int>(lane) == leader) pos = atomicAdd(&st.info[3], static_cast<unsigned long long>(__popc(m)));
            pos = __shfl_sync(0xFFFFFFFFu, pos, leader) + __popc(m & lt);
            if (emit && pos < cap) keys[pos] = key;
        }
        __syncthreads();
    }
    // own seeds
    for (unsigned long long b = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; b < nbig;
         b += stride) {
        const uint32_t L = st.big_list[b];
        const uint32_t p = st.order[begin + L];
        if (st.seed[p] == kNone) continue;
        const unsigned long long pos = atomicAdd(&st.info[3], 1ull);
        if (pos < cap) keys[pos] = (static_cast<K>(b) << shift) | static_cast<K>(st.seed[p]);
    }
}

// Sizes and first positions of the merged unions (keys sorted, duplicates removed).
template <class K>
__global__ void level_runs(const K* __restrict__ keys, size_t n, PlateauSets st, int shift) {
    PMA_GRID_STRIDE(i, n) {
        const K hi = keys[i] >> shift;
        const uint32_t L = key_plateau(st, keys[i], shift);
        if (i == 0 || (keys[i - 1] >> shift) != hi) st.first[L] = i;
        atomicAdd(&st.cnt[L], 1ull);
    }
}

// Sort path of a level whose big unions hold few keys in all (kSmallMerge): one block expands,
// sorts (bitonic, shared memory) and de-duplicates them, and fills cnt/first like level_runs.
// No host round trip: the number of merged keys stays on the device (*merged).
constexpr int kSmallMerge = 4096;

__global__ void __launch_bounds__(1024) level_merge_small(PlateauSets st, size_t begin,
                                                          unsigned long long* __restrict__ keys,
                                                          unsigned long long* __restrict__ merged) {
    __shared__ unsigned long long sk[kSmallMerge];
    __shared__ unsigned int s_count;
    __shared__ unsigned int wsum[32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned long long nbig = st.info[1];
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    for (unsigned long long b = warp; b < nbig; b += nw) {
        const uint32_t L = st.big_list[b];
        const uint32_t p = st.order[begin + L];
        const unsigned e0 = st.eoff[p], e1 = st.eoff[p + 1];
        const unsigned long long hi = static_cast<unsigned long long>(b) << 32;
        // lanes take 32 edges' sets at once and reserve their room; the warp then copies the
        // sets one after another, 32 elements a step
        for (unsigned eb = e0; eb < e1; eb += 32) {
            uint32_t len = 0;
            unsigned long long off = 0;
            unsigned pos = 0;
            if (eb + lane < e1) {
                const uint32_t q = __ldg(st.edges + eb + lane);
                len = __ldg(st.slen + q);
                off = __ldg(st.soff + q);
                pos = atomicAdd(&s_count, len);
            }
            const unsigned ne = min(32u, e1 - eb);
            for (unsigned t = 0; t < ne; ++t) {
                const uint32_t tl = __shfl_sync(0xFFFFFFFFu, len, t);
                const unsigned tp = __shfl_sync(0xFFFFFFFFu, pos, t);
                const uint32_t* src = st.pool + __shfl_sync(0xFFFFFFFFu, off, t);
                for (uint32_t r = lane; r < tl; r += 32)
                    if (tp + r < kSmallMerge) sk[tp + r] = hi | __ldg(src + r);
            }
        }
        if (lane == 0 && st.seed[p] != kNone) {
            const unsigned pos = atomicAdd(&s_count, 1u);
            if (pos < kSmallMerge) sk[pos] = hi | st.seed[p];
        }
    }
    __syncthreads();
    const unsigned n = min(s_count, static_cast<unsigned>(kSmallMerge));
    unsigned N = 1;
    while (N < n) N <<= 1;
    for (unsigned i = n + threadIdx.x; i < N; i += blockDim.x) sk[i] = ~0ull;
    __syncthreads();
    for (unsigned k = 2; k <= N; k <<= 1)  // bitonic sort, ascending
        for (unsigned j = k >> 1; j > 0; j >>= 1) {
            for (unsigned i = threadIdx.x; i < N; i += blockDim.x) {
                const unsigned q = i ^ j;
                if (q > i) {
                    const unsigned long long a = sk[i], c = sk[q];
                    if (((i & k) == 0) ? (a > c) : (a < c)) {
                        sk[i] = c;
                        sk[q] = a;
                    }
                }
            }
            __syncthreads();
        }
    // first copies, compacted in order: each thread owns a contiguous run of 4 positions
    const unsigned per = (N + blockDim.x - 1) / blockDim.x;  // <= 4
    const unsigned i0 = threadIdx.x * per;
    unsigned mine = 0;
    for (unsigned t = 0; t < per; ++t) {
        const unsigned i = i0 + t;
        if (i < n && (i == 0 || sk[i - 1] != sk[i])) ++mine;
    }
    unsigned incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<unsigned>(o)) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned run = 0;
        for (unsigned w = 0; w < nw; ++w) {
            const unsigned v = wsum[w];
            wsum[w] = run;
            run += v;
        }
        *merged = run;
    }
    __syncthreads();
    unsigned u = wsum[warp] + incl - mine;
    for (unsigned t = 0; t < per; ++t) {
        const unsigned i = i0 + t;
        if (!(i < n && (i == 0 || sk[i - 1] != sk[i]))) continue;
        const uint32_t bhi = static_cast<uint32_t>(sk[i] >> 32);  // index in the big list
        const uint32_t L = st.big_list[bhi];
        keys[u] = sk[i];
        // sk[i] is a first copy, so sk[i - 1] is the previous distinct key
        if (i == 0 || static_cast<uint32_t>(sk[i - 1] >> 32) != bhi) st.first[L] = u;
        atomicAdd(&st.cnt[L], 1ull);
        ++u;
    }
}

// Writes the small unions (recomputed) and the list offsets of all plateaus of the level.
__global__ void level_write(PlateauSets st, size_t begin, size_t end, const unsigned long long* __restrict__ base) {
    __shared__ uint32_t wbuf[kLevelWarps][kSmallSet];
    __shared__ unsigned int wfill[kLevelWarps];
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t stride = static_cast<size_t>(gridDim.x) * kLevelWarps;
    const unsigned long long b0 = *base;
    for (size_t i = begin + static_cast<size_t>(blockIdx.x) * kLevelWarps + w; i < end; i += stride) {
        const size_t L = i - begin;
        const uint32_t p = st.order[i];
        const unsigned long long pos = b0 + st.off[L], k = st.cnt[L];
        // A list that does not fit is recorded empty so later levels never read past the
        // pool; the overflow flag makes the host redo the sweep with a larger pool.
        const bool fits = pos + k <= st.pool_cap;
        if (lane == 0) {
            st.soff[p] = fits ? pos : 0;
            st.slen[p] = fits ? static_cast<uint32_t>(k) : 0u;
            if (!fits) atomicOr(st.err, 2u);
        }
        if (st.big[L] == 1) continue;
        if (st.big[L] == 2) {  // sorted by level_seeds
            const uint32_t* src = st.mtmp + st.mtoff[L];
            for (unsigned long long r = lane; r < k; r += 32)
                if (fits) st.pool[pos + r] = src[r];
            continue;
        }
        uint32_t v;
        bool keep;
        int rank;
        warp_small_union(st, st.eoff[p], st.eoff[p + 1], st.seed[p], wbuf[w], &wfill[w], lane, v, keep, rank);
        if (keep && fits) st.pool[pos + rank] = v;
    }
}

template <class K>
__global__ void level_copy_big(const K* __restrict__ keys, size_t n_host, PlateauSets st,
                               const unsigned long long* __restrict__ base, int shift,
                               const unsigned long long* __restrict__ n_dev) {
    const unsigned long long b0 = *base;
    const K low = (static_cast<K>(1) << shift) - 1;
    const size_t n = n_dev ? static_cast<size_t>(*n_dev) : n_host;
    PMA_GRID_STRIDE(i, n) {
        const uint32_t L = key_plateau(st, keys[i], shift);
        const unsigned long long pos = b0 + st.off[L], r = i - st.first[L];  // rank within the set
        if (r >= st.cnt[L]) {  // keys and set bounds disagree: never write outside the set
            atomicOr(st.err, 32u);
            continue;
        }
        if (pos + st.cnt[L] <= st.pool_cap) st.pool[pos + r] = static_cast<uint32_t>(keys[i] & low);
    }
}

__global__ void level_advance(unsigned long long* __restrict__ base, const unsigned long long* __restrict__ off,
                              const unsigned long long* __restrict__ cnt, size_t nlev) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *base += off[nlev - 1] + cnt[nlev - 1];
}

__global__ void throat_hashes(const unsigned long long* __restrict__ soff, const uint32_t* __restrict__ slen,
                              const uint32_t* __restrict__ pool, const uint32_t* __restrict__ multi,
                              size_t nm, unsigned long long* __restrict__ h1o,
                              unsigned long long* __restrict__ h2o) {
    PMA_GRID_STRIDE(i, nm) {
        const uint32_t p = multi[i];
        unsigned long long a, b;
        list_hash(pool + soff[p], slen[p], a, b);
        h1o[i] = a;
        h2o[i] = b;
    }
}

__global__ void flag_multi(const uint32_t* __restrict__ slen, size_t np, uint8_t* __restrict__ f) {
    PMA_GRID_STRIDE(p, np) f[p] = slen[p] >= 2;
}

// Group starts among plateaus sorted by (h1, h2); verifies list equality within groups.
__global__ void group_starts(const uint32_t* __restrict__ sorted_p, const unsigned long long* __restrict__ h1,
                             const unsigned long long* __restrict__ h2, size_t nm,
                             const unsigned long long* __restrict__ soff, const uint32_t* __restrict__ slen,
                             const uint32_t* __restrict__ pool, uint32_t* __restrict__ start,
                             unsigned int* __restrict__ err) {
    PMA_GRID_STRIDE(i, nm) {
        bool s = (i == 0) || h1[i] != h1[i - 1] || h2[i] != h2[i - 1];
        // equal first hashes, different second ones: sorted by the first hash alone, such sets
        // may interleave (the host then sorts by both)
        if (i > 0 && h1[i] == h1[i - 1] && h2[i] != h2[i - 1]) atomicOr(err, 64u);
        if (!s) {
            const uint32_t a = sorted_p[i], b = sorted_p[i - 1];
            bool eq = slen[a] == slen[b];
            for (uint32_t k = 0; eq && k < slen[a]; ++k) eq = pool[soff[a] + k] == pool[soff[b] + k];
            if (!eq) atomicOr(err, 4u);  // 128-bit hash collision between different sets
        }
        start[i] = s ? 1u : 0u;
    }
}

struct GroupOut {
    uint32_t* group_of;             // per multi index (sorted order) -> group
    unsigned long long* gvol;       // per group
    unsigned long long* gfirst;     // per group: smallest root voxel index
    uint32_t* grep;                 // per group: representative plateau
};

__global__ void group_reduce(const uint32_t* __restrict__ sorted_p, const uint32_t* __restrict__ gid,
                             size_t nm, const unsigned int* __restrict__ psize,
                             const uint32_t* __restrict__ roots, GroupOut go,
                             uint32_t* __restrict__ plateau_group) {
    PMA_GRID_STRIDE(i, nm) {
        const uint32_t p = sorted_p[i];
        const uint32_t gr = gid[i];
        plateau_group[p] = gr;
        atomicAdd(&go.gvol[gr], static_cast<unsigned long long>(psize[p]));
        atomicMin(&go.gfirst[gr], static_cast<unsigned long long>(roots[p]));
        if (i == 0 || gid[i - 1] != gr) go.grep[gr] = p;
    }
}

struct PoreAcc {
    const uint32_t* rank2pore;       // ball rank -> pore index (kNone if not a seed)
    unsigned long long* pvol;
    unsigned int* pbound;
};

__global__ void pore_accumulate(const unsigned long long* __restrict__ soff, const uint32_t* __restrict__ slen,
                                const uint32_t* __restrict__ pool, const unsigned int* __restrict__ psize,
                                const unsigned int* __restrict__ pface, size_t np, PoreAcc pa) {
    const unsigned lane = threadIdx.x & 31;
    PMA_GRID_STRIDE(p, np) {
        const uint32_t n = slen[p];
        const uint32_t* s = pool + soff[p];
        // plateaus of one pore met by a warp add their sizes with one atomic
        const uint32_t pore = n == 1 ? pa.rank2pore[s[0]] : kNone;
        const unsigned long long size = n == 1 ? psize[p] : 0ull;
        const unsigned peers = __match_any_sync(__activemask(), pore);
        unsigned long long sum = 0;
        for (unsigned m = peers; m; m &= m - 1) sum += __shfl_sync(peers, size, __ffs(m) - 1);
        if (pore != kNone && static_cast<int>(lane) == __ffs(peers) - 1) atomicAdd(&pa.pvol[pore], sum);
        if (pface[p])
            for (uint32_t k = 0; k < n; ++k) pa.pbound[pa.rank2pore[s[k]]] = 1;
    }
}

__global__ void plateau_labels(const unsigned long long* __restrict__ soff, const uint32_t* __restrict__ slen,
                               const uint32_t* __restrict__ pool, const uint32_t* __restrict__ rank2id,
                               const uint32_t* __restrict__ plateau_group,
                               const uint32_t* __restrict__ group_tid, size_t np,
                               uint32_t* __restrict__ plabel) {
    PMA_GRID_STRIDE(p, np) {
        const uint32_t n = slen[p];
        uint32_t lab = 0;
        if (n == 1) lab = rank2id[pool[soff[p]]];
        else if (n >= 2) lab = group_tid[plateau_group[p]];
        plabel[p] = lab;
    }
}

__global__ void voxel_labels(const uint32_t* __restrict__ pid, const uint32_t* __restrict__ plabel,
                             size_t n, uint32_t* __restrict__ labels) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t p = pid[v];
        labels[v] = (p == kNone) ? 0u : plabel[p];
    }
}

// Old -> new label remap by binary search in sorted old ids.
__global__ void remap_labels(uint32_t* __restrict__ labels, size_t n, const uint32_t* __restrict__ old_ids,
                             const uint32_t* __restrict__ new_ids, uint32_t m) {
    const uint32_t first = m ? old_ids[0] : 0xFFFFFFFFu;  // pore labels are below every type id
    PMA_GRID_STRIDE(v, n) {
        const uint32_t l = labels[v];
        if (l == 0 || l < first || m == 0) continue;
        uint32_t lo = 0, hi = m;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (old_ids[mid] < l) lo = mid + 1;
            else hi = mid;
        }
        if (lo < m && old_ids[lo] == l) labels[v] = new_ids[lo];
    }
}

__global__ void to_group_index(const uint32_t* __restrict__ excl, const uint32_t* start, size_t m,
                               uint32_t* out) {
    PMA_GRID_STRIDE(i, m) out[i] = excl[i] + start[i] - 1u;
}

// Pore ids of each group's seed list (ascending ranks give ascending ids).
__global__ void gather_lists(const unsigned long long* __restrict__ soff, const uint32_t* __restrict__ slen,
                             const uint32_t* __restrict__ pool, const uint32_t* __restrict__ rep,
                             const unsigned long long* __restrict__ roff, size_t ng,
                             const uint32_t* __restrict__ rank2id, uint32_t* __restrict__ out) {
    PMA_GRID_STRIDE(gi, ng) {
        const uint32_t p = rep[gi];
        for (uint32_t k = 0; k < slen[p]; ++k) out[roff[gi] + k] = rank2id[pool[soff[p] + k]];
    }
}

template <class T>
T* buf(pma_ctx* ctx, const char* tag, size_t count) {
    return static_cast<T*>(ctx->scratch(tag, std::max<size_t>(count, 1) * sizeof(T)));
}

}  // namespace

void reference_type_ids(pma_ctx* ctx, pma_table* t, uint32_t* labels, const uint32_t* crad2, pma_dims d,
                        pma_stencil st);

pma_table* pores(pma_ctx* ctx, const uint8_t* mask, const uint32_t* edt2, const uint32_t* crad2,
                 pma_dims d, pma_stencil st, uint32_t* labels) {
    KernelTimer kt_stage(ctx, "stage_pores");  // the whole stage, for the untimed remainder
    check_dims(d);
    PMA_REQUIRE(mask && edt2 && crad2 && labels, PMA_ERR_ARGUMENT, "pma_pores: null device pointer");
    cudaStream_t s = ctx->stream;
    const size_t n = voxels(d);
    const Grid g{d.sx, d.sy, d.sz};
    const int d3q7 = st == PMA_D3Q7 ? 1 : 0;
    const unsigned G = grid_for(ctx, n);
    int64_t* d_count = buf<int64_t>(ctx, "pores.count", 4);
    unsigned int* err = reinterpret_cast<unsigned int*>(d_count + 2);
    PMA_CUDA(cudaMemsetAsync(d_count, 0, 32, s));

    // a8: maximum balls in z, x, y scan order (PoreAndThroatComputer.cpp:93-119) = linear order.
    uint8_t* flags = buf<uint8_t>(ctx, "pores.flags", n);
    flag_outer<<<G, 256, 0, s>>>(mask, n, flags);
    ctx->check_launch("flag_outer");
    uint32_t* balls = buf<uint32_t>(ctx, "pores.balls", n);
    const int64_t nb = select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), flags, balls,
                                      static_cast<int64_t>(n), d_count);
    uint32_t* ball_r2 = buf<uint32_t>(ctx, "pores.ball_r2", nb);
    if (nb) {
        gather_u32<<<grid_for(ctx, nb), 256, 0, s>>>(edt2, balls, nb, ball_r2);
        ctx->check_launch("gather_u32");
    }
    // std::sort with the reference's comparator (PoreAndThroatComputer.cpp:121-122), run on
    // host threads (ordered_sort: the same permutation) while the plateau kernels below run.
    // The items are 8-byte (r2, voxel index) pairs compared on r2 alone: std::sort's moves
    // depend only on comparison results, so the permutation equals the one the reference's
    // 16-byte balls go through, and the sorted items carry each rank's voxel. They are packed
    // on the device and sorted in a page-locked buffer of the context.
    auto kt_balls_host = std::make_unique<KernelTimer>(ctx, "pores_balls_to_host");
    auto* items = static_cast<unsigned long long*>(ctx->host_buffer("pores.items", nb * 8));
    auto* voxel_of_rank = static_cast<uint32_t*>(ctx->host_buffer("pores.voxel_of_rank", nb * 4));
    if (nb) {
        auto* d_items = buf<unsigned long long>(ctx, "pores.d_items", nb);
        pack_items<<<grid_for(ctx, nb), 256, 0, s>>>(ball_r2, balls, nb, d_items);
        ctx->check_launch("pack_items");
        copy_to_host(ctx, items, d_items, nb * 8);
        ctx->sync();
    }
    kt_balls_host.reset();
    struct Joiner {
        std::thread t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } sorter;
    // up to 16 leaf tasks (levels 4) where the host has the cores and each leaf gets at least
    // 2^16 balls: the leaves' sorts are most of the time, the top partition steps run on one
    // to eight threads; small volumes (the batched and serving forms run many at once) sort
    // on this one thread
    int sort_levels = 0;
    while (sort_levels < 4 && (2u << sort_levels) <= std::thread::hardware_concurrency() &&
           (static_cast<unsigned long long>(nb) >> (16 + sort_levels + 1)) > 0)
        ++sort_levels;
    // then the voxel of each rank, taken from the sorted items on host threads too
    sorter.t = std::thread([items, voxel_of_rank, nb, sort_levels] {
        ordered_sort(
            items, items + nb,
            [](unsigned long long a, unsigned long long b) { return (a >> 32) > (b >> 32); }, sort_levels);
        const int64_t m = nb;
        auto gather = [&](int64_t lo, int64_t hi) {
            for (int64_t r = lo; r < hi; ++r) voxel_of_rank[r] = static_cast<uint32_t>(items[r]);
        };
        const int nt = m >= (1 << 20) ? (1 << sort_levels) : 1;
        std::vector<std::thread> ts;
        for (int t = 1; t < nt; ++t) {
            try {
                ts.emplace_back(gather, m * t / nt, m * (t + 1) / nt);
            } catch (const std::system_error&) {
                gather(m * t / nt, m * (t + 1) / nt);  // no thread to be had: in line
            }
        }
        gather(0, m / nt);
        for (auto& th : ts) th.join();
    });

    // Plateaus: connected sets of equal crad under the stencil.
    uint32_t* pid = buf<uint32_t>(ctx, "pores.pid", n);  // root voxel, then plateau id
    uf_init<<<G, 256, 0, s>>>(crad2, g, n, d3q7, pid);
    ctx->check_launch("uf_init");
    {
        KernelTimer kt(ctx, "uf_jump");
        if (n >= kJumpMinVoxels) {
            unsigned int* changed =
                reinterpret_cast<unsigned int*>(buf<unsigned long long>(ctx, "pores.jump", kJumpPasses));
            PMA_CUDA(cudaMemsetAsync(changed, 0, kJumpPasses * 4, s));
            for (int pass = 0; pass < kJumpPasses; ++pass) uf_jump<<<G, 256, 0, s>>>(n, pid, changed, pass);
            ctx->count_launch(kJumpPasses - 1);
            ctx->check_launch("uf_jump");
        }
    }
    {
        KernelTimer kt(ctx, "uf_hook");
        if (n >= kJumpMinVoxels) {
            // parent pairs, then their unions (the buffer grows to what a call needed)
            auto* pcount = reinterpret_cast<unsigned long long*>(d_count + 1);  // free until the edges
            unsigned long long pcap = std::max<unsigned long long>(
                std::max<unsigned long long>(n / 64, 1ull << 20), ctx->cached_bytes("pores.uf_pairs") / 8);
            unsigned long long npairs = 0;
            unsigned long long* pairs = nullptr;
            for (int attempt = 0;; ++attempt) {
                pairs = buf<unsigned long long>(ctx, "pores.uf_pairs", pcap);
                PMA_CUDA(cudaMemsetAsync(pcount, 0, 8, s));
                uf_pairs<<<G, 256, 0, s>>>(crad2, g, n, d3q7, pid, pairs, pcap, pcount);
                ctx->check_launch("uf_pairs");
                PMA_CUDA(cudaMemcpyAsync(&npairs, pcount, 8, cudaMemcpyDeviceToHost, s));
                ctx->sync();
                if (npairs <= pcap) break;
                PMA_REQUIRE(attempt < 3, PMA_ERR_INTERNAL, "pma_pores: plateau pair count did not settle");
                pcap = npairs + npairs / 8 + 1024;
            }
            if (npairs) {
                uf_union_pairs<<<grid_for(ctx, npairs), 256, 0, s>>>(pairs, npairs, pid, err,
                                                                      ctx->limits.union_limit);
                ctx->check_launch("uf_union_pairs");
            }
        } else {
            uf_hook<<<G, 256, 0, s>>>(crad2, g, n, d3q7, pid, err, ctx->limits.union_limit);
        }
    }
    ctx->check_launch("uf_hook");
    auto kt_ids = std::make_unique<KernelTimer>(ctx, "plateau_ids");
    uf_flatten<<<G, 256, 0, s>>>(n, pid);
    ctx->check_launch("uf_flatten");
    flag_roots<<<G, 256, 0, s>>>(pid, n, flags);
    ctx->check_launch("flag_roots");
    uint32_t* roots = buf<uint32_t>(ctx, "pores.roots", n);
    const int64_t np = select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), flags, roots,
                                      static_cast<int64_t>(n), d_count);
    if (np) {
        scatter_pid<<<grid_for(ctx, np), 256, 0, s>>>(roots, np, labels);  // labels as scratch
        ctx->check_launch("scatter_pid");
        to_pid<<<G, 256, 0, s>>>(labels, n, np, pid, err);
        ctx->check_launch("to_pid");
    }
    {
        // the union-find's own bound (bit 1) is read here: the level sweep reuses the word
        unsigned int h_err = 0;
        PMA_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        PMA_REQUIRE(!(h_err & 1u), PMA_ERR_LIMIT, "pma_pores: plateau union-find did not converge");
        PMA_REQUIRE(!(h_err & 8u), PMA_ERR_INTERNAL, "pma_pores: plateau labelling left a non-root parent");
    }
    kt_ids.reset();
    // Edges between plateaus, sorted by destination.
    auto kt_edges = std::make_unique<KernelTimer>(ctx, "plateau_edges");
    int sb = 1;  // bits of a plateau id
    while (sb < 32 && (1ull << sb) < static_cast<unsigned long long>(np)) ++sb;
    auto* ecount = reinterpret_cast<unsigned long long*>(d_count + 1);
    // One pass writes the edges into a buffer of at least n/8 entries, or of what an earlier
    // call needed (the edges kept after the per-block de-duplication are far fewer than the
    // voxels); when they do not fit, the pass is repeated with the size it counted.
    unsigned long long ecap = std::max<unsigned long long>(
        std::max<unsigned long long>(n / 8, 1ull << 20), ctx->cached_bytes("pores.edges_raw") / 8);
    unsigned long long* edges_raw = nullptr;
    unsigned long long ne_kept = 0;
    for (int attempt = 0;; ++attempt) {
        edges_raw = buf<unsigned long long>(ctx, "pores.edges_raw", ecap);
        PMA_CUDA(cudaMemsetAsync(ecount, 0, 8, s));
        {
            KernelTimer kt(ctx, "edges_write");
            plateau_edges<<<G, 256, 0, s>>>(pid, crad2, g, d3q7, sb, ecount, edges_raw, ecap);
        }
        ctx->check_launch("plateau_edges");
        PMA_CUDA(cudaMemcpyAsync(&ne_kept, ecount, 8, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        if (ne_kept <= ecap) break;
        PMA_REQUIRE(attempt < 3, PMA_ERR_INTERNAL, "pma_pores: plateau edge count did not settle");
        ecap = ne_kept + ne_kept / 8 + 1024;
    }
    // Keys are (destination << sb | source): sorting groups the predecessors of each plateau.
    int64_t ne = 0;
    if (ne_kept) {
        auto* edges = buf<unsigned long long>(ctx, "pores.edges", ne_kept);
        sort_keys(ctx, edges_raw, edges, static_cast<int64_t>(ne_kept), 2 * sb);  // used bits only
        ne = unique(ctx, edges, edges_raw, static_cast<int64_t>(ne_kept), d_count);
    }
    ctx->count("pores.plateaus", static_cast<double>(np));
    ctx->count("pores.plateau_edges", static_cast<double>(ne));
    ctx->count("pores.plateau_edges_written", static_cast<double>(ne_kept));
    uint32_t* by_dst = buf<uint32_t>(ctx, "pores.esrc", std::max<int64_t>(ne, 1));
    unsigned int* eoff = buf<unsigned int>(ctx, "pores.eoff", np + 1);
    PMA_CUDA(cudaMemsetAsync(eoff, 0, (np + 1) * 4, s));
    edge_offsets<<<grid_for(ctx, ne + 1), 256, 0, s>>>(edges_raw, ne, np, sb, eoff, by_dst);
    ctx->check_launch("edge_offsets");
    kt_edges.reset();

    auto kt_join = std::make_unique<KernelTimer>(ctx, "pores_sort_wait");
    sorter.t.join();
    kt_join.reset();
    auto kt_stats = std::make_unique<KernelTimer>(ctx, "plateau_stats");
    uint32_t* crank = buf<uint32_t>(ctx, "pores.crank", n);
    fill_u32<<<G, 256, 0, s>>>(crank, n, kNone);
    ctx->check_launch("fill_u32");
    if (nb) {
        copy_from_host(ctx, balls, voxel_of_rank, nb * 4);
        scatter_rank<<<grid_for(ctx, nb), 256, 0, s>>>(balls, nb, crank);
        ctx->check_launch("scatter_rank");
    }
    uint32_t* pcrad = buf<uint32_t>(ctx, "pores.pcrad", np);
    unsigned int* psize = buf<unsigned int>(ctx, "pores.psize", np);
    unsigned int* pface = buf<unsigned int>(ctx, "pores.pface", np);
    uint32_t* pminrank = buf<uint32_t>(ctx, "pores.pminrank", np);
    PMA_CUDA(cudaMemsetAsync(psize, 0, std::max<int64_t>(np, 1) * 4, s));
    PMA_CUDA(cudaMemsetAsync(pface, 0, std::max<int64_t>(np, 1) * 4, s));
    fill_u32<<<grid_for(ctx, np), 256, 0, s>>>(pminrank, np, kNone);
    ctx->check_launch("fill_u32");
    plateau_stats<<<G, 256, 0, s>>>(pid, crad2, crank, g, n, pcrad, psize, pface, pminrank);
    ctx->check_launch("plateau_stats");
    kt_stats.reset();

    // Levels: plateaus in decreasing crad.
    uint32_t* lkey = buf<uint32_t>(ctx, "pores.lkey", np);
    uint32_t* lval = buf<uint32_t>(ctx, "pores.lval", np);
    uint32_t* lkey2 = buf<uint32_t>(ctx, "pores.lkey2", np);
    uint32_t* order = buf<uint32_t>(ctx, "pores.order", np);
    std::vector<size_t> level_begin;
    if (np) {
        KernelTimer kt(ctx, "level_order");
        level_keys<<<grid_for(ctx, np), 256, 0, s>>>(pcrad, np, lkey, lval);
        ctx->check_launch("level_keys");
        sort_pairs(ctx, lkey, lkey2, lval, order, np);
        // first position of each level, found on the device (a few hundred of np positions)
        level_starts<<<grid_for(ctx, np), 256, 0, s>>>(lkey2, np, flags);
        ctx->check_launch("level_starts");
        const int64_t nl = select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), flags, lval, np, d_count);
        std::vector<uint32_t> starts(nl);
        if (nl) PMA_CUDA(cudaMemcpyAsync(starts.data(), lval, nl * 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        for (int64_t i = 0; i < nl; ++i) level_begin.push_back(static_cast<size_t>(starts[i]));
    }
    level_begin.push_back(static_cast<size_t>(np));

    // Level sweep.
    size_t max_level = 1;
    for (size_t l = 0; l + 1 < level_begin.size(); ++l)
        max_level = std::max(max_level, level_begin[l + 1] - level_begin[l]);
    PlateauSets ps;
    ps.eoff = eoff;
    ps.edges = by_dst;
    ps.order = order;
    ps.minrank = pminrank;
    ps.m = buf<uint32_t>(ctx, "pores.m", np);
    ps.seed = buf<uint32_t>(ctx, "pores.seed", np);
    ps.soff = buf<unsigned long long>(ctx, "pores.soff", np);
    ps.slen = buf<uint32_t>(ctx, "pores.slen", np);
    ps.err = err;
    ps.cnt = buf<unsigned long long>(ctx, "pores.cnt", max_level);
    ps.off = buf<unsigned long long>(ctx, "pores.off", max_level);
    ps.first = buf<unsigned long long>(ctx, "pores.first", max_level);
    ps.big = buf<uint8_t>(ctx, "pores.big", max_level);
    ps.heavy = buf<uint32_t>(ctx, "pores.heavy", max_level);
    ps.big_list = buf<uint32_t>(ctx, "pores.big_list", max_level);
    ps.info = buf<unsigned long long>(ctx, "pores.info", 5);
    ps.mtoff = buf<unsigned long long>(ctx, "pores.mtoff", max_level);
    // medium unions of one level: a buffer of its own (a full buffer sends the rest to the sort path)
    ps.mtmp_cap = std::min<unsigned long long>(std::max<unsigned long long>(1ull << 22, 16ull * np), 1ull << 27);
    ps.mtmp = buf<uint32_t>(ctx, "pores.mtmp", ps.mtmp_cap);
    unsigned long long* base = reinterpret_cast<unsigned long long*>(d_count + 3);
    auto* h_info = static_cast<unsigned long long*>(ctx->host_staging(32));
    unsigned long long pool_cap = std::max<unsigned long long>(1ull << 22, 32ull * np);
    int rank_bits = 1;  // bits of a ball rank
    while (rank_bits < 32 && (1ull << rank_bits) < static_cast<unsigned long long>(nb)) ++rank_bits;
    const unsigned heavy_grid = static_cast<unsigned>(ctx->num_sms * 2);
    for (int attempt = 0; attempt < 3; ++attempt) {
        ps.pool = buf<uint32_t>(ctx, "pores.pool", pool_cap);
        ps.pool_cap = pool_cap;
        PMA_CUDA(cudaMemsetAsync(base, 0, 8, s));
        PMA_CUDA(cudaMemsetAsync(err, 0, 4, s));
        KernelTimer kt(ctx, "level_sets");
        // per size class of the levels (plateaus in the level, log2), when timing is on
        static const char* const kLevelClass[32] = {"levels.plateaus_2^0", "levels.plateaus_2^1", "levels.plateaus_2^2", "levels.plateaus_2^3", "levels.plateaus_2^4", "levels.plateaus_2^5", "levels.plateaus_2^6", "levels.plateaus_2^7", "levels.plateaus_2^8", "levels.plateaus_2^9", "levels.plateaus_2^10", "levels.plateaus_2^11", "levels.plateaus_2^12", "levels.plateaus_2^13", "levels.plateaus_2^14", "levels.plateaus_2^15", "levels.plateaus_2^16", "levels.plateaus_2^17", "levels.plateaus_2^18", "levels.plateaus_2^19", "levels.plateaus_2^20", "levels.plateaus_2^21", "levels.plateaus_2^22", "levels.plateaus_2^23", "levels.plateaus_2^24", "levels.plateaus_2^25", "levels.plateaus_2^26", "levels.plateaus_2^27", "levels.plateaus_2^28", "levels.plateaus_2^29", "levels.plateaus_2^30", "levels.plateaus_2^31"};
        for (size_t l = 0; l + 1 < level_begin.size(); ++l) {
            const size_t b = level_begin[l], e = level_begin[l + 1];
            int lclass = 0;
            while (lclass < 31 && (2ull << lclass) <= e - b) ++lclass;
            KernelTimer kt_level(ctx, kLevelClass[lclass]);
            if (ctx->timing) ctx->count(std::string(kLevelClass[lclass]) + ".count", 1);
            const unsigned lg = grid_for(ctx, (e - b) * 32, kLevelWarps * 32);
            PMA_CUDA(cudaMemsetAsync(ps.info, 0, 40, s));
            {
                KernelTimer kt2(ctx, "level_seeds");
                // slabs small enough for every warp of the launch to get some of mtmp, and
                // at least a medium union's largest size
                const unsigned slab = static_cast<unsigned>(std::min<unsigned long long>(
                    kMedSlab, std::max<unsigned long long>(kMedCap, ps.mtmp_cap / (1ull * lg * kLevelWarps))));
                level_seeds<<<lg, kLevelWarps * 32, 0, s>>>(ps, b, e, slab);
                level_heavy<<<heavy_grid, 512, 0, s>>>(ps, b);
                ctx->count_launch(2);
            }
            {
                ReadBack rb;
                rb.add(h_info, ps.info, 32);
                read_back(ctx, rb);
            }
            const unsigned long long nbig = h_info[1], total = h_info[2];
            ctx->count("pores.levels", 1);
            if (nbig) {
                ctx->count("pores.big_sets", static_cast<double>(nbig));
                ctx->count("pores.big_set_elements_expanded", static_cast<double>(total));
            }
            if (h_info[0]) ctx->count("pores.heavy_plateaus", static_cast<double>(h_info[0]));
            int64_t merged = 0;
            int shift = 32;
            void* keys = nullptr;
            bool narrow = false;
            const unsigned long long* merged_dev = nullptr;  // merged count left on the device
            if (nbig && total <= static_cast<unsigned long long>(kSmallMerge)) {
                KernelTimer kt2(ctx, "level_merge");
                auto* k64 = buf<unsigned long long>(ctx, "pores.lkeys", kSmallMerge);
                merged_dev = ps.info + 3;
                level_merge_small<<<1, 1024, 0, s>>>(ps, b, k64, ps.info + 3);
                ctx->check_launch("level_merge_small");
                keys = k64;
                merged = kSmallMerge;  // upper bound for the copy launch below
            } else if (nbig) {
                KernelTimer kt2(ctx, "level_merge");
                PMA_REQUIRE(total < (1ull << 40), PMA_ERR_MEMORY, "pma_pores: seed-set union too large");
                int big_bits = 0;
                while ((1ull << big_bits) < nbig) ++big_bits;
                narrow = rank_bits < 32 && rank_bits + big_bits <= 32;
                auto read_emitted = [&]() {
                    ReadBack rb;
                    rb.add(h_info, ps.info, 32);
                    read_back(ctx, rb);
                    return static_cast<int64_t>(std::min<unsigned long long>(h_info[3], total));
                };
                auto* deg = buf<unsigned long long>(ctx, "pores.bdeg", nbig);
                auto* doff = buf<unsigned long long>(ctx, "pores.bdoff", nbig);
                level_big_degrees<<<grid_for(ctx, nbig), 256, 0, s>>>(ps, b, deg);
                ctx->check_launch("level_big_degrees");
                exclusive_sum(ctx, deg, doff, static_cast<int64_t>(nbig));
                const unsigned eg = static_cast<unsigned>(ctx->num_sms * 16);
                if (narrow) {
                    shift = rank_bits;
                    auto* k32 = buf<uint32_t>(ctx, "pores.lkeys32", total);
                    auto* k32b = buf<uint32_t>(ctx, "pores.lkeys32b", total);
                    int64_t emitted = 0;
                    {
                        KernelTimer kt3(ctx, "merge_expand");
                        level_expand<uint32_t><<<eg, 256, 0, s>>>(ps, b, doff, deg, nbig, k32, total, shift);
                        ctx->check_launch("level_expand");
                        emitted = read_emitted();
                    }
                    {
                        KernelTimer kt3(ctx, "merge_sort");
                        sort_keys(ctx, k32, k32b, emitted, rank_bits + big_bits);
                        merged = unique(ctx, k32b, k32, emitted, d_count);
                    }
                    keys = k32;
                    if (merged) {
                        level_runs<uint32_t><<<grid_for(ctx, merged), 256, 0, s>>>(k32, merged, ps, shift);
                        ctx->check_launch("level_runs");
                    }
                } else {
                    shift = rank_bits;
                    auto* k64 = buf<unsigned long long>(ctx, "pores.lkeys", total);
                    auto* k64b = buf<unsigned long long>(ctx, "pores.lkeys2", total);
                    int64_t emitted = 0;
                    {
                        KernelTimer kt3(ctx, "merge_expand");
                        level_expand<unsigned long long><<<eg, 256, 0, s>>>(ps, b, doff, deg, nbig, k64, total, shift);
                        ctx->check_launch("level_expand");
                        emitted = read_emitted();
                    }
                    const int bits = rank_bits + big_bits;  // radix passes over the used bits only
                    {
                        KernelTimer kt3(ctx, "merge_sort");
                        sort_keys(ctx, k64, k64b, emitted, bits);
                        merged = unique(ctx, k64b, k64, emitted, d_count);
                    }
                    keys = k64;
                    if (merged) {
                        level_runs<unsigned long long><<<grid_for(ctx, merged), 256, 0, s>>>(k64, merged, ps, shift);
                        ctx->check_launch("level_runs");
                    }
                }
            }
            if (merged && !merged_dev) ctx->count("pores.big_set_elements_merged", static_cast<double>(merged));
            KernelTimer kt3(ctx, "level_write");
            exclusive_sum(ctx, ps.cnt, ps.off, static_cast<int64_t>(e - b));
            level_write<<<lg, kLevelWarps * 32, 0, s>>>(ps, b, e, base);
            ctx->count_launch(1);
            if (merged) {
                if (narrow)
                    level_copy_big<uint32_t><<<grid_for(ctx, merged), 256, 0, s>>>(
                        static_cast<uint32_t*>(keys), merged, ps, base, shift, nullptr);
                else
                    level_copy_big<unsigned long long><<<grid_for(ctx, merged), 256, 0, s>>>(
                        static_cast<unsigned long long*>(keys), merged, ps, base, shift, merged_dev);
                ctx->count_launch(1);
            }
            level_advance<<<1, 32, 0, s>>>(base, ps.off, ps.cnt, e - b);
            ctx->count_launch(1);
        }
        ctx->check_launch("level_sets");
        unsigned int h_err = 0;
        unsigned long long used = 0;
        PMA_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(&used, base, 8, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        PMA_REQUIRE(!(h_err & 32u), PMA_ERR_INTERNAL, "pma_pores: merged seed sets disagree with their bounds");
        if (!(h_err & 2u)) break;
        PMA_REQUIRE(attempt < 2, PMA_ERR_MEMORY, "pma_pores: seed-set pool overflow");
        pool_cap = used + (used >> 2) + 1024;
    }

    // Seeds -> pores in rank order.
    KernelTimer kt_tables(ctx, "pores_tables");
    auto kt_seeds = std::make_unique<KernelTimer>(ctx, "tables_seeds");
    // the seeds' ball ranks, compacted on the device (a few thousand of up to 10^8 plateaus)
    std::vector<uint32_t> seed_ranks;
    if (np) {
        flag_seeds<<<grid_for(ctx, np), 256, 0, s>>>(ps.seed, np, flags);
        ctx->check_launch("flag_seeds");
        uint32_t* d_seeds = buf<uint32_t>(ctx, "pores.seed_ranks", np);
        const int64_t ns = select_flagged(ctx, ps.seed, flags, d_seeds, np, d_count);
        seed_ranks.resize(ns);
        if (ns) PMA_CUDA(cudaMemcpyAsync(seed_ranks.data(), d_seeds, ns * 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
    }
    std::sort(seed_ranks.begin(), seed_ranks.end());
    const size_t npores = seed_ranks.size();
    const std::vector<uint32_t> ids = pore_id_sequence(npores);
    // rank -> pore index and rank -> pore id tables on the device
    const size_t nrank = std::max<int64_t>(nb, 1);
    uint32_t* d_rank2pore = buf<uint32_t>(ctx, "pores.rank2pore", nrank);
    uint32_t* d_rank2id = buf<uint32_t>(ctx, "pores.rank2id", nrank);
    fill_u32<<<grid_for(ctx, nrank), 256, 0, s>>>(d_rank2pore, nrank, kNone);
    ctx->check_launch("fill_u32");
    PMA_CUDA(cudaMemsetAsync(d_rank2id, 0, nrank * 4, s));
    if (npores) {
        std::vector<uint32_t> up(2 * npores);
        std::copy(seed_ranks.begin(), seed_ranks.end(), up.begin());
        std::copy(ids.begin(), ids.end(), up.begin() + npores);
        uint32_t* d_up = buf<uint32_t>(ctx, "pores.seed_up", up.size());
        PMA_CUDA(cudaMemcpyAsync(d_up, up.data(), up.size() * 4, cudaMemcpyHostToDevice, s));
        scatter_seed_ids<<<grid_for(ctx, npores), 256, 0, s>>>(d_up, npores, d_rank2pore, d_rank2id);
        ctx->check_launch("scatter_seed_ids");
    }
    PoreAcc pa;
    pa.rank2pore = d_rank2pore;
    pa.pvol = buf<unsigned long long>(ctx, "pores.pvol", npores);
    pa.pbound = buf<unsigned int>(ctx, "pores.pbound", npores);
    PMA_CUDA(cudaMemsetAsync(pa.pvol, 0, std::max<size_t>(npores, 1) * 8, s));
    PMA_CUDA(cudaMemsetAsync(pa.pbound, 0, std::max<size_t>(npores, 1) * 4, s));
    if (np) {
        pore_accumulate<<<grid_for(ctx, np), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, psize, pface, np, pa);
        ctx->check_launch("pore_accumulate");
    }

    kt_seeds.reset();
    // Throats: plateaus with two or more seeds, grouped by equal seed sets.
    auto kt_groups = std::make_unique<KernelTimer>(ctx, "tables_groups");
    if (np) {
        flag_multi<<<grid_for(ctx, np), 256, 0, s>>>(ps.slen, np, flags);
        ctx->check_launch("flag_multi");
    }
    uint32_t* multi = buf<uint32_t>(ctx, "pores.multi", np);
    const int64_t nm = np ? select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), flags, multi,
                                           np, d_count)
                          : 0;
    std::vector<uint32_t> group_tid_h;
    uint32_t* plateau_group = buf<uint32_t>(ctx, "pores.pgroup", np);
    uint32_t* group_tid = nullptr;
    pma_table* t = new pma_table;
    std::vector<unsigned long long> h_gvol, h_gfirst;
    std::vector<uint32_t> h_grep;
    std::vector<uint32_t> flat;                // pore ids of each group's list, concatenated
    std::vector<unsigned long long> roff(1, 0);  // list offsets into flat
    int64_t ngroups = 0;
    if (nm) {
        auto* h1 = buf<unsigned long long>(ctx, "pores.h1", nm);
        auto* h2 = buf<unsigned long long>(ctx, "pores.h2", nm);
        auto* ktmp = buf<unsigned long long>(ctx, "pores.ktmp", nm);
        uint32_t* v1 = buf<uint32_t>(ctx, "pores.v1", nm);
        uint32_t* v2 = buf<uint32_t>(ctx, "pores.v2", nm);
        // Group plateaus with equal seed sets: a radix sort by the first hash puts equal sets
        // side by side unless two different sets share it (about n^2 / 2^65 likely), which
        // group_starts flags; then stable sorts by the second hash and then the first put
        // equal (h1, h2) pairs side by side.
        uint32_t* gstart = buf<uint32_t>(ctx, "pores.gstart", nm);
        uint32_t* gid = buf<uint32_t>(ctx, "pores.gid", nm);
        throat_hashes<<<grid_for(ctx, nm), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, multi, nm, h1, h2);
        ctx->check_launch("throat_hashes");
        sort_pairs(ctx, h1, ktmp, multi, v2, nm);
        throat_hashes<<<grid_for(ctx, nm), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, v2, nm, h1, h2);
        ctx->check_launch("throat_hashes");
        group_starts<<<grid_for(ctx, nm), 256, 0, s>>>(v2, h1, h2, nm, ps.soff, ps.slen, ps.pool, gstart, err);
        ctx->check_launch("group_starts");
        {
            unsigned int h_err0 = 0;
            PMA_CUDA(cudaMemcpyAsync(&h_err0, err, 4, cudaMemcpyDeviceToHost, s));
            ctx->sync();
            if (h_err0 & 64u) {
                PMA_CUDA(cudaMemsetAsync(err, 0, 4, s));
                throat_hashes<<<grid_for(ctx, nm), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, multi, nm, h1, h2);
                ctx->check_launch("throat_hashes");
                sort_pairs(ctx, h2, ktmp, multi, v1, nm);
                throat_hashes<<<grid_for(ctx, nm), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, v1, nm, h1, h2);
                ctx->check_launch("throat_hashes");
                sort_pairs(ctx, h1, ktmp, v1, v2, nm);
                throat_hashes<<<grid_for(ctx, nm), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, v2, nm, h1, h2);
                ctx->check_launch("throat_hashes");
                group_starts<<<grid_for(ctx, nm), 256, 0, s>>>(v2, h1, h2, nm, ps.soff, ps.slen, ps.pool, gstart, err);
                ctx->check_launch("group_starts");
            }
        }
        exclusive_sum(ctx, gstart, gid, nm);
        uint32_t last_off = 0, last_start = 0;
        PMA_CUDA(cudaMemcpyAsync(&last_off, gid + nm - 1, 4, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(&last_start, gstart + nm - 1, 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        ngroups = static_cast<int64_t>(last_off) + last_start;
        to_group_index<<<grid_for(ctx, nm), 256, 0, s>>>(gid, gstart, nm, gstart);
        ctx->check_launch("to_group_index");
        GroupOut go;
        go.gvol = buf<unsigned long long>(ctx, "pores.gvol", ngroups);
        go.gfirst = buf<unsigned long long>(ctx, "pores.gfirst", ngroups);
        go.grep = buf<uint32_t>(ctx, "pores.grep", ngroups);
        go.group_of = nullptr;
        PMA_CUDA(cudaMemsetAsync(go.gvol, 0, ngroups * 8, s));
        PMA_CUDA(cudaMemsetAsync(go.gfirst, 0xFF, ngroups * 8, s));
        group_reduce<<<grid_for(ctx, nm), 256, 0, s>>>(v2, gstart, nm, psize, roots, go, plateau_group);
        ctx->check_launch("group_reduce");
        h_gvol.resize(ngroups);
        h_gfirst.resize(ngroups);
        h_grep.resize(ngroups);
        PMA_CUDA(cudaMemcpyAsync(h_gvol.data(), go.gvol, ngroups * 8, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(h_gfirst.data(), go.gfirst, ngroups * 8, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(h_grep.data(), go.grep, ngroups * 4, cudaMemcpyDeviceToHost, s));
        unsigned int h_err = 0;
        PMA_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        PMA_REQUIRE(!(h_err & 4u), PMA_ERR_INTERNAL, "pma_pores: seed-set hash collision");
        // Representative seed lists, gathered into one buffer.
        std::vector<uint32_t> rlen(ngroups);
        uint32_t* d_rep_len = buf<uint32_t>(ctx, "pores.rlen", ngroups);
        gather_u32<<<grid_for(ctx, ngroups), 256, 0, s>>>(ps.slen, go.grep, ngroups, d_rep_len);
        ctx->check_launch("gather_u32");
        PMA_CUDA(cudaMemcpyAsync(rlen.data(), d_rep_len, ngroups * 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        roff.assign(ngroups + 1, 0);
        for (int64_t gi = 0; gi < ngroups; ++gi) roff[gi + 1] = roff[gi] + rlen[gi];
        auto* d_roff = buf<unsigned long long>(ctx, "pores.roff", ngroups + 1);
        uint32_t* d_rlist = buf<uint32_t>(ctx, "pores.rlist", roff[ngroups]);
        PMA_CUDA(cudaMemcpyAsync(d_roff, roff.data(), (ngroups + 1) * 8, cudaMemcpyHostToDevice, s));
        gather_lists<<<grid_for(ctx, ngroups), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, go.grep, d_roff,
                                                            ngroups, d_rank2id, d_rlist);
        ctx->check_launch("gather_lists");
        flat.resize(roff[ngroups]);
        PMA_CUDA(cudaMemcpyAsync(flat.data(), d_rlist, flat.size() * 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
    }
    kt_groups.reset();
    auto kt_host = std::make_unique<KernelTimer>(ctx, "tables_ids");
    // Throat ids: order by (last pore of the type, first voxel), counting down from
    // UINT32_MAX - 1 (BasePoreAndThroatComputer.cpp:122-130).
    // key = (last pore id << 32) | first voxel; both fit 32 bits and first voxels are distinct
    std::vector<std::pair<unsigned long long, int64_t>> gkey(ngroups);
    for (int64_t i = 0; i < ngroups; ++i)
        gkey[i] = {(static_cast<unsigned long long>(flat[roff[i + 1] - 1]) << 32) | (h_gfirst[i] & 0xFFFFFFFFull), i};
    std::sort(gkey.begin(), gkey.end());
    std::vector<int64_t> gorder(ngroups);
    for (int64_t k = 0; k < ngroups; ++k) gorder[k] = gkey[k].second;
    group_tid_h.assign(std::max<int64_t>(ngroups, 1), 0);
    for (int64_t k = 0; k < ngroups; ++k) group_tid_h[gorder[k]] = 0xFFFFFFFFu - 1u - static_cast<uint32_t>(k);
    group_tid = buf<uint32_t>(ctx, "pores.gtid", group_tid_h.size());
    PMA_CUDA(cudaMemcpyAsync(group_tid, group_tid_h.data(), group_tid_h.size() * 4, cudaMemcpyHostToDevice, s));

    kt_host.reset();
    auto kt_labels = std::make_unique<KernelTimer>(ctx, "tables_labels");
    // Labels.
    uint32_t* plabel = buf<uint32_t>(ctx, "pores.plabel", np);
    if (np) {
        plateau_labels<<<grid_for(ctx, np), 256, 0, s>>>(ps.soff, ps.slen, ps.pool, d_rank2id, plateau_group,
                                                         group_tid, np, plabel);
        ctx->check_launch("plateau_labels");
    }
    voxel_labels<<<G, 256, 0, s>>>(pid, plabel, n, labels);
    ctx->check_launch("voxel_labels");

    kt_labels.reset();
    KernelTimer kt_rows(ctx, "tables_rows");
    // Table (pores in id order, throats in id order).
    std::vector<unsigned long long> pvol(npores);
    std::vector<unsigned int> pbound(npores);
    if (npores) {
        PMA_CUDA(cudaMemcpyAsync(pvol.data(), pa.pvol, npores * 8, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(pbound.data(), pa.pbound, npores * 4, cudaMemcpyDeviceToHost, s));
    }
    ctx->sync();
    for (size_t k = 0; k < npores; ++k) {
        const uint32_t r = seed_ranks[k];
        int x, y, z;
        g.coords(voxel_of_rank[r], x, y, z);
        pma_pore p;
        std::memset(&p, 0, sizeof(p));
        p.id = ids[k];
        p.seed_x = x;
        p.seed_y = y;
        p.seed_z = z;
        p.seed_r2 = static_cast<uint32_t>(items[r] >> 32);
        p.is_boundary = pbound[k] ? 1 : 0;
        p.volume = pvol[k];
        t->pores.push_back(p);
    }
    // Throat rows: pore list in processing order [second, first, third, ...]
    // (BasePoreAndThroatComputer.cpp:338-340, 370-371), sorted by id.
    t->throats.resize(ngroups);
    t->pool.resize(roff[ngroups]);
    size_t at = 0;
    for (int64_t k = 0; k < ngroups; ++k) {
        const int64_t gi = gorder[ngroups - 1 - k];
        pma_throat& th = t->throats[k];
        th.id = group_tid_h[gi];
        th.volume = h_gvol[gi];
        th.pool_offset = at;
        const uint32_t* L = flat.data() + roff[gi];
        const size_t nl = roff[gi + 1] - roff[gi];
        th.n_pores = static_cast<uint32_t>(nl);
        t->pool[at++] = L[1];
        t->pool[at++] = L[0];
        for (size_t j = 2; j < nl; ++j) t->pool[at++] = L[j];
    }
    if (ctx->reference_throat_ids && ngroups) {
        KernelTimer kt_exact(ctx, "exact_type_ids");
        reference_type_ids(ctx, t, labels, crad2, d, st);
    }
    return t;
}

// Renumbers the shared types of the initial propagation in the reference's creation order
// (exact_ids.cpp) and relabels their voxels.
void reference_type_ids(pma_ctx* ctx, pma_table* t, uint32_t* labels, const uint32_t* crad2, pma_dims d,
                        pma_stencil st) {
    cudaStream_t s = ctx->stream;
    const size_t n = voxels(d);
    const size_t ng = t->throats.size();
    std::vector<uint32_t> h_labels(n), h_crad(n);
    PMA_CUDA(cudaMemcpyAsync(h_labels.data(), labels, n * 4, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(h_crad.data(), crad2, n * 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    std::vector<std::vector<uint32_t>> lists(ng);
    std::vector<uint32_t> fast(ng);
    for (size_t g = 0; g < ng; ++g) {
        const pma_throat& th = t->throats[g];
        lists[g].assign(t->pool.begin() + th.pool_offset, t->pool.begin() + th.pool_offset + th.n_pores);
        std::sort(lists[g].begin(), lists[g].end());
        fast[g] = th.id;
    }
    const std::vector<uint32_t> exact =
        replay_type_ids(h_crad.data(), h_labels.data(), d, st == PMA_D3Q7, t->pores, lists, fast);
    // voxels: old id -> new id (old ids ascending, as the rows are)
    std::vector<uint32_t> old_ids(ng), new_ids(ng);
    for (size_t g = 0; g < ng; ++g) {
        old_ids[g] = fast[g];
        new_ids[g] = exact[g];
    }
    PMA_REQUIRE(std::is_sorted(old_ids.begin(), old_ids.end()), PMA_ERR_INTERNAL, "pma_pores: type rows out of order");
    uint32_t* d_old = buf<uint32_t>(ctx, "pores.exact_old", ng);
    uint32_t* d_new = buf<uint32_t>(ctx, "pores.exact_new", ng);
    PMA_CUDA(cudaMemcpyAsync(d_old, old_ids.data(), ng * 4, cudaMemcpyHostToDevice, s));
    PMA_CUDA(cudaMemcpyAsync(d_new, new_ids.data(), ng * 4, cudaMemcpyHostToDevice, s));
    remap_labels<<<grid_for(ctx, n), 256, 0, s>>>(labels, n, d_old, d_new, static_cast<uint32_t>(ng));
    ctx->check_launch("remap_labels");
    // rows in ascending (new) id order
    std::vector<size_t> order(ng);
    for (size_t g = 0; g < ng; ++g) order[g] = g;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return exact[a] < exact[b]; });
    std::vector<pma_throat> rows;
    std::vector<uint32_t> pool;
    rows.reserve(ng);
    pool.reserve(t->pool.size());
    for (size_t k = 0; k < ng; ++k) {
        pma_throat th = t->throats[order[k]];
        const uint64_t off = th.pool_offset;
        th.id = exact[order[k]];
        th.pool_offset = pool.size();
        pool.insert(pool.end(), t->pool.begin() + off, t->pool.begin() + off + th.n_pores);
        rows.push_back(th);
    }
    t->throats.swap(rows);
    t->pool.swap(pool);
    ctx->sync();
}

// a11: EmptyPoresRemover.cpp:31-244 on the host table, then one relabel launch.
void remove_empty_pores(pma_ctx* ctx, pma_table* t, uint32_t* labels, pma_dims d) {
    KernelTimer kt_stage(ctx, "stage_removal");
    check_dims(d);
    PMA_REQUIRE(labels, PMA_ERR_ARGUMENT, "pma_remove_empty_pores: null labels");
    auto kt_host = std::make_unique<KernelTimer>(ctx, "removal_tables");
    auto mark = std::chrono::steady_clock::now();
    auto phase = [&](const char* name) {  // host time of each part, with the timing report
        const auto now = std::chrono::steady_clock::now();
        ctx->count(name, std::chrono::duration<double, std::milli>(now - mark).count());
        mark = now;
    };
    // EPR.cpp:193-244: drop zero-volume pores and remove them from the type lists.
    std::vector<uint32_t> empty;
    std::vector<pma_pore> kept;
    for (const pma_pore& p : t->pores) {
        if (p.volume == 0) empty.push_back(p.id);
        else kept.push_back(p);
    }
    std::sort(empty.begin(), empty.end());
    // empty pores by id (pore ids are below every type id and dense enough for a flag array)
    uint32_t max_pore = 0;
    for (const pma_pore& p : t->pores) max_pore = std::max(max_pore, p.id);
    std::vector<uint8_t> is_empty(static_cast<size_t>(max_pore) + 1, 0);
    for (uint32_t id : empty) is_empty[id] = 1;
    // Types in ascending id order with sorted, filtered pore lists (flat arrays).
    const size_t nt = t->throats.size();
    std::vector<uint32_t> by_id(nt);
    for (size_t i = 0; i < nt; ++i) by_id[i] = static_cast<uint32_t>(i);
    auto id_less = [&](uint32_t a, uint32_t b) { return t->throats[a].id < t->throats[b].id; };
    if (!std::is_sorted(by_id.begin(), by_id.end(), id_less)) std::sort(by_id.begin(), by_id.end(), id_less);
    // On host threads when there are many types: a count pass, then the lists written in place.
    std::vector<uint32_t> lists;
    std::vector<size_t> loff(nt + 1, 0);
    auto filter = [&](size_t lo, size_t hi, bool write) {
        std::vector<uint32_t> tmp;
        for (size_t k = lo; k < hi; ++k) {
            const pma_throat& th = t->throats[by_id[k]];
            tmp.assign(t->pool.begin() + th.pool_offset, t->pool.begin() + th.pool_offset + th.n_pores);
            if (!std::is_sorted(tmp.begin(), tmp.end())) std::sort(tmp.begin(), tmp.end());
            size_t at = write ? loff[k] : 0;
            for (uint32_t pid : tmp)
                if (pid > max_pore || !is_empty[pid]) {
                    if (write) lists[at] = pid;
                    ++at;
                }
            if (!write) loff[k + 1] = at;
        }
    };
    const unsigned nth = nt >= (1u << 15) ? std::max(1u, std::min(8u, std::thread::hardware_concurrency())) : 1u;
    auto parallel = [&](bool write) {
        std::vector<std::thread> ts;
        for (unsigned i = 1; i < nth; ++i) {
            try {
                ts.emplace_back(filter, nt * i / nth, nt * (i + 1) / nth, write);
            } catch (const std::system_error&) {
                filter(nt * i / nth, nt * (i + 1) / nth, write);  // no thread to be had: in line
            }
        }
        filter(0, nt / nth, write);
        for (auto& th : ts) th.join();
    };
    parallel(false);  // loff[k + 1] = kept length of type k
    for (size_t k = 0; k < nt; ++k) loff[k + 1] += loff[k];
    lists.resize(loff[nt]);
    parallel(true);
    auto len = [&](size_t k) { return loff[k + 1] - loff[k]; };
    phase("removal.filter_ms");
    ctx->count("removal.types", static_cast<double>(nt));
    std::vector<char> alive(nt, 1);
    std::vector<std::pair<uint32_t, uint32_t>> remap;  // (old id, new id)
    // EPR.cpp:167-191: types with fewer than two pores.
    for (size_t k = 0; k < nt; ++k)
        if (len(k) < 2) {
            if (len(k) == 1) remap.emplace_back(t->throats[by_id[k]].id, lists[loff[k]]);
            alive[k] = 0;
        }
    // EPR.cpp:126-165: merge types with equal pore lists into the largest id. Lists are put
    // side by side through a hash of their contents and grouped by comparing them element by
    // element within a hash (the groups, not their order, decide the result).
    auto same_list = [&](uint32_t a, uint32_t b) {
        return len(a) == len(b) && std::equal(lists.begin() + loff[a], lists.begin() + loff[a + 1],
                                              lists.begin() + loff[b]);
    };
    std::vector<unsigned long long> lhash(nt);  // hashes of the lists, on the filter's threads
    auto hash_range = [&](size_t lo, size_t hi) {
        for (size_t k = lo; k < hi; ++k) {
            unsigned long long h = 1469598103934665603ull ^ len(k);
            for (size_t i = loff[k]; i < loff[k + 1]; ++i) h = (h ^ lists[i]) * 1099511628211ull;
            lhash[k] = h;
        }
    };
    {
        std::vector<std::thread> ts;
        for (unsigned i = 1; i < nth; ++i) {
            try {
                ts.emplace_back(hash_range, nt * i / nth, nt * (i + 1) / nth);
            } catch (const std::system_error&) {
                hash_range(nt * i / nth, nt * (i + 1) / nth);  // no thread to be had: in line
            }
        }
        hash_range(0, nt / nth);
        for (auto& th : ts) th.join();
    }
    std::vector<std::pair<unsigned long long, uint32_t>> live;  // (hash of the list, type)
    for (size_t k = 0; k < nt; ++k)
        if (alive[k]) live.emplace_back(lhash[k], static_cast<uint32_t>(k));
    std::sort(live.begin(), live.end());
    std::vector<uint32_t> members;
    for (size_t i = 0; i < live.size();) {
        size_t j = i + 1;
        while (j < live.size() && live[j].first == live[i].first) ++j;
        for (size_t a = i; a < j && j - i > 1; ++a) {  // equal hashes: exact groups among them
            if (!alive[live[a].second]) continue;
            members.assign(1, live[a].second);
            for (size_t b = a + 1; b < j; ++b)
                if (alive[live[b].second] && same_list(live[a].second, live[b].second))
                    members.push_back(live[b].second);
            if (members.size() < 2) continue;
            uint32_t keep = 0;
            for (uint32_t m : members) keep = std::max(keep, t->throats[by_id[m]].id);
            for (uint32_t m : members) {
                const uint32_t id = t->throats[by_id[m]].id;
                if (id != keep) {
                    alive[m] = 0;
                    remap.emplace_back(id, keep);
                }
            }
        }
        i = j;
    }
    phase("removal.merge_ms");
    std::vector<pma_throat> throats;
    std::vector<uint32_t> pool;
    for (size_t k = 0; k < nt; ++k) {
        if (!alive[k]) continue;
        pma_throat th;
        th.id = t->throats[by_id[k]].id;
        th.volume = t->throats[by_id[k]].volume;
        th.n_pores = static_cast<uint32_t>(len(k));
        th.pool_offset = pool.size();
        pool.insert(pool.end(), lists.begin() + loff[k], lists.begin() + loff[k + 1]);
        throats.push_back(th);
    }
    t->pores = kept;
    t->throats.swap(throats);
    t->pool.swap(pool);
    std::sort(remap.begin(), remap.end());
    phase("removal.rows_ms");
    kt_host.reset();
    if (remap.empty()) return;  // EPR.cpp:54-57
    std::vector<uint32_t> o, nw;
    for (auto& kv : remap) {
        o.push_back(kv.first);
        nw.push_back(kv.second);
    }  // ascending old ids: remap_labels searches them
    cudaStream_t s = ctx->stream;
    uint32_t* d_old = buf<uint32_t>(ctx, "remove.old", o.size());
    uint32_t* d_new = buf<uint32_t>(ctx, "remove.new", nw.size());
    PMA_CUDA(cudaMemcpyAsync(d_old, o.data(), o.size() * 4, cudaMemcpyHostToDevice, s));
    PMA_CUDA(cudaMemcpyAsync(d_new, nw.data(), nw.size() * 4, cudaMemcpyHostToDevice, s));
    const size_t n = voxels(d);
    remap_labels<<<grid_for(ctx, n), 256, 0, s>>>(labels, n, d_old, d_new, static_cast<uint32_t>(o.size()));
    ctx->check_launch("remap_labels");
    ctx->sync();
}

}  // namespace pma
