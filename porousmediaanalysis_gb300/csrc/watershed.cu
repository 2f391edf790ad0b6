// Watershed pore and throat labelling (WatershedComputer.cpp:30-219), bit-exact.
//
// The reference floods from all seeds with one FIFO queue per depth (containing radius
// squared), deepest first. A popped node of pore P visits its stencil neighbours in loop
// order; a void neighbour w with crad(w) <= depth is "touched": the first touch claims w
// for P and queues it at depth crad(w); later touches by other pores only extend w's
// shared type ([second, first, third, ...], BasePoreAndThroatComputer.cpp:37-110) and do
// not queue it. Queued nodes keep propagating their claimer's pore.
//
// Parallel replay. Within one depth the FIFO runs generation by generation: generation 0 is
// the queue content when the depth starts (seeds in pore-id order, then nodes queued while
// deeper levels ran, in queue order); generation k+1 is what generation k queues at the same
// depth, in push order. Every touch gets the time (generation, node position * 27 +
// neighbour index), which orders touches exactly as the sequential loop does. Per generation:
//   claim    - the smallest-time touch of each unclaimed voxel wins (atomicMin on time);
//   resolve  - the winner records the claim; a voxel of the same depth joins the next
//              generation, a shallower one is appended, time-stamped, to its depth's bucket,
//              which is sorted by time when that depth starts; in the same pass, touches by
//              pores other than the voxel's owner record, per voxel and pore, their first
//              touch time (extensions).
// Frontier sizes stay on the device; the next generation is compacted in event order (see
// ws_generations).
//
// Voxel state: one 64-bit word per voxel holds the claim state, which is the untouched mark,
// the smallest touch of the running generation (kTouched | event), or the claimer (pore
// index + 1). Claimed < touched < untouched numerically, so the claim phase's atomicMin keeps
// the smallest touch and never undoes a claim; a touched voxel is always claimed by the
// generation's resolve phase, so no touch outlives its generation. When the containing radii
// fit 16 bits (radius below 256 voxels) they ride in the word's low bits: a touch then costs one
// random load, and its atomic hits the same sector.
//
// Shared types: a voxel's key is its claimer plus its extending pores in time order; every
// prefix of length >= 2 was created at the time of its last extension. All prefixes are
// hashed, grouped with radix sorts and ranked by creation time on the device, which
// reproduces the reference's id sequence (UINT32_MAX - 1, - 2, ...) exactly, including
// types whose volume later dropped to zero. A voxel's extending pores are kept in a chain of
// fixed-size records, so a key may hold as many pores as the stencil lets touch one voxel
// (the reference keys types by an unbounded pore-id vector,
// BasePoreAndThroatComputer.cpp:112-133).
#include <cooperative_groups.h>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "devutil.cuh"

namespace pma {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kSlots = 6;         // extending pores per record; a voxel chains more records
constexpr int kMaxExt = 26;       // extending pores of one voxel at most (26 neighbours touch it)
constexpr int kMaxHops = (kMaxExt + kSlots - 1) / kSlots;  // records in one voxel's chain
constexpr int kKeyMax = kMaxExt + 1;  // longest key: the claimer and every extending pore
constexpr int kChunk = 1024;      // event slots per compaction block
constexpr int kGensPerLaunch = 64;  // generations per cooperative launch (host checks between)
constexpr unsigned long long kMaxGen = 1ull << 23;              // generations per call
constexpr unsigned long long kSeqMask = (1ull << 40) - 1;       // touch time within a generation
constexpr unsigned long long kUntouched = (1ull << 48) - 1;     // claim states (48-bit field)
constexpr unsigned long long kTouched = 1ull << 46;
constexpr uint32_t kRecBusy = 0xFFFFFFFFu;  // ext[w] while its record is being allocated

struct WsState {
    Grid g;
    int d3q7;
    const uint32_t* crad;
    unsigned long long* state;    // per voxel: claim state, << 16 | radius when packed
    int packed;                   // 1: radii below 2^16 are held in the state words
    uint32_t* ext;                // shared-voxel record + 1, 0 = none
    uint32_t* ext_pore;           // [records][kSlots]
    unsigned long long* ext_time;
    uint32_t* ext_next;           // [records]: the voxel's next record + 1, 0 = none
    unsigned int* ext_count;
    uint32_t ext_cap;
    unsigned int* pbound;         // per pore
    unsigned int* err;
    int spin_limit;               // polls of one wait on another block before giving up
    unsigned long long* gen_hist; // NULL, or per log2 of the frontier size: [c] generations,
                                  // [64 + c] ns in claim phases, [128 + c] ns in resolve phases;
                                  // [192], [193]: block 0's ns resolving events, scan + look-back
    int time_shift;               // bucket entry time = (generation << time_shift) | event
    uint8_t* ev_touch;            // per event slot: phase 0 touched an unclaimed voxel
    const unsigned long long* boff;  // bucket offsets
    unsigned int* bfill;
    unsigned long long* ent_time;
    unsigned long long* ent_val;
};

__host__ __device__ __forceinline__ unsigned long long ws_word(int packed, unsigned long long st, uint32_t r) {
    return packed ? (st << 16) | r : st;
}

// Claim state of a state word: the claimer (pore index + 1) or 0.
__device__ __forceinline__ uint32_t ws_claimer(int packed, unsigned long long word) {
    const unsigned long long st = packed ? word >> 16 : word;
    return st < kTouched ? static_cast<uint32_t>(st) : 0u;
}

// The radius and claim state of voxel w (one load when packed).
__device__ __forceinline__ void ws_load(const WsState& s, size_t w, uint32_t& r, unsigned long long& st) {
    const unsigned long long word = __ldcg(s.state + w);
    if (s.packed) {
        r = static_cast<uint32_t>(word & 0xFFFFu);
        st = word >> 16;
    } else {
        r = __ldg(s.crad + w);
        st = word;
    }
}

__global__ void ws_init(size_t n, const uint32_t* __restrict__ crad, int packed,
                        unsigned long long* __restrict__ state, uint32_t* __restrict__ ext) {
    PMA_GRID_STRIDE(v, n) {
        state[v] = ws_word(packed, kUntouched, packed ? crad[v] : 0u);
        ext[v] = 0;
    }
}

__global__ void ws_seed(const uint32_t* __restrict__ seed_voxel, size_t np, const uint32_t* __restrict__ crad,
                        int packed, unsigned long long* __restrict__ state) {
    PMA_GRID_STRIDE(k, np) {
        const uint32_t v = seed_voxel[k];
        state[v] = ws_word(packed, k + 1, packed ? crad[v] : 0u);
    }
}

__global__ void ws_seed_entries(const unsigned long long* __restrict__ a, size_t np,
                                unsigned long long* __restrict__ ent_time,
                                unsigned long long* __restrict__ ent_val) {
    PMA_GRID_STRIDE(k, np) {
        ent_time[a[k]] = a[np + k];
        ent_val[a[k]] = a[2 * np + k];
    }
}

// Voxel count per containing radius. Few distinct radii take most voxels, so counts gather
// in a shared-memory copy of the bins first when they fit (nb <= kHistShared).
constexpr uint32_t kHistShared = 8192;

__global__ void ws_histograms(const uint32_t* __restrict__ crad, size_t n, uint32_t nb,
                              unsigned int* __restrict__ hist) {
    __shared__ unsigned int local[kHistShared];
    const bool shared = nb <= kHistShared;
    if (shared)
        for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) local[i] = 0;
    __syncthreads();
    PMA_GRID_STRIDE(v, n) {
        const uint32_t r = crad[v];
        if (!r) continue;
        if (shared) atomicAdd(&local[r], 1u);
        else atomicAdd(&hist[r], 1u);
    }
    __syncthreads();
    if (shared)
        for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x)
            if (local[i]) atomicAdd(&hist[i], local[i]);
}

// The record a link (ext[w] or a record's next field) points to, allocated by the one touch
// that moves the link from 0 to kRecBusy; touches that meet kRecBusy wait (a few
// instructions) for the record number. Returns 0 when the records ran out (err bit 1: the
// flood is redone with more) or the wait gave up (err bit 8).
__device__ __forceinline__ uint32_t ws_follow(uint32_t* link, const WsState& s) {
    uint32_t rec = *reinterpret_cast<volatile uint32_t*>(link);
    if (rec == 0) {
        rec = atomicCAS(link, 0u, kRecBusy);
        if (rec == 0) {
            // the warp's allocating lanes take their record numbers with one atomic (a single
            // counter for every new shared voxel of the flood would serialise them)
            const unsigned peers = __activemask();
            const int leader = __ffs(peers) - 1;
            const unsigned lane = threadIdx.x & 31;
            unsigned first = 0;
            if (static_cast<int>(lane) == leader) first = atomicAdd(s.ext_count, static_cast<unsigned>(__popc(peers)));
            first = __shfl_sync(peers, first, leader);
            const uint32_t fresh = first + __popc(peers & ((1u << lane) - 1u)) + 1;
            if (fresh > s.ext_cap) {  // out of records: flag a redo with more
                atomicExch(link, 0u);
                atomicOr(s.err, 1u);
                return 0;
            }
            atomicExch(link, fresh);
            return fresh;
        }
    }
    for (int spins = 0; rec == kRecBusy; ++spins) {
        if (spins > s.spin_limit) {
            atomicOr(s.err, 8u);
            return 0;
        }
        rec = atomicAdd(link, 0u);
    }
    if (rec == 0) atomicOr(s.err, 1u);  // the allocating touch ran out of records
    return rec;
}

// Records that `pore` touched shared voxel w at time t (its first touch per pore is kept).
// Out of line: it is the rare path of the touch kernel. Slots fill in order along the
// voxel's record chain, so two touches by one pore meet at the same slot.
__device__ __noinline__ void ws_extend(const WsState& s, size_t w, uint32_t pore, unsigned long long t) {
    uint32_t rec = ws_follow(s.ext + w, s);
    for (int hop = 0; hop < kMaxHops && rec; ++hop) {
        for (int k = 0; k < kSlots; ++k) {
            const size_t slot = static_cast<size_t>(rec - 1) * kSlots + k;
            const uint32_t cur = atomicCAS(&s.ext_pore[slot], kNone, pore);
            if (cur == kNone || cur == pore) {
                atomicMin(&s.ext_time[slot], t);
                return;
            }
        }
        if (hop + 1 < kMaxHops) rec = ws_follow(s.ext_next + (rec - 1), s);
    }
    if (rec) atomicOr(s.err, 2u);  // more extending pores than neighbours: cannot happen
}

// Touch events of the generation's nodes. Phase 0 claims: the smallest touch time of each
// unclaimed voxel wins (atomicMin on its state word). A touch of a voxel claimed in an
// earlier generation is final in phase 0 already: it is an extension when the toucher is not the owner (claims
// never change, and extensions keep each pore's smallest time, so the order of recording
// does not matter). Phase 0 flags, per event, a touch of an unclaimed voxel; phase 1 resolves
// only those: the winner records its claim, and every other touch by a pore other than the
// winner's is an extension.
// One thread per event (node i, stencil position j): seq = i * 27 + j.
// All generations of a launch run in one kernel (see ws_generations), so data written by
// other blocks earlier in the launch is read with __ldcg (L2, not a possibly stale L1 line);
// only the radii, which never change, go through the read-only path.
__device__ __forceinline__ void ws_claim_event(const WsState& s, const uint32_t* gv, const uint32_t* gp,
                                               unsigned long long seq, uint32_t depth, unsigned long long gen) {
    const unsigned long long i = seq / 27;
    const int j = static_cast<int>(seq - i * 27);
    uint8_t touched = 0;
    int dx, dy, dz;
    if (stencil_offset(j, s.d3q7, dx, dy, dz)) {
        const uint32_t v = __ldcg(gv + i);
        const uint32_t pore = __ldcg(gp + i);
        int x, y, z;
        s.g.coords(v, x, y, z);
        const int nx = x + dx, ny = y + dy, nz = z + dz;
        if (!s.g.inside(nx, ny, nz)) {  // WC.cpp:140-144
            s.pbound[pore] = 1;
        } else {
            const size_t w = s.g.idx(nx, ny, nz);
            uint32_t r;
            unsigned long long st;
            ws_load(s, w, r, st);
            if (r != 0 && r <= depth) {  // WC.cpp:152-156
                if (st >= kTouched) {
                    atomicMin(&s.state[w], ws_word(s.packed, kTouched | seq, r));
                    touched = 1;
                } else if (st - 1 != pore) {
                    ws_extend(s, w, pore, (gen << 40) | seq);
                }
            }
        }
    }
    s.ev_touch[seq] = touched;
}

// Returns true when the event claims a voxel of the same depth (a node of the next
// generation: voxel nw of pore np_out).
__device__ __forceinline__ bool ws_resolve_event(const WsState& s, const uint32_t* gv, const uint32_t* gp,
                                                 unsigned long long seq, uint32_t depth, unsigned long long gen,
                                                 uint32_t& nw, uint32_t& np_out) {
    const unsigned long long i = seq / 27;
    const int j = static_cast<int>(seq - i * 27);
    // the node (shared by the event's warp neighbours) is loaded along with the flag
    const uint8_t touched = __ldcg(s.ev_touch + seq);
    const uint32_t v = __ldcg(gv + i);
    const uint32_t pore = __ldcg(gp + i);
    if (!touched) return false;
    int dx, dy, dz;
    stencil_offset(j, s.d3q7, dx, dy, dz);
    // the neighbour is inside the box (phase 0 touched it)
    const size_t w = static_cast<size_t>(static_cast<long long>(v) +
                                         (static_cast<long long>(dz) * s.g.SX + dx) * s.g.SY + dy);
    uint32_t r;
    unsigned long long st;
    ws_load(s, w, r, st);
    if (st == (kTouched | seq)) {
        s.state[w] = ws_word(s.packed, pore + 1, r);  // one 64-bit store: readers see either word
        if (r == depth) {
            nw = static_cast<uint32_t>(w);
            np_out = pore;
            return true;
        }
        // lanes of the warp appending to the same depth take their slots with one atomic: a
        // generation's claims of shallower voxels mostly go to a few depths, and one counter
        // per depth would serialise them
        const unsigned active = __activemask();
        const unsigned peers = __match_any_sync(active, r);
        const int leader = __ffs(peers) - 1;
        const unsigned lane = threadIdx.x & 31;
        unsigned first = 0;
        if (static_cast<int>(lane) == leader) first = atomicAdd(&s.bfill[r], static_cast<unsigned>(__popc(peers)));
        first = __shfl_sync(peers, first, leader);
        const unsigned pos = first + __popc(peers & ((1u << lane) - 1u));
        const unsigned long long at = s.boff[r] + pos;
        s.ent_time[at] = (gen << s.time_shift) | seq;
        s.ent_val[at] = (static_cast<unsigned long long>(pore) << 32) | w;
        return false;
    }
    // the winner's pore: already stored as the claimer, or that of the winning touch's node
    const uint32_t owner = st < kTouched ? static_cast<uint32_t>(st - 1) : __ldcg(gp + (st & kSeqMask) / 27);
    if (owner != pore) ws_extend(s, w, pore, (gen << 40) | seq);
    return false;
}

// Ordered compaction of a generation's same-depth claims into the next frontier, in event
// order, inside the resolve phase: each chunk of kChunk events (one block, four per thread)
// ranks its claims, and its offset comes from a decoupled look-back over the chunks before it,
// read 256 descriptors at a time by one warp. A descriptor holds (generation << 40) | state << 38
// | count, state 1 = the chunk's own count, 2 = the inclusive prefix; one of an older
// generation is not yet published. Chunks publish their own count before looking back and
// every block of the cooperative grid is resident, so the look-back always ends; it is bounded
// all the same (err bit 16). A generation thus needs two grid-wide barriers (after the claims,
// after the resolved frontier) instead of four for a separate count, scan and scatter.
// (Measured at 1024^3: 894 ms per step, against 910-950 ms with the count / scan / scatter
// form for generations of more than 256 chunks, and 1108 ms with a look-back that read one
// descriptor at a time.)
constexpr unsigned long long kDescOwn = 1ull << 38;
constexpr unsigned long long kDescIncl = 2ull << 38;
constexpr unsigned long long kDescVal = (1ull << 38) - 1;

// Called by all 32 lanes of one warp; returns the exclusive prefix of chunk c, reading 32
// descriptors a poll. Used where chunks are dealt round-robin: its light polling leaves the L2 to
// the blocks still resolving (a 256-wide poll made single-round generations 10-40 % slower).
__device__ unsigned long long ws_lookback32(unsigned long long* desc, unsigned long long c, unsigned long long gen,
                                          unsigned long long own, unsigned int* err, int spin_limit,
                                          unsigned lane) {
    volatile unsigned long long* vd = desc;
    const unsigned long long tg = gen << 40;
    if (lane == 0) vd[c] = tg | (c == 0 ? kDescIncl : kDescOwn) | own;
    if (c == 0) return 0;
    __threadfence();
    unsigned long long excl = 0;
    long long top = static_cast<long long>(c) - 1;
    int spins = 0;
    while (true) {
        const long long p = top - static_cast<long long>(lane);
        const bool valid = p >= 0;
        const unsigned long long d = valid ? vd[p] : 0ull;
        const bool ready = !valid || (d >> 40) == gen;
        if (!__all_sync(0xFFFFFFFFu, ready)) {  // a predecessor has not published yet
            if (++spins > spin_limit) {
                if (lane == 0) atomicOr(err, 16u);
                break;
            }
            continue;
        }
        // the nearest inclusive prefix ends the walk; owns before it are added
        const unsigned incl = __ballot_sync(0xFFFFFFFFu, valid && (d & kDescIncl) != 0);
        const int stop = incl ? __ffs(incl) - 1 : 31;
        unsigned long long v = (valid && static_cast<int>(lane) <= stop) ? (d & kDescVal) : 0ull;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        excl += v;
        if (incl || top < 32) break;  // chunk 0 is always inclusive
        top -= 32;
    }
    if (lane == 0) {
        __threadfence();
        vd[c] = tg | kDescIncl | (excl + own);
    }
    return excl;
}

// Called by all 32 lanes of one warp; returns the exclusive prefix of range c. Each poll reads
// kLookbackPer descriptors per lane (256 ranges, nearest first) and needs them published only
// up to the nearest inclusive prefix, so a range far from its last inclusive predecessor
// reaches it in a few polls instead of one per 32. Used once per block and generation by the
// contiguous-range compaction.
constexpr int kLookbackPer = 8;
__device__ unsigned long long ws_lookback(unsigned long long* desc, unsigned long long c, unsigned long long gen,
                                          unsigned long long own, unsigned int* err, int spin_limit,
                                          unsigned lane) {
    volatile unsigned long long* vd = desc;
    const unsigned long long tg = gen << 40;
    if (lane == 0) vd[c] = tg | (c == 0 ? kDescIncl : kDescOwn) | own;
    if (c == 0) return 0;
    __threadfence();
    unsigned long long excl = 0;
    long long top = static_cast<long long>(c) - 1;
    int spins = 0;
    while (true) {
        // lane l holds chunks top - l * kLookbackPer - j; before chunk 0 reads as an inclusive
        // zero (chunk 0 is always inclusive, so the walk stops there anyway)
        unsigned long long d[kLookbackPer];
#pragma unroll
        for (int j = 0; j < kLookbackPer; ++j) {
            const long long p = top - static_cast<long long>(lane) * kLookbackPer - j;
            d[j] = p >= 0 ? vd[p] : (tg | kDescIncl);
        }
        int fi = kLookbackPer, fn = kLookbackPer;  // this lane's first inclusive / first unpublished
#pragma unroll
        for (int j = kLookbackPer - 1; j >= 0; --j) {
            if ((d[j] >> 40) != gen) fn = j;
            else if (d[j] & kDescIncl) fi = j;
        }
        const unsigned incl = __ballot_sync(0xFFFFFFFFu, fi < fn);
        const unsigned gap = __ballot_sync(0xFFFFFFFFu, fn < fi);
        const unsigned any = incl | gap;
        const int stop = any ? __ffs(any) - 1 : 32;  // the lane that decides this poll
        if (stop < 32 && ((gap >> stop) & 1u)) {     // a predecessor before the inclusive is unpublished
            if (++spins > spin_limit) {
                if (lane == 0) atomicOr(err, 16u);
                break;
            }
            continue;
        }
        const int upto = static_cast<int>(lane) < stop ? kLookbackPer : (static_cast<int>(lane) == stop ? fi + 1 : 0);
        unsigned long long v = 0;
#pragma unroll
        for (int j = 0; j < kLookbackPer; ++j)
            if (j < upto) v += d[j] & kDescVal;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        excl += v;
        if (stop < 32) break;
        top -= 32 * kLookbackPer;
    }
    if (lane == 0) {
        __threadfence();
        vd[c] = tg | kDescIncl | (excl + own);
    }
    return excl;
}

// A look-back at a chunk descriptor that nothing publishes (chunk 0 of generation 0 while
// chunk 1 of generation 1 waits for it): each bounded wait of the frontier compaction (the
// 32-wide one in err[0], the 256-wide one in err[1]) runs out after spin_limit polls and sets
// bit 16, the path a stalled generation would take.
__global__ void ws_wait_selftest(unsigned long long* desc, unsigned int* err, int spin_limit) {
    ws_lookback32(desc, 1, 1, 0, err, spin_limit, threadIdx.x & 31);
    ws_lookback(desc, 1, 1, 0, err + 1, spin_limit, threadIdx.x & 31);
}

__device__ __forceinline__ unsigned long long ws_clock() {  // ns
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Up to max_gens generations of one depth in a single cooperative launch, two grid-wide
// barriers per generation. ng[2] holds the two frontier sizes; the frontier starts on side
// `cur`. out[0] = generations run, out[1] = the side holding the next frontier.
__global__ void __launch_bounds__(kChunk / 4, 4) ws_generations(WsState s, uint32_t* gv0, uint32_t* gp0, uint32_t* gv1,
                                                             uint32_t* gp1, unsigned int* ng,
                                                             unsigned long long* desc, uint32_t depth,
                                                             unsigned long long gen0, int max_gens, int cur,
                                                             unsigned long long* out) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ unsigned int part[33];
    const unsigned long long tid = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, lt = (1u << lane) - 1u;
    unsigned long long gen = gen0;
    int it = 0;
    for (; it < max_gens; ++it) {
        const unsigned long long nev = static_cast<unsigned long long>(__ldcg(ng + cur)) * 27;
        if (nev == 0) break;
        ++gen;
        const int hc = min(63, 63 - __clzll(nev / 27));
        unsigned long long t_start = 0;
        if (s.gen_hist && tid == 0) {
            atomicAdd(&s.gen_hist[hc], 1ull);
            t_start = ws_clock();
        }
        const uint32_t* gv = cur ? gv1 : gv0;
        const uint32_t* gp = cur ? gp1 : gp0;
        uint32_t* nv = cur ? gv0 : gv1;
        uint32_t* np_ = cur ? gp0 : gp1;
        for (unsigned long long seq = tid; seq < nev; seq += stride) ws_claim_event(s, gv, gp, seq, depth, gen);
        grid.sync();
        if (s.gen_hist && tid == 0) {
            const unsigned long long t = ws_clock();
            atomicAdd(&s.gen_hist[64 + hc], t - t_start);
            t_start = t;
        }
        const unsigned long long nchunks = (nev + kChunk - 1) / kChunk;
        if (nchunks > 8ull * gridDim.x) {
            // More than eight rounds of chunks: each block resolves one contiguous range of
            // events (each warp a contiguous part of it, 32 events a step) and counts its
            // same-depth claims, marking them in ev_touch; one look-back per block gives its
            // offset, and a second sweep over the range writes the marked claims in event order.
            // (Chunks dealt round-robin wait, round after round, for the slowest of their
            // predecessors in the previous round: at 1024^3, 720 against 837 us per generation
            // of 2^20 nodes; with fewer rounds the extra sweep costs more than it saves. Issuing
            // each thread's loads of several events together did not pay in either phase.)
            const bool probe = s.gen_hist && blockIdx.x == 0 && threadIdx.x == 0;
            const unsigned long long ta = probe ? ws_clock() : 0;
            const unsigned nwarp = blockDim.x >> 5;
            const unsigned long long steps = (nev + 31) / 32;
            const unsigned long long per_block = (steps + gridDim.x - 1) / gridDim.x;
            const unsigned long long used = (steps + per_block - 1) / per_block;  // blocks with events
            const unsigned long long per_warp = (per_block + nwarp - 1) / nwarp;
            const unsigned long long b0 = blockIdx.x * per_block;
            const unsigned long long b1 = min(b0 + per_block, steps);
            const unsigned long long w0 = min(b0 + warp * per_warp, b1);
            const unsigned long long w1 = min(w0 + per_warp, b1);
            if (blockIdx.x < used) {
                unsigned cnt = 0;
                for (unsigned long long st = w0; st < w1; ++st) {
                    const unsigned long long seq = st * 32 + lane;
                    uint32_t wv, wp;
                    const bool f = seq < nev && ws_resolve_event(s, gv, gp, seq, depth, gen, wv, wp);
                    if (f) s.ev_touch[seq] = 2;
                    cnt += __popc(__ballot_sync(0xFFFFFFFFu, f));
                }
                if (lane == 0) part[warp] = cnt;
                __syncthreads();
                const unsigned long long tb = probe ? ws_clock() : 0;
                if (warp == 0) {
                    const unsigned v = lane < nwarp ? part[lane] : 0u;
                    unsigned incl = v;
                    for (int o = 1; o < 32; o <<= 1) {
                        const unsigned t2 = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                        if (lane >= static_cast<unsigned>(o)) incl += t2;
                    }
                    const unsigned total = __shfl_sync(0xFFFFFFFFu, incl, 31);
                    if (lane < nwarp) part[lane] = incl - v;
                    const unsigned long long base = ws_lookback(desc, blockIdx.x, gen, total, s.err, s.spin_limit, lane);
                    if (lane == 0) {
                        part[32] = static_cast<unsigned int>(base);
                        if (blockIdx.x == used - 1) ng[cur ^ 1] = static_cast<unsigned int>(base + total);
                    }
                }
                __syncthreads();
                if (probe) {
                    const unsigned long long tc = ws_clock();
                    atomicAdd(&s.gen_hist[192], tb - ta);
                    atomicAdd(&s.gen_hist[193], tc - tb);
                }
                unsigned long long pos = static_cast<unsigned long long>(part[32]) + part[warp];
                // four steps at a time, every load issued before the stores
                for (unsigned long long st = w0; st < w1; st += 4) {
                    bool f[4];
                    uint32_t v[4], pr[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const unsigned long long seq = (st + k) * 32 + lane;
                        f[k] = st + k < w1 && seq < nev && __ldcg(s.ev_touch + seq) == 2;  // L2: no stale L1 line
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const unsigned long long i = ((st + k) * 32 + lane) / 27;
                        v[k] = f[k] ? __ldcg(gv + i) : 0u;
                        pr[k] = f[k] ? __ldcg(gp + i) : 0u;
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const unsigned m = __ballot_sync(0xFFFFFFFFu, f[k]);
                        if (f[k]) {
                            const unsigned long long seq = (st + k) * 32 + lane;
                            const int j = static_cast<int>(seq - seq / 27 * 27);
                            int dx, dy, dz;
                            stencil_offset(j, s.d3q7, dx, dy, dz);
                            const unsigned long long at = pos + __popc(m & lt);
                            nv[at] = static_cast<uint32_t>(static_cast<long long>(v[k]) +
                                                           (static_cast<long long>(dz) * s.g.SX + dx) * s.g.SY + dy);
                            np_[at] = pr[k];
                        }
                        pos += __popc(m);
                    }
                }
            }
        } else
        // Resolve by chunks of kChunk events: event k * blockDim + t of a chunk is thread t's
        // k-th, so event order is k-major, then thread.
        for (unsigned long long c = blockIdx.x; c < nchunks; c += gridDim.x) {
            const bool probe = s.gen_hist && blockIdx.x == 0 && threadIdx.x == 0;  // block 0's split
            const unsigned long long ta = probe ? ws_clock() : 0;
            bool f[4];
            uint32_t wv[4], wp[4];
            unsigned m[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned long long seq = c * kChunk + k * (kChunk / 4) + threadIdx.x;
                f[k] = seq < nev && ws_resolve_event(s, gv, gp, seq, depth, gen, wv[k], wp[k]);
                m[k] = __ballot_sync(0xFFFFFFFFu, f[k]);
                if (lane == 0) part[k * (kChunk / 128) + warp] = __popc(m[k]);
            }
            __syncthreads();
            const unsigned long long tb = probe ? ws_clock() : 0;
            if (warp == 0) {  // 4 rounds x 8 warps = 32 counts in event order
                const unsigned v = part[lane];
                unsigned incl = v;
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned t2 = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= static_cast<unsigned>(o)) incl += t2;
                }
                const unsigned total = __shfl_sync(0xFFFFFFFFu, incl, 31);
                part[lane] = incl - v;
                const unsigned long long base = ws_lookback32(desc, c, gen, total, s.err, s.spin_limit, lane);
                if (lane == 0) {
                    part[32] = static_cast<unsigned int>(base);
                    if (c == nchunks - 1) ng[cur ^ 1] = static_cast<unsigned int>(base + total);
                }
            }
            __syncthreads();
            if (probe) {
                const unsigned long long tc = ws_clock();
                atomicAdd(&s.gen_hist[192], tb - ta);  // events resolved
                atomicAdd(&s.gen_hist[193], tc - tb);  // scan and look-back
            }
            const unsigned base = part[32];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (f[k]) {
                    const unsigned pos = base + part[k * (kChunk / 128) + warp] + __popc(m[k] & lt);
                    nv[pos] = wv[k];
                    np_[pos] = wp[k];
                }
            __syncthreads();  // part is reused by the next chunk
        }
        grid.sync();
        if (s.gen_hist && tid == 0) atomicAdd(&s.gen_hist[128 + hc], ws_clock() - t_start);
        cur ^= 1;
    }
    if (tid == 0) {
        out[0] = static_cast<unsigned long long>(it);
        out[1] = static_cast<unsigned long long>(cur);
    }
}

// A small depth bucket (n <= kSmallBucket entries) sorted by time in one block and unpacked
// into the first generation, with its size; replaces a radix sort and two more launches.
constexpr int kSmallBucket = 2048;

__global__ void __launch_bounds__(1024) ws_sort_small(const unsigned long long* __restrict__ time,
                                                      const unsigned long long* __restrict__ val, unsigned n,
                                                      uint32_t* __restrict__ gv, uint32_t* __restrict__ gp,
                                                      unsigned int* __restrict__ ng) {
    __shared__ unsigned long long st[kSmallBucket];
    __shared__ unsigned long long sv[kSmallBucket];
    unsigned N = 1;
    while (N < n) N <<= 1;
    for (unsigned i = threadIdx.x; i < N; i += blockDim.x) {
        st[i] = i < n ? time[i] : ~0ull;
        sv[i] = i < n ? val[i] : 0ull;
    }
    __syncthreads();
    for (unsigned k = 2; k <= N; k <<= 1)  // bitonic sort by time (times are distinct)
        for (unsigned j = k >> 1; j > 0; j >>= 1) {
            for (unsigned i = threadIdx.x; i < N; i += blockDim.x) {
                const unsigned q = i ^ j;
                if (q > i) {
                    const unsigned long long a = st[i], c = st[q];
                    if (((i & k) == 0) ? (a > c) : (a < c)) {
                        st[i] = c;
                        st[q] = a;
                        const unsigned long long t = sv[i];
                        sv[i] = sv[q];
                        sv[q] = t;
                    }
                }
            }
            __syncthreads();
        }
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) {
        gv[i] = static_cast<uint32_t>(sv[i]);
        gp[i] = static_cast<uint32_t>(sv[i] >> 32);
    }
    if (threadIdx.x == 0) *ng = n;
}

__global__ void ws_unpack_entries(const unsigned long long* __restrict__ val, size_t n,
                                  uint32_t* __restrict__ gv, uint32_t* __restrict__ gp) {
    PMA_GRID_STRIDE(i, n) {
        gv[i] = static_cast<uint32_t>(val[i]);
        gp[i] = static_cast<uint32_t>(val[i] >> 32);
    }
}

__global__ void ws_volumes(const unsigned long long* __restrict__ state, int packed,
                           const uint32_t* __restrict__ ext, size_t n, unsigned long long* __restrict__ pvol,
                           uint8_t* __restrict__ shared_flag) {
    // lanes of a warp claimed by the same pore combine their counts
    const unsigned lane = threadIdx.x & 31;
    PMA_GRID_STRIDE(v, n) {
        const uint32_t c = ws_claimer(packed, state[v]);
        const bool sh = ext[v] != 0;
        shared_flag[v] = sh;
        const uint32_t key = (c && !sh) ? c : 0u;
        const unsigned peers = __match_any_sync(__activemask(), key);
        if (key && static_cast<int>(lane) == __ffs(peers) - 1)
            atomicAdd(&pvol[key - 1], static_cast<unsigned long long>(__popc(peers)));
    }
}

// --- shared types -------------------------------------------------------------------------

// Extending pores of the shared voxel whose chain starts at record `rec`, with their first
// touch times, in slot order; returns how many (at most kMaxExt).
__device__ __forceinline__ int ws_chain(const uint32_t* __restrict__ ext_pore,
                                        const unsigned long long* __restrict__ ext_time,
                                        const uint32_t* __restrict__ ext_next, uint32_t rec, uint32_t* p,
                                        unsigned long long* t) {
    int m = 0;
    for (int hop = 0; hop < kMaxHops && rec != 0 && rec != kRecBusy; ++hop) {
        for (int k = 0; k < kSlots; ++k) {
            const size_t slot = static_cast<size_t>(rec - 1) * kSlots + k;
            const uint32_t pk = ext_pore[slot];
            if (pk == kNone) return m;
            if (p) {
                p[m] = pk;
                t[m] = ext_time[slot];
            }
            ++m;
        }
        rec = ext_next[rec - 1];
    }
    return m;
}

// Key length (claimer + extending pores) of each shared voxel, for the offsets of its key and
// of its prefix records.
__global__ void ws_key_lengths(const uint32_t* __restrict__ sv, size_t ns, const uint32_t* __restrict__ ext,
                               const uint32_t* __restrict__ ext_pore, const uint32_t* __restrict__ ext_next,
                               uint8_t* __restrict__ klen, unsigned long long* __restrict__ klen64) {
    PMA_GRID_STRIDE(i, ns) {
        const int len = ws_chain(ext_pore, nullptr, ext_next, ext[sv[i]], nullptr, nullptr) + 1;
        klen[i] = static_cast<uint8_t>(len);
        klen64[i] = static_cast<unsigned long long>(len);
    }
}

// Key of shared voxel i: [first extension, claimer, later extensions...] in pore indices, at
// kseq[koff[i] ..], and one record per prefix of length L = 2..len at record
// koff[i] - i + L - 2 (its hashes, creation time and voxel).
__global__ void ws_keys(const uint32_t* __restrict__ sv, size_t ns, const unsigned long long* __restrict__ state,
                        int packed,
                        const uint32_t* __restrict__ ext, const uint32_t* __restrict__ ext_pore,
                        const unsigned long long* __restrict__ ext_time, const uint32_t* __restrict__ ext_next,
                        const unsigned long long* __restrict__ koff, uint32_t* __restrict__ kseq,
                        unsigned long long* __restrict__ rh1, unsigned long long* __restrict__ rh2,
                        unsigned long long* __restrict__ rtime, uint32_t* __restrict__ rvox) {
    PMA_GRID_STRIDE(i, ns) {
        const uint32_t v = sv[i];
        uint32_t p[kMaxExt];
        unsigned long long t[kMaxExt];
        const int m = ws_chain(ext_pore, ext_time, ext_next, ext[v], p, t);
        for (int a = 1; a < m; ++a)  // insertion sort by time
            for (int b = a; b > 0 && t[b] < t[b - 1]; --b) {
                const unsigned long long tt = t[b];
                t[b] = t[b - 1];
                t[b - 1] = tt;
                const uint32_t pp = p[b];
                p[b] = p[b - 1];
                p[b - 1] = pp;
            }
        uint32_t key[kKeyMax];
        key[0] = p[0];
        key[1] = ws_claimer(packed, state[v]) - 1;
        for (int k = 1; k < m; ++k) key[k + 1] = p[k];
        const int len = m + 1;
        const unsigned long long base = koff[i];
        for (int k = 0; k < len; ++k) kseq[base + k] = key[k];
        const unsigned long long rbase = base - i;
        for (int L = 2; L <= len; ++L) {
            const unsigned long long r = rbase + (L - 2);
            unsigned long long h1, h2;
            list_hash(key, static_cast<uint32_t>(L), h1, h2);
            rh1[r] = h1;
            rh2[r] = h2;
            rtime[r] = t[L - 2];
            rvox[r] = static_cast<uint32_t>(i);
        }
    }
}

__global__ void ws_iota(uint32_t* __restrict__ a, size_t n) {
    PMA_GRID_STRIDE(i, n) a[i] = static_cast<uint32_t>(i);
}

__global__ void ws_gather_h(const unsigned long long* __restrict__ h, const uint32_t* __restrict__ idx,
                            size_t n, unsigned long long* __restrict__ out) {
    PMA_GRID_STRIDE(i, n) out[i] = h[idx[i]];
}

// Prefix record r: its voxel, the start of that voxel's key and the prefix length.
struct RecRef {
    uint32_t vi;
    unsigned long long kbase;
    uint32_t L;
};

__device__ __forceinline__ RecRef ws_rec(uint32_t r, const uint32_t* __restrict__ rvox,
                                         const unsigned long long* __restrict__ koff) {
    RecRef x;
    x.vi = rvox[r];
    x.kbase = koff[x.vi];
    x.L = static_cast<uint32_t>(r - (x.kbase - x.vi)) + 2u;
    return x;
}

__global__ void ws_group_starts(const uint32_t* __restrict__ rec, size_t nr,
                                const unsigned long long* __restrict__ rh1,
                                const unsigned long long* __restrict__ rh2, const uint32_t* __restrict__ kseq,
                                const unsigned long long* __restrict__ koff, const uint32_t* __restrict__ rvox,
                                uint32_t* __restrict__ start, unsigned int* __restrict__ err) {
    PMA_GRID_STRIDE(i, nr) {
        const uint32_t r = rec[i];
        bool s = i == 0;
        if (!s) {
            const uint32_t q = rec[i - 1];
            s = rh1[r] != rh1[q] || rh2[r] != rh2[q];
            // equal first hashes, different second ones: sorted by the first hash alone, such
            // prefixes may interleave (the host then sorts by both)
            if (rh1[r] == rh1[q] && rh2[r] != rh2[q]) atomicOr(err, 64u);
            if (!s) {  // verify: same prefix
                const RecRef a = ws_rec(r, rvox, koff), b = ws_rec(q, rvox, koff);
                bool eq = a.L == b.L;
                for (uint32_t k = 0; eq && k < a.L; ++k) eq = kseq[a.kbase + k] == kseq[b.kbase + k];
                if (!eq) atomicOr(err, 4u);
            }
        }
        start[i] = s ? 1u : 0u;
    }
}

__global__ void ws_group_reduce(const uint32_t* __restrict__ rec, const uint32_t* __restrict__ excl,
                                const uint32_t* __restrict__ start, size_t nr,
                                const unsigned long long* __restrict__ rtime, const uint8_t* __restrict__ klen,
                                const unsigned long long* __restrict__ koff, const uint32_t* __restrict__ rvox,
                                unsigned long long* __restrict__ gtime, unsigned long long* __restrict__ gvol,
                                uint32_t* __restrict__ grep, uint32_t* __restrict__ final_group) {
    PMA_GRID_STRIDE(i, nr) {
        const uint32_t r = rec[i];
        const uint32_t g = excl[i] + start[i] - 1u;
        atomicMin(&gtime[g], rtime[r]);
        const RecRef a = ws_rec(r, rvox, koff);
        if (a.L == klen[a.vi]) {
            atomicAdd(&gvol[g], 1ull);
            final_group[a.vi] = g;
        }
        if (start[i]) grep[g] = r;
    }
}

__global__ void ws_labels(const unsigned long long* __restrict__ state, int packed, size_t n,
                          const uint32_t* __restrict__ pore_id, uint32_t* __restrict__ labels) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t c = ws_claimer(packed, state[v]);
        labels[v] = c ? pore_id[c - 1] : 0u;
    }
}

__global__ void ws_shared_labels(const uint32_t* __restrict__ sv, const uint32_t* __restrict__ final_group,
                                 const uint32_t* __restrict__ gid, size_t ns, uint32_t* __restrict__ labels) {
    PMA_GRID_STRIDE(i, ns) labels[sv[i]] = gid[final_group[i]];
}

__global__ void ws_group_rows(const uint32_t* __restrict__ grep, size_t ngr, const uint32_t* __restrict__ kseq,
                              const unsigned long long* __restrict__ koff, const uint32_t* __restrict__ rvox,
                              uint32_t* __restrict__ out) {
    PMA_GRID_STRIDE(g, ngr) {
        const RecRef a = ws_rec(grep[g], rvox, koff);
        for (uint32_t k = 0; k < kKeyMax; ++k) out[g * kKeyMax + k] = k < a.L ? kseq[a.kbase + k] : kNone;
    }
}

template <class T>
T* buf(pma_ctx* ctx, const char* tag, size_t count) {
    return static_cast<T*>(ctx->scratch(tag, std::max<size_t>(count, 1) * sizeof(T)));
}

}  // namespace

pma_table* watershed(pma_ctx* ctx, const pma_table* pt, const uint32_t* crad2, pma_dims d,
                     pma_stencil st, uint32_t max_edt2, uint32_t* labels) {
    KernelTimer kt_stage(ctx, "stage_watershed");  // the whole stage, for the untimed remainder
    check_dims(d);
    PMA_REQUIRE(crad2 && labels, PMA_ERR_ARGUMENT, "pma_watershed: null device pointer");
    cudaStream_t s = ctx->stream;
    const size_t n = voxels(d);
    const Grid g{d.sx, d.sy, d.sz};
    const unsigned G = grid_for(ctx, n);
    const size_t npores = pt->pores.size();
    const uint32_t nb = max_edt2 + 1;

    // Seeds (WatershedComputer.cpp:183-219), in pore-id order.
    std::vector<pma_pore> pores = pt->pores;
    std::sort(pores.begin(), pores.end(), [](const pma_pore& a, const pma_pore& b) { return a.id < b.id; });
    std::vector<uint32_t> seed_voxel(npores);
    std::vector<uint32_t> seed_hist(nb, 0);
    for (size_t k = 0; k < npores; ++k) {
        const pma_pore& p = pores[k];
        PMA_REQUIRE(g.inside(p.seed_x, p.seed_y, p.seed_z), PMA_ERR_ARGUMENT,
                    "pma_watershed: pore seed outside the image");
        PMA_REQUIRE(p.seed_r2 <= max_edt2, PMA_ERR_ARGUMENT, "pma_watershed: pore seed radius above max_edt2");
        seed_voxel[k] = static_cast<uint32_t>(g.idx(p.seed_x, p.seed_y, p.seed_z));
        seed_hist[p.seed_r2]++;
    }
    {
        std::vector<uint32_t> sv = seed_voxel;
        std::sort(sv.begin(), sv.end());
        PMA_REQUIRE(std::adjacent_find(sv.begin(), sv.end()) == sv.end(), PMA_ERR_ARGUMENT,
                    "pma_watershed: two pores share a seed voxel");
    }

    int64_t* d_count = buf<int64_t>(ctx, "ws.count", 4);
    unsigned int* d_ng = reinterpret_cast<unsigned int*>(d_count + 3);  // two frontier sizes
    WsState ws;
    ws.g = g;
    ws.d3q7 = st == PMA_D3Q7 ? 1 : 0;
    ws.crad = crad2;
    ws.state = buf<unsigned long long>(ctx, "ws.state", n);
    ws.packed = max_edt2 < 65536u ? 1 : 0;  // radii up to max_edt2 fit the word's low 16 bits
    ws.ext = buf<uint32_t>(ctx, "ws.ext", n);
    ws.ext_count = reinterpret_cast<unsigned int*>(d_count + 1);
    ws.err = reinterpret_cast<unsigned int*>(d_count + 2);
    ws.spin_limit = ctx->limits.spin_limit;
    ws.gen_hist = nullptr;
    if (ctx->timing) {  // frontier sizes of the generations, for the timing report
        ws.gen_hist = buf<unsigned long long>(ctx, "ws.gen_hist", 194);
        PMA_CUDA(cudaMemsetAsync(ws.gen_hist, 0, 194 * 8, s));
    }
    ws.pbound = buf<unsigned int>(ctx, "ws.pbound", npores);
    // Shared-voxel records: a first guess of n/32; the pool doubles (copying the records)
    // whenever it is more than half used at a host synchronisation point, and a flood that
    // still runs out is redone with four times as many (up to two per voxel).
    const size_t max_records = std::min<size_t>(2 * n + 4096, 0x7FFFFFFF / kSlots);
    size_t ext_cap = std::min<size_t>(std::max<size_t>(n / 32, 4096), max_records);
    int ext_side = 0;  // which of two scratch tags holds the records
    auto ext_tag = [&](const char* base) { return std::string(base) + (ext_side ? ".1" : ".0"); };
    auto grow_records = [&](size_t used) {
        if (2 * used <= ws.ext_cap || ws.ext_cap >= max_records) return;
        const size_t old_cap = ws.ext_cap;
        const size_t cap2 = std::min<size_t>(std::max<size_t>(2 * old_cap, 4 * used), max_records);
        const std::string old_p = ext_tag("ws.ext_pore"), old_t = ext_tag("ws.ext_time"),
                          old_n = ext_tag("ws.ext_next");
        ext_side ^= 1;
        auto* np_ = buf<uint32_t>(ctx, ext_tag("ws.ext_pore").c_str(), cap2 * kSlots);
        auto* nt_ = buf<unsigned long long>(ctx, ext_tag("ws.ext_time").c_str(), cap2 * kSlots);
        auto* nn_ = buf<uint32_t>(ctx, ext_tag("ws.ext_next").c_str(), cap2);
        PMA_CUDA(cudaMemcpyAsync(np_, ws.ext_pore, old_cap * kSlots * 4, cudaMemcpyDeviceToDevice, s));
        PMA_CUDA(cudaMemcpyAsync(nt_, ws.ext_time, old_cap * kSlots * 8, cudaMemcpyDeviceToDevice, s));
        PMA_CUDA(cudaMemcpyAsync(nn_, ws.ext_next, old_cap * 4, cudaMemcpyDeviceToDevice, s));
        PMA_CUDA(cudaMemsetAsync(np_ + old_cap * kSlots, 0xFF, (cap2 - old_cap) * kSlots * 4, s));
        PMA_CUDA(cudaMemsetAsync(nt_ + old_cap * kSlots, 0xFF, (cap2 - old_cap) * kSlots * 8, s));
        PMA_CUDA(cudaMemsetAsync(nn_ + old_cap, 0, (cap2 - old_cap) * 4, s));
        ctx->release(old_p);
        ctx->release(old_t);
        ctx->release(old_n);
        ws.ext_pore = np_;
        ws.ext_time = nt_;
        ws.ext_next = nn_;
        ws.ext_cap = static_cast<uint32_t>(cap2);
    };
    unsigned int h_err = 0;
    for (;;) {
        const size_t start_cap = ext_cap;
        ws.ext_cap = static_cast<uint32_t>(ext_cap);
        ws.ext_pore = buf<uint32_t>(ctx, ext_tag("ws.ext_pore").c_str(), static_cast<size_t>(ws.ext_cap) * kSlots);
        ws.ext_time = buf<unsigned long long>(ctx, ext_tag("ws.ext_time").c_str(),
                                              static_cast<size_t>(ws.ext_cap) * kSlots);
        ws.ext_next = buf<uint32_t>(ctx, ext_tag("ws.ext_next").c_str(), ws.ext_cap);
        PMA_CUDA(cudaMemsetAsync(ws.ext_next, 0, static_cast<size_t>(ws.ext_cap) * 4, s));
        PMA_CUDA(cudaMemsetAsync(d_count, 0, 32, s));
        PMA_CUDA(cudaMemsetAsync(ws.ext_pore, 0xFF, static_cast<size_t>(ws.ext_cap) * kSlots * 4, s));
        PMA_CUDA(cudaMemsetAsync(ws.ext_time, 0xFF, static_cast<size_t>(ws.ext_cap) * kSlots * 8, s));
        PMA_CUDA(cudaMemsetAsync(ws.pbound, 0, std::max<size_t>(npores, 1) * 4, s));
        ws_init<<<G, 256, 0, s>>>(n, crad2, ws.packed, ws.state, ws.ext);
        ctx->check_launch("ws_init");

        // Buckets: capacity = voxels of that crad + seeds of that radius.
        unsigned int* hist = buf<unsigned int>(ctx, "ws.hist", nb);
        PMA_CUDA(cudaMemsetAsync(hist, 0, nb * 4ull, s));
        ws_histograms<<<G, 256, 0, s>>>(crad2, n, nb, hist);
        ctx->check_launch("ws_histograms");
        std::vector<unsigned int> h_hist(nb);
        PMA_CUDA(cudaMemcpyAsync(h_hist.data(), hist, nb * 4ull, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        std::vector<unsigned long long> boff(nb + 1, 0);
        size_t max_bucket = 1;
        for (uint32_t b = 0; b < nb; ++b) {
            const unsigned long long c = static_cast<unsigned long long>(h_hist[b]) + seed_hist[b];
            boff[b + 1] = boff[b] + c;
            max_bucket = std::max<size_t>(max_bucket, c);
        }
        const unsigned long long total = boff[nb];
        auto* d_boff = buf<unsigned long long>(ctx, "ws.boff", nb + 1);
        ws.boff = d_boff;
        ws.bfill = buf<unsigned int>(ctx, "ws.bfill", nb);
        ws.ent_time = buf<unsigned long long>(ctx, "ws.ent_time", total);
        ws.ent_val = buf<unsigned long long>(ctx, "ws.ent_val", total);
        auto* srt_time = buf<unsigned long long>(ctx, "ws.srt_time", max_bucket);
        auto* srt_val = buf<unsigned long long>(ctx, "ws.srt_val", max_bucket);
        const size_t max_events = max_bucket * 27;
        // bucket entry times: events (and the seeds' pore indices) below 2^time_shift, so that a
        // depth's sort needs only time_shift + bits(generation) key bits
        ws.time_shift = 1;
        while (ws.time_shift < 41 && (1ull << ws.time_shift) <= std::max<size_t>(max_events, npores)) ++ws.time_shift;

        ws.ev_touch = buf<uint8_t>(ctx, "ws.ev_touch", max_events);  // written for every event by phase 0
        // chunk descriptors of the frontier compaction; generations restart at 1 in this attempt
        const size_t max_chunks = (max_events + kChunk - 1) / kChunk;
        auto* desc = buf<unsigned long long>(ctx, "ws.desc", max_chunks);
        PMA_CUDA(cudaMemsetAsync(desc, 0, max_chunks * 8, s));
        PMA_CUDA(cudaMemcpyAsync(d_boff, boff.data(), (nb + 1) * 8ull, cudaMemcpyHostToDevice, s));
        std::vector<unsigned int> h_fill(nb, 0);
        if (npores) {
            std::vector<unsigned long long> a(3 * npores);
            for (size_t k = 0; k < npores; ++k) {
                const uint32_t b = pores[k].seed_r2;
                a[k] = boff[b] + h_fill[b]++;
                a[npores + k] = k;  // seeds come first in their bucket, in pore-id order
                a[2 * npores + k] = (static_cast<unsigned long long>(k) << 32) | seed_voxel[k];
            }
            auto* d_a = buf<unsigned long long>(ctx, "ws.seed_at", 3 * npores);
            PMA_CUDA(cudaMemcpyAsync(d_a, a.data(), 3 * npores * 8, cudaMemcpyHostToDevice, s));
            ws_seed_entries<<<grid_for(ctx, npores), 256, 0, s>>>(d_a, npores, ws.ent_time, ws.ent_val);
            ctx->check_launch("ws_seed_entries");
            uint32_t* d_seed = buf<uint32_t>(ctx, "ws.seedvox", npores);
            PMA_CUDA(cudaMemcpyAsync(d_seed, seed_voxel.data(), npores * 4, cudaMemcpyHostToDevice, s));
            ws_seed<<<grid_for(ctx, npores), 256, 0, s>>>(d_seed, npores, crad2, ws.packed, ws.state);
            ctx->check_launch("ws_seed");
            ctx->sync();
        }
        PMA_CUDA(cudaMemcpyAsync(ws.bfill, h_fill.data(), nb * 4ull, cudaMemcpyHostToDevice, s));
        ctx->sync();

        // Depth sweep (WatershedComputer.cpp:80-102).
        uint32_t* gvb[2] = {buf<uint32_t>(ctx, "ws.gv0", max_bucket), buf<uint32_t>(ctx, "ws.gv1", max_bucket)};
        uint32_t* gpb[2] = {buf<uint32_t>(ctx, "ws.gp0", max_bucket), buf<uint32_t>(ctx, "ws.gp1", max_bucket)};
        // cooperative grid: every block resident at once (grid-wide barriers)
        int per_sm = 0;
        PMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ws_generations, kChunk / 4, 0));
        PMA_REQUIRE(per_sm > 0, PMA_ERR_CUDA, "pma_watershed: generation kernel does not fit an SM");
        // sized to the largest frontier (about 16 events per thread and phase), so that the
        // launches of small volumes leave the rest of the GPU to other streams (batch lanes).
        // (Sizing each launch to its starting frontier instead, at about 4 events per thread,
        // made barriers cheaper but the step slower: 950 -> 971 ms at 1024^3.)
        const size_t coop_need = (max_events + 16 * (kChunk / 4) - 1) / (16 * (kChunk / 4));
        const unsigned coop_grid = static_cast<unsigned>(
            std::max<size_t>(1, std::min<size_t>(coop_need, static_cast<size_t>(ctx->num_sms) * std::min(per_sm, 8))));
        unsigned long long gen = 0;
        // generations of this call at most: the context's bound, within the entry-time range
        const unsigned long long max_gen =
            std::min<unsigned long long>(ctx->limits.watershed_generations, kMaxGen - 1);
        unsigned int* h_small = static_cast<unsigned int*>(ctx->host_staging(64));
        auto* d_out = buf<unsigned long long>(ctx, "ws.coop_out", 2);
        unsigned long long* h_out = reinterpret_cast<unsigned long long*>(h_small + 8);
        // depths that can hold entries, deepest first
        std::vector<int64_t> depths;
        for (int64_t depth = static_cast<int64_t>(nb) - 1; depth >= 0; --depth)
            if (boff[depth + 1] != boff[depth]) depths.push_back(depth);
        bool have_count = false;  // entry count of depths[di] read with the previous depth's sync
        size_t n0 = 0;
        for (size_t di = 0; di < depths.size(); ++di) {
            const int64_t depth = depths[di];
            if (!have_count) {
                ReadBack rb;
                rb.add(h_small, ws.bfill + depth, 4);
                rb.add(h_small + 4, ws.ext_count, 4);
                read_back(ctx, rb);
                grow_records(h_small[4]);
                n0 = h_small[0];
            }
            have_count = false;
            if (n0 == 0) continue;
            int cur = 0;
            auto kt_sort = std::make_unique<KernelTimer>(ctx, "ws_depth_sort");
            if (n0 <= static_cast<size_t>(kSmallBucket)) {
                ws_sort_small<<<1, 1024, 0, s>>>(ws.ent_time + boff[depth], ws.ent_val + boff[depth],
                                                 static_cast<unsigned>(n0), gvb[cur], gpb[cur], d_ng + cur);
                ctx->check_launch("ws_sort_small");
            } else {
                int gen_bits = 0;
                while (gen_bits < 24 && (1ull << gen_bits) <= gen) ++gen_bits;
                sort_pairs(ctx, ws.ent_time + boff[depth], srt_time, ws.ent_val + boff[depth], srt_val,
                           static_cast<int64_t>(n0), std::min(64, ws.time_shift + gen_bits));
                ws_unpack_entries<<<grid_for(ctx, n0), 256, 0, s>>>(srt_val, n0, gvb[cur], gpb[cur]);
                ctx->check_launch("ws_unpack_entries");
                h_small[2] = static_cast<unsigned int>(n0);
                PMA_CUDA(cudaMemcpyAsync(d_ng + cur, &h_small[2], 4, cudaMemcpyHostToDevice, s));
            }
            kt_sort.reset();
            const int64_t next_depth = di + 1 < depths.size() ? depths[di + 1] : -1;
            KernelTimer kt(ctx, "ws_generations");
            while (true) {
                const uint32_t dep = static_cast<uint32_t>(depth);
                PMA_REQUIRE(gen < max_gen, PMA_ERR_LIMIT, "pma_watershed: generation limit reached");
                int gens = static_cast<int>(std::min<unsigned long long>(kGensPerLaunch, max_gen - gen));
                void* args[] = {&ws, &gvb[0], &gpb[0], &gvb[1], &gpb[1], &d_ng, &desc,
                                const_cast<uint32_t*>(&dep), &gen, &gens, &cur, &d_out};
                PMA_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(ws_generations), coop_grid,
                                                     kChunk / 4, args, 0, s));
                ctx->count_launch(1);
                ctx->count("ws.cooperative_launches", 1);
                {
                    ReadBack rb;
                    rb.add(h_out, d_out, 16);
                    rb.add(h_small + 4, ws.ext_count, 4);
                    rb.add(h_small + 6, d_ng, 8);
                    // the next depth's entries are final once this depth is done: read them along
                    if (next_depth >= 0) rb.add(h_small, ws.bfill + next_depth, 4);
                    read_back(ctx, rb);
                }
                gen += h_out[0];
                cur = static_cast<int>(h_out[1]);
                grow_records(h_small[4]);
                if (h_small[6 + cur] == 0) break;
            }
            if (next_depth >= 0) {
                n0 = h_small[0];
                have_count = true;
            }
        }
        PMA_CUDA(cudaMemcpyAsync(&h_err, ws.err, 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        if (!(h_err & 1u)) break;
        PMA_REQUIRE(start_cap < max_records, PMA_ERR_MEMORY, "pma_watershed: shared-voxel records exhausted");
        ext_cap = std::min<size_t>(std::max<size_t>(ws.ext_cap, start_cap * 4), max_records);
    }
    PMA_REQUIRE(!(h_err & 2u), PMA_ERR_INTERNAL, "pma_watershed: a shared voxel recorded more pores than touch it");
    PMA_REQUIRE(!(h_err & 8u), PMA_ERR_LIMIT, "pma_watershed: shared-voxel record allocation did not finish");
    PMA_REQUIRE(!(h_err & 16u), PMA_ERR_LIMIT, "pma_watershed: frontier compaction look-back did not finish");
    if (ws.gen_hist) {
        unsigned long long hh[194];
        PMA_CUDA(cudaMemcpyAsync(hh, ws.gen_hist, sizeof(hh), cudaMemcpyDeviceToHost, s));
        ctx->sync();
        for (int b = 0; b < 64; ++b)
            if (hh[b]) {
                const std::string c = "ws.generations.frontier_2^" + std::to_string(b);
                ctx->count(c, static_cast<double>(hh[b]));
                ctx->count(c + ".claim_ms", hh[64 + b] * 1e-6);
                ctx->count(c + ".resolve_ms", hh[128 + b] * 1e-6);
            }
        ctx->count("ws.block0.resolve_events_ms", hh[192] * 1e-6);
        ctx->count("ws.block0.scan_lookback_ms", hh[193] * 1e-6);
    }

    KernelTimer kt_tables(ctx, "ws_tables");  // to the end of the stage
    // Volumes, labels and shared voxels.
    auto* pvol = buf<unsigned long long>(ctx, "ws.pvol", npores);
    uint8_t* shared_flag = buf<uint8_t>(ctx, "ws.shared_flag", n);
    PMA_CUDA(cudaMemsetAsync(pvol, 0, std::max<size_t>(npores, 1) * 8, s));
    ws_volumes<<<G, 256, 0, s>>>(ws.state, ws.packed, ws.ext, n, pvol, shared_flag);
    ctx->check_launch("ws_volumes");
    std::vector<uint32_t> pore_id(std::max<size_t>(npores, 1));
    for (size_t k = 0; k < npores; ++k) pore_id[k] = pores[k].id;
    uint32_t* d_pid = buf<uint32_t>(ctx, "ws.pid", pore_id.size());
    PMA_CUDA(cudaMemcpyAsync(d_pid, pore_id.data(), pore_id.size() * 4, cudaMemcpyHostToDevice, s));
    ws_labels<<<G, 256, 0, s>>>(ws.state, ws.packed, n, d_pid, labels);
    ctx->check_launch("ws_labels");
    uint32_t* sv = buf<uint32_t>(ctx, "ws.sv", n);
    const int64_t nsh = select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), shared_flag, sv,
                                       static_cast<int64_t>(n), d_count);

    pma_table* t = new pma_table;
    std::vector<unsigned long long> h_pvol(npores);
    std::vector<unsigned int> h_pbound(npores);
    if (npores) {
        PMA_CUDA(cudaMemcpyAsync(h_pvol.data(), pvol, npores * 8, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(h_pbound.data(), ws.pbound, npores * 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
    }
    for (size_t k = 0; k < npores; ++k) {
        pma_pore p = pores[k];
        p.volume = h_pvol[k];
        p.is_boundary = h_pbound[k] ? 1 : 0;
        t->pores.push_back(p);
    }
    if (nsh == 0) return t;

    // Shared types on the device: key lengths, key and prefix-record offsets, keys and
    // prefix records, then the prefixes grouped by hash and ranked by creation time.
    uint8_t* klen = buf<uint8_t>(ctx, "ws.klen", nsh);
    auto* klen64 = buf<unsigned long long>(ctx, "ws.klen64", nsh);
    auto* koff = buf<unsigned long long>(ctx, "ws.koff", nsh);
    ws_key_lengths<<<grid_for(ctx, nsh), 256, 0, s>>>(sv, nsh, ws.ext, ws.ext_pore, ws.ext_next, klen, klen64);
    ctx->check_launch("ws_key_lengths");
    exclusive_sum(ctx, klen64, koff, nsh);
    unsigned long long kl[2] = {0, 0};
    PMA_CUDA(cudaMemcpyAsync(&kl[0], koff + nsh - 1, 8, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(&kl[1], klen64 + nsh - 1, 8, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    const unsigned long long nkey = kl[0] + kl[1];      // key elements of all shared voxels
    const unsigned long long nrec_u = nkey - static_cast<unsigned long long>(nsh);  // prefixes
    PMA_REQUIRE(nrec_u < 0xFFFFFFFFull, PMA_ERR_LIMIT, "pma_watershed: too many shared voxels");
    const int64_t nr = static_cast<int64_t>(nrec_u);
    uint32_t* kseq = buf<uint32_t>(ctx, "ws.kseq", nkey);
    auto* rh1 = buf<unsigned long long>(ctx, "ws.rh1", nr);
    auto* rh2 = buf<unsigned long long>(ctx, "ws.rh2", nr);
    auto* rtime = buf<unsigned long long>(ctx, "ws.rtime", nr);
    uint32_t* rvox = buf<uint32_t>(ctx, "ws.rvox", nr);
    ws_keys<<<grid_for(ctx, nsh), 256, 0, s>>>(sv, nsh, ws.state, ws.packed, ws.ext, ws.ext_pore, ws.ext_time, ws.ext_next,
                                               koff, kseq, rh1, rh2, rtime, rvox);
    ctx->check_launch("ws_keys");
    uint32_t* rec = buf<uint32_t>(ctx, "ws.rec", nr);
    uint32_t* rec2 = buf<uint32_t>(ctx, "ws.rec2", nr);
    ws_iota<<<grid_for(ctx, nr), 256, 0, s>>>(rec, nr);
    ctx->check_launch("ws_iota");
    // Equal prefixes become adjacent: a radix sort by the first hash (values: record ids),
    // unless two different prefixes share it (about n^2 / 2^65 likely), which ws_group_starts
    // flags; then stable sorts by the second hash and then the first.
    auto* kh = buf<unsigned long long>(ctx, "ws.kh", nr);
    auto* kh2 = buf<unsigned long long>(ctx, "ws.kh2", nr);
    uint32_t* gstart = buf<uint32_t>(ctx, "ws.gstart", nr);
    uint32_t* gexcl = buf<uint32_t>(ctx, "ws.gexcl", nr);
    sort_pairs(ctx, rh1, kh2, rec, rec2, nr);
    ws_group_starts<<<grid_for(ctx, nr), 256, 0, s>>>(rec2, nr, rh1, rh2, kseq, koff, rvox, gstart, ws.err);
    ctx->check_launch("ws_group_starts");
    PMA_CUDA(cudaMemcpyAsync(&h_err, ws.err, 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    if (h_err & 64u) {
        PMA_CUDA(cudaMemsetAsync(ws.err, 0, 4, s));
        sort_pairs(ctx, rh2, kh2, rec, rec2, nr);
        ws_gather_h<<<grid_for(ctx, nr), 256, 0, s>>>(rh1, rec2, nr, kh);
        ctx->check_launch("ws_gather_h");
        sort_pairs(ctx, kh, kh2, rec2, rec, nr);
        PMA_CUDA(cudaMemcpyAsync(rec2, rec, nr * 4, cudaMemcpyDeviceToDevice, s));
        ws_group_starts<<<grid_for(ctx, nr), 256, 0, s>>>(rec2, nr, rh1, rh2, kseq, koff, rvox, gstart, ws.err);
        ctx->check_launch("ws_group_starts");
    }
    rec = rec2;  // records in group order from here on
    exclusive_sum(ctx, gstart, gexcl, nr);
    uint32_t last[2] = {0, 0};
    PMA_CUDA(cudaMemcpyAsync(&last[0], gexcl + nr - 1, 4, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(&last[1], gstart + nr - 1, 4, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(&h_err, ws.err, 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    PMA_REQUIRE(!(h_err & 4u), PMA_ERR_INTERNAL, "pma_watershed: shared-type hash collision");
    const int64_t ngr = static_cast<int64_t>(last[0]) + last[1];
    auto* gtime = buf<unsigned long long>(ctx, "ws.gtime", ngr);
    auto* gvol = buf<unsigned long long>(ctx, "ws.gvol", ngr);
    uint32_t* grep = buf<uint32_t>(ctx, "ws.grep", ngr);
    uint32_t* final_group = buf<uint32_t>(ctx, "ws.fgroup", nsh);
    PMA_CUDA(cudaMemsetAsync(gtime, 0xFF, ngr * 8, s));
    PMA_CUDA(cudaMemsetAsync(gvol, 0, ngr * 8, s));
    ws_group_reduce<<<grid_for(ctx, nr), 256, 0, s>>>(rec, gexcl, gstart, nr, rtime, klen, koff, rvox, gtime,
                                                      gvol, grep, final_group);
    ctx->check_launch("ws_group_reduce");
    uint32_t* rows = buf<uint32_t>(ctx, "ws.rows", static_cast<size_t>(ngr) * kKeyMax);
    ws_group_rows<<<grid_for(ctx, ngr), 256, 0, s>>>(grep, ngr, kseq, koff, rvox, rows);
    ctx->check_launch("ws_group_rows");
    std::vector<unsigned long long> h_gtime(ngr), h_gvol(ngr);
    std::vector<uint32_t> h_rows(static_cast<size_t>(ngr) * kKeyMax);
    PMA_CUDA(cudaMemcpyAsync(h_gtime.data(), gtime, ngr * 8, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(h_gvol.data(), gvol, ngr * 8, cudaMemcpyDeviceToHost, s));
    PMA_CUDA(cudaMemcpyAsync(h_rows.data(), rows, h_rows.size() * 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    // ids in creation order
    std::vector<std::pair<unsigned long long, uint32_t>> by_time(ngr);  // creation times are distinct
    for (int64_t i = 0; i < ngr; ++i) by_time[i] = {h_gtime[i], static_cast<uint32_t>(i)};
    std::sort(by_time.begin(), by_time.end());
    std::vector<uint32_t> order(ngr);
    for (int64_t k = 0; k < ngr; ++k) order[k] = by_time[k].second;
    std::vector<uint32_t> gid(ngr);
    for (int64_t k = 0; k < ngr; ++k) gid[order[k]] = 0xFFFFFFFFu - 1u - static_cast<uint32_t>(k);
    uint32_t* d_gid = buf<uint32_t>(ctx, "ws.gid", ngr);
    PMA_CUDA(cudaMemcpyAsync(d_gid, gid.data(), ngr * 4, cudaMemcpyHostToDevice, s));
    ws_shared_labels<<<grid_for(ctx, nsh), 256, 0, s>>>(sv, final_group, d_gid, nsh, labels);
    ctx->check_launch("ws_shared_labels");
    ctx->sync();
    // rows in id order (ascending id = reverse creation order)
    t->throats.reserve(ngr);
    t->pool.reserve(static_cast<size_t>(ngr) * 3);
    for (int64_t k = ngr - 1; k >= 0; --k) {
        const uint32_t gi = order[k];
        pma_throat th;
        th.id = gid[gi];
        th.volume = h_gvol[gi];
        th.pool_offset = t->pool.size();
        uint32_t L = 0;
        for (int j = 0; j < kKeyMax && h_rows[static_cast<size_t>(gi) * kKeyMax + j] != kNone; ++j, ++L)
            t->pool.push_back(pore_id[h_rows[static_cast<size_t>(gi) * kKeyMax + j]]);
        th.n_pores = L;
        t->throats.push_back(th);
    }
    return t;
}

void wait_selftest(pma_ctx* ctx, int* timed_out) {
    unsigned long long* desc = buf<unsigned long long>(ctx, "ws.selftest", 3);
    unsigned int* err = reinterpret_cast<unsigned int*>(desc + 2);
    PMA_CUDA(cudaMemsetAsync(desc, 0, 3 * 8, ctx->stream));
    ws_wait_selftest<<<1, 32, 0, ctx->stream>>>(desc, err, ctx->limits.spin_limit);
    ctx->count_launch();
    ctx->check_launch("ws_wait_selftest");
    unsigned int h[2] = {0, 0};
    PMA_CUDA(cudaMemcpyAsync(h, err, 8, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    *timed_out = (h[0] & h[1] & 16u) ? 1 : 0;
}

}  // namespace pma
