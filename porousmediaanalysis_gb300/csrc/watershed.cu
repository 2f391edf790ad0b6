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
// depth, in push order. Every touch gets the time (generation, position of its node in the
// generation * 27 + neighbour index), which orders touches exactly as the sequential loop
// does. Per generation:
//   claim    - the smallest-time touch of each unclaimed voxel wins (atomicMin on time);
//   extend   - touches by other pores record, per voxel and pore, their first touch time;
//   queue    - claimed voxels in time order form the next generation (same depth) or are
//              appended, time-stamped, to the bucket of their depth, which is sorted by time
//              when that depth starts.
// Shared types are created at their first extension time, so sorting keys by that time
// reproduces the reference's id sequence (UINT32_MAX - 1, - 2, ...) exactly, including types
// whose volume later drops to zero.
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "devutil.cuh"

namespace pma {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr unsigned long long kNoTime = ~0ull;
constexpr int kSlots = 6;  // distinct extending pores recorded per shared voxel

struct WsState {
    Grid g;
    int d3q7;
    const uint32_t* crad;
    uint32_t* claim;             // pore index + 1, 0 = unclaimed
    unsigned long long* ckey;    // per-generation claim time (kNoTime when idle)
    uint32_t* ext;               // shared-voxel record + 1, 0 = none
    uint32_t* ext_pore;          // [records][kSlots]
    unsigned long long* ext_time;
    unsigned int* ext_count;
    uint32_t ext_cap;
    unsigned int* pbound;        // per pore
    unsigned int* err;
};

__global__ void ws_init(size_t n, uint32_t* __restrict__ claim, unsigned long long* __restrict__ ckey,
                        uint32_t* __restrict__ ext) {
    PMA_GRID_STRIDE(v, n) {
        claim[v] = 0;
        ckey[v] = kNoTime;
        ext[v] = 0;
    }
}

__global__ void ws_seed(const uint32_t* __restrict__ seed_voxel, size_t np, uint32_t* __restrict__ claim) {
    PMA_GRID_STRIDE(k, np) claim[seed_voxel[k]] = static_cast<uint32_t>(k + 1);
}

// Touch events of generation nodes: claims (phase 0), claim resolution (phase 1),
// extensions (phase 2). Node i, neighbour j has event number i * 27 + j.
template <int kPhase>
__global__ void ws_touch(WsState s, const uint32_t* __restrict__ gv, const uint32_t* __restrict__ gp,
                         size_t ng, uint32_t depth, unsigned long long gen,
                         uint32_t* __restrict__ slot_voxel) {
    PMA_GRID_STRIDE(i, ng) {
        const uint32_t v = gv[i];
        const uint32_t pore = gp[i];
        int x, y, z;
        s.g.coords(v, x, y, z);
        for (int j = 0; j < 27; ++j) {
            int dx, dy, dz;
            if (!stencil_offset(j, s.d3q7, dx, dy, dz)) continue;
            const int nx = x + dx, ny = y + dy, nz = z + dz;
            if (!s.g.inside(nx, ny, nz)) {  // WC.cpp:140-144
                if (kPhase == 0) s.pbound[pore] = 1;
                continue;
            }
            const size_t w = s.g.idx(nx, ny, nz);
            const uint32_t r = s.crad[w];
            if (r == 0 || r > depth) continue;  // WC.cpp:152-156
            const unsigned long long seq = static_cast<unsigned long long>(i) * 27 + j;
            if (kPhase == 0) {
                if (s.claim[w] == 0) atomicMin(&s.ckey[w], seq);
            } else if (kPhase == 1) {
                if (s.ckey[w] == seq) {
                    s.claim[w] = pore + 1;
                    s.ckey[w] = kNoTime;
                    slot_voxel[seq] = static_cast<uint32_t>(w);
                }
            } else {
                if (s.claim[w] == pore + 1) continue;
                // record (pore, first touch time) for w
                uint32_t rec = s.ext[w];
                if (rec == 0) {
                    const uint32_t fresh = atomicAdd(s.ext_count, 1u) + 1;
                    if (fresh > s.ext_cap) {
                        atomicOr(s.err, 1u);
                        continue;
                    }
                    const uint32_t old = atomicCAS(&s.ext[w], 0u, fresh);
                    rec = old ? old : fresh;
                }
                const unsigned long long t = (gen << 40) | seq;
                bool placed = false;
                for (int k = 0; k < kSlots && !placed; ++k) {
                    const size_t slot = static_cast<size_t>(rec - 1) * kSlots + k;
                    const uint32_t cur = atomicCAS(&s.ext_pore[slot], kNone, pore);
                    if (cur == kNone || cur == pore) {
                        atomicMin(&s.ext_time[slot], t);
                        placed = true;
                    }
                }
                if (!placed) atomicOr(s.err, 2u);
            }
        }
    }
}

struct SlotTaken {
    const uint32_t* slot_voxel;
    __host__ __device__ bool operator()(uint32_t seq) const { return slot_voxel[seq] != kNone; }
};

struct AtDepth {
    const uint32_t* slot_voxel;
    const uint32_t* crad;
    uint32_t depth;
    __host__ __device__ bool operator()(uint32_t seq) const { return crad[slot_voxel[seq]] == depth; }
};

// Claimed voxels in event order: same depth -> next generation, deeper -> their bucket.
__global__ void ws_distribute(const uint32_t* __restrict__ claimed, size_t nc,
                              const uint32_t* __restrict__ slot_voxel, const uint32_t* __restrict__ gp,
                              const uint32_t* __restrict__ crad, uint32_t depth, unsigned long long gen,
                              const unsigned long long* __restrict__ boff, unsigned int* __restrict__ bfill,
                              unsigned long long* __restrict__ ent_time,
                              unsigned long long* __restrict__ ent_val) {
    PMA_GRID_STRIDE(r, nc) {
        const uint32_t seq = claimed[r];
        const uint32_t w = slot_voxel[seq];
        const uint32_t b = crad[w];
        if (b == depth) continue;
        const unsigned pos = atomicAdd(&bfill[b], 1u);
        const unsigned long long at = boff[b] + pos;
        ent_time[at] = (gen << 40) | r;
        ent_val[at] = (static_cast<unsigned long long>(gp[seq / 27]) << 32) | w;
    }
}

__global__ void ws_next_generation(const uint32_t* __restrict__ sel, size_t n,
                                   const uint32_t* __restrict__ slot_voxel, const uint32_t* __restrict__ gp,
                                   uint32_t* __restrict__ nv, uint32_t* __restrict__ np_) {
    PMA_GRID_STRIDE(i, n) {
        const uint32_t seq = sel[i];
        nv[i] = slot_voxel[seq];
        np_[i] = gp[seq / 27];
    }
}

__global__ void ws_unpack_entries(const unsigned long long* __restrict__ val, size_t n,
                                  uint32_t* __restrict__ gv, uint32_t* __restrict__ gp) {
    PMA_GRID_STRIDE(i, n) {
        gv[i] = static_cast<uint32_t>(val[i]);
        gp[i] = static_cast<uint32_t>(val[i] >> 32);
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

__global__ void ws_histograms(const uint32_t* __restrict__ crad, size_t n, unsigned int* __restrict__ hist) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t r = crad[v];
        if (r) atomicAdd(&hist[r], 1u);
    }
}

__global__ void ws_volumes(const uint32_t* __restrict__ claim, const uint32_t* __restrict__ ext, size_t n,
                           unsigned long long* __restrict__ pvol, uint8_t* __restrict__ shared_flag) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t c = claim[v];
        const bool sh = ext[v] != 0;
        shared_flag[v] = sh;
        if (c && !sh) atomicAdd(&pvol[c - 1], 1ull);
    }
}

__global__ void ws_gather_shared(const uint32_t* __restrict__ sv, size_t ns, const uint32_t* __restrict__ claim,
                                 const uint32_t* __restrict__ ext, const uint32_t* __restrict__ ext_pore,
                                 const unsigned long long* __restrict__ ext_time, uint32_t* __restrict__ oc,
                                 uint32_t* __restrict__ op, unsigned long long* __restrict__ ot) {
    PMA_GRID_STRIDE(i, ns) {
        const uint32_t v = sv[i];
        oc[i] = claim[v];
        const uint32_t rec = ext[v] - 1;
        for (int k = 0; k < kSlots; ++k) {
            op[i * kSlots + k] = ext_pore[static_cast<size_t>(rec) * kSlots + k];
            ot[i * kSlots + k] = ext_time[static_cast<size_t>(rec) * kSlots + k];
        }
    }
}

__global__ void ws_labels(const uint32_t* __restrict__ claim, size_t n, const uint32_t* __restrict__ pore_id,
                          uint32_t* __restrict__ labels) {
    PMA_GRID_STRIDE(v, n) {
        const uint32_t c = claim[v];
        labels[v] = c ? pore_id[c - 1] : 0u;
    }
}

__global__ void ws_shared_labels(const uint32_t* __restrict__ sv, const uint32_t* __restrict__ id, size_t ns,
                                 uint32_t* __restrict__ labels) {
    PMA_GRID_STRIDE(i, ns) labels[sv[i]] = id[i];
}

template <class T>
T* buf(pma_ctx* ctx, const char* tag, size_t count) {
    return static_cast<T*>(ctx->scratch(tag, std::max<size_t>(count, 1) * sizeof(T)));
}

template <class Pred>
int64_t select_seqs(pma_ctx* ctx, Pred pred, const uint32_t* in_or_null, uint32_t* out, int64_t n,
                    int64_t* d_count) {
    size_t bytes = 0;
    if (in_or_null) {
        PMA_CUDA(cub::DeviceSelect::If(nullptr, bytes, in_or_null, out, d_count, n, pred, ctx->stream));
        void* tmp = ctx->scratch("cub.tmp", bytes);
        PMA_CUDA(cub::DeviceSelect::If(tmp, bytes, in_or_null, out, d_count, n, pred, ctx->stream));
    } else {
        thrust::counting_iterator<uint32_t> it(0);
        PMA_CUDA(cub::DeviceSelect::If(nullptr, bytes, it, out, d_count, n, pred, ctx->stream));
        void* tmp = ctx->scratch("cub.tmp", bytes);
        PMA_CUDA(cub::DeviceSelect::If(tmp, bytes, it, out, d_count, n, pred, ctx->stream));
    }
    int64_t h = 0;
    PMA_CUDA(cudaMemcpyAsync(&h, d_count, 8, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->count_launch(1);
    return h;
}

}  // namespace

pma_table* watershed(pma_ctx* ctx, const pma_table* pt, const uint32_t* crad2, pma_dims d,
                     pma_stencil st, uint32_t max_edt2, uint32_t* labels) {
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
        PMA_REQUIRE(p.seed_r2 <= max_edt2, PMA_ERR_ARGUMENT,
                    "pma_watershed: pore seed radius above max_edt2");
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
    WsState ws;
    ws.g = g;
    ws.d3q7 = st == PMA_D3Q7 ? 1 : 0;
    ws.crad = crad2;
    ws.claim = buf<uint32_t>(ctx, "ws.claim", n);
    ws.ckey = buf<unsigned long long>(ctx, "ws.ckey", n);
    ws.ext = buf<uint32_t>(ctx, "ws.ext", n);
    ws.ext_cap = static_cast<uint32_t>(std::min<size_t>(std::max<size_t>(n / 8, 4096), 0x7FFFFFFF / kSlots));
    ws.ext_pore = buf<uint32_t>(ctx, "ws.ext_pore", static_cast<size_t>(ws.ext_cap) * kSlots);
    ws.ext_time = buf<unsigned long long>(ctx, "ws.ext_time", static_cast<size_t>(ws.ext_cap) * kSlots);
    ws.ext_count = reinterpret_cast<unsigned int*>(d_count + 1);
    ws.err = reinterpret_cast<unsigned int*>(d_count + 2);
    ws.pbound = buf<unsigned int>(ctx, "ws.pbound", npores);
    PMA_CUDA(cudaMemsetAsync(d_count, 0, 32, s));
    PMA_CUDA(cudaMemsetAsync(ws.ext_pore, 0xFF, static_cast<size_t>(ws.ext_cap) * kSlots * 4, s));
    PMA_CUDA(cudaMemsetAsync(ws.ext_time, 0xFF, static_cast<size_t>(ws.ext_cap) * kSlots * 8, s));
    PMA_CUDA(cudaMemsetAsync(ws.pbound, 0, std::max<size_t>(npores, 1) * 4, s));
    ws_init<<<G, 256, 0, s>>>(n, ws.claim, ws.ckey, ws.ext);
    ctx->check_launch("ws_init");

    // Buckets: capacity = voxels of that crad + seeds of that radius.
    unsigned int* hist = buf<unsigned int>(ctx, "ws.hist", nb);
    PMA_CUDA(cudaMemsetAsync(hist, 0, nb * 4ull, s));
    ws_histograms<<<G, 256, 0, s>>>(crad2, n, hist);
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
    unsigned int* bfill = buf<unsigned int>(ctx, "ws.bfill", nb);
    auto* ent_time = buf<unsigned long long>(ctx, "ws.ent_time", total);
    auto* ent_val = buf<unsigned long long>(ctx, "ws.ent_val", total);
    auto* srt_time = buf<unsigned long long>(ctx, "ws.srt_time", max_bucket);
    auto* srt_val = buf<unsigned long long>(ctx, "ws.srt_val", max_bucket);
    PMA_CUDA(cudaMemcpyAsync(d_boff, boff.data(), (nb + 1) * 8ull, cudaMemcpyHostToDevice, s));
    // Seeds first in their bucket, in pore-id order (time = pore index).
    std::vector<unsigned int> h_fill(nb, 0);
    if (npores) {
        std::vector<unsigned long long> at(npores), tv(npores), vv(npores);
        for (size_t k = 0; k < npores; ++k) {
            const uint32_t b = pores[k].seed_r2;
            at[k] = boff[b] + h_fill[b]++;
            tv[k] = k;
            vv[k] = (static_cast<unsigned long long>(k) << 32) | seed_voxel[k];
        }
        auto* d_at = buf<unsigned long long>(ctx, "ws.seed_at", 3 * npores);
        PMA_CUDA(cudaMemcpyAsync(d_at, at.data(), npores * 8, cudaMemcpyHostToDevice, s));
        PMA_CUDA(cudaMemcpyAsync(d_at + npores, tv.data(), npores * 8, cudaMemcpyHostToDevice, s));
        PMA_CUDA(cudaMemcpyAsync(d_at + 2 * npores, vv.data(), npores * 8, cudaMemcpyHostToDevice, s));
        ws_seed_entries<<<grid_for(ctx, npores), 256, 0, s>>>(d_at, npores, ent_time, ent_val);
        ctx->check_launch("ws_seed_entries");
    }
    PMA_CUDA(cudaMemcpyAsync(bfill, h_fill.data(), nb * 4ull, cudaMemcpyHostToDevice, s));
    ctx->sync();
    if (npores) {
        uint32_t* d_seed = buf<uint32_t>(ctx, "ws.seedvox", npores);
        PMA_CUDA(cudaMemcpyAsync(d_seed, seed_voxel.data(), npores * 4, cudaMemcpyHostToDevice, s));
        ws_seed<<<grid_for(ctx, npores), 256, 0, s>>>(d_seed, npores, ws.claim);
        ctx->check_launch("ws_seed");
    }

    // Depth sweep (WatershedComputer.cpp:80-102).
    uint32_t* gv = buf<uint32_t>(ctx, "ws.gv", max_bucket);
    uint32_t* gpv = buf<uint32_t>(ctx, "ws.gp", max_bucket);
    uint32_t* nv = buf<uint32_t>(ctx, "ws.nv", max_bucket);
    uint32_t* npv = buf<uint32_t>(ctx, "ws.np", max_bucket);
    unsigned long long gen = 0;
    std::vector<unsigned int> cur_fill(1);
    for (int64_t depth = static_cast<int64_t>(nb) - 1; depth >= 0; --depth) {
        const unsigned long long cap = boff[depth + 1] - boff[depth];
        if (cap == 0) continue;
        PMA_CUDA(cudaMemcpyAsync(cur_fill.data(), bfill + depth, 4, cudaMemcpyDeviceToHost, s));
        ctx->sync();
        size_t ng = cur_fill[0];
        if (ng == 0) continue;
        // generation 0: the bucket's entries in time order
        sort_pairs(ctx, ent_time + boff[depth], srt_time, ent_val + boff[depth], srt_val,
                   static_cast<int64_t>(ng));
        ws_unpack_entries<<<grid_for(ctx, ng), 256, 0, s>>>(srt_val, ng, gv, gpv);
        ctx->check_launch("ws_unpack_entries");
        while (ng > 0) {
            ++gen;
            const size_t nev = ng * 27;
            uint32_t* slot_voxel = buf<uint32_t>(ctx, "ws.slots", nev);
            uint32_t* claimed = buf<uint32_t>(ctx, "ws.claimed", nev);
            PMA_CUDA(cudaMemsetAsync(slot_voxel, 0xFF, nev * 4, s));
            const unsigned tg = grid_for(ctx, ng, 128);
            KernelTimer kt(ctx, "ws_touch");
            ws_touch<0><<<tg, 128, 0, s>>>(ws, gv, gpv, ng, static_cast<uint32_t>(depth), gen, slot_voxel);
            ws_touch<1><<<tg, 128, 0, s>>>(ws, gv, gpv, ng, static_cast<uint32_t>(depth), gen, slot_voxel);
            ws_touch<2><<<tg, 128, 0, s>>>(ws, gv, gpv, ng, static_cast<uint32_t>(depth), gen, slot_voxel);
            ctx->count_launch(2);
            ctx->check_launch("ws_touch");
            const int64_t nc = select_seqs(ctx, SlotTaken{slot_voxel}, nullptr, claimed,
                                           static_cast<int64_t>(nev), d_count);
            if (nc == 0) break;
            ws_distribute<<<grid_for(ctx, nc), 256, 0, s>>>(claimed, nc, slot_voxel, gpv, crad2,
                                                            static_cast<uint32_t>(depth), gen, d_boff,
                                                            bfill, ent_time, ent_val);
            ctx->check_launch("ws_distribute");
            uint32_t* same = buf<uint32_t>(ctx, "ws.same", nc);
            const int64_t ns = select_seqs(ctx, AtDepth{slot_voxel, crad2, static_cast<uint32_t>(depth)},
                                           claimed, same, nc, d_count);
            if (ns) {
                ws_next_generation<<<grid_for(ctx, ns), 256, 0, s>>>(same, ns, slot_voxel, gpv, nv, npv);
                ctx->check_launch("ws_next_generation");
            }
            std::swap(gv, nv);
            std::swap(gpv, npv);
            ng = static_cast<size_t>(ns);
        }
    }
    unsigned int h_err = 0;
    PMA_CUDA(cudaMemcpyAsync(&h_err, ws.err, 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    PMA_REQUIRE(!(h_err & 1u), PMA_ERR_MEMORY, "pma_watershed: shared-voxel records exhausted");
    PMA_REQUIRE(!(h_err & 2u), PMA_ERR_LIMIT, "pma_watershed: more than 7 pores touch one voxel");

    // Volumes and shared voxels.
    auto* pvol = buf<unsigned long long>(ctx, "ws.pvol", npores);
    uint8_t* shared_flag = buf<uint8_t>(ctx, "ws.shared_flag", n);
    PMA_CUDA(cudaMemsetAsync(pvol, 0, std::max<size_t>(npores, 1) * 8, s));
    ws_volumes<<<G, 256, 0, s>>>(ws.claim, ws.ext, n, pvol, shared_flag);
    ctx->check_launch("ws_volumes");
    uint32_t* sv = buf<uint32_t>(ctx, "ws.sv", n);
    const int64_t nsh = select_flagged(ctx, thrust::counting_iterator<uint32_t>(0), shared_flag, sv,
                                       static_cast<int64_t>(n), d_count);
    std::vector<uint32_t> h_claim(nsh), h_pore(nsh * kSlots);
    std::vector<unsigned long long> h_time(nsh * kSlots);
    if (nsh) {
        uint32_t* oc = buf<uint32_t>(ctx, "ws.oc", nsh);
        uint32_t* op = buf<uint32_t>(ctx, "ws.op", nsh * kSlots);
        auto* ot = buf<unsigned long long>(ctx, "ws.ot", nsh * kSlots);
        ws_gather_shared<<<grid_for(ctx, nsh), 256, 0, s>>>(sv, nsh, ws.claim, ws.ext, ws.ext_pore,
                                                            ws.ext_time, oc, op, ot);
        ctx->check_launch("ws_gather_shared");
        PMA_CUDA(cudaMemcpyAsync(h_claim.data(), oc, nsh * 4, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(h_pore.data(), op, nsh * kSlots * 4, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(h_time.data(), ot, nsh * kSlots * 8, cudaMemcpyDeviceToHost, s));
    }
    std::vector<unsigned long long> h_pvol(npores);
    std::vector<unsigned int> h_pbound(npores);
    if (npores) {
        PMA_CUDA(cudaMemcpyAsync(h_pvol.data(), pvol, npores * 8, cudaMemcpyDeviceToHost, s));
        PMA_CUDA(cudaMemcpyAsync(h_pbound.data(), ws.pbound, npores * 4, cudaMemcpyDeviceToHost, s));
    }
    ctx->sync();

    // Keys of shared voxels and their creation times (host; shared voxels are few).
    struct KeyInfo {
        unsigned long long created = kNoTime;
        unsigned long long volume = 0;
    };
    std::map<std::vector<uint32_t>, KeyInfo> keys;
    std::vector<const std::vector<uint32_t>*> final_key(nsh);
    std::vector<std::pair<unsigned long long, uint32_t>> ext;
    for (int64_t i = 0; i < nsh; ++i) {
        ext.clear();
        for (int k = 0; k < kSlots; ++k) {
            const uint32_t p = h_pore[i * kSlots + k];
            if (p != kNone) ext.push_back({h_time[i * kSlots + k], p});
        }
        std::sort(ext.begin(), ext.end());
        std::vector<uint32_t> key;
        key.push_back(pores[ext[0].second].id);
        key.push_back(pores[h_claim[i] - 1].id);
        auto it = keys.emplace(key, KeyInfo()).first;
        it->second.created = std::min(it->second.created, ext[0].first);
        for (size_t k = 1; k < ext.size(); ++k) {
            key.push_back(pores[ext[k].second].id);
            it = keys.emplace(key, KeyInfo()).first;
            it->second.created = std::min(it->second.created, ext[k].first);
        }
        it->second.volume++;
        final_key[i] = &it->first;
    }
    std::vector<std::pair<unsigned long long, const std::vector<uint32_t>*>> by_time;
    for (auto& kv : keys) by_time.push_back({kv.second.created, &kv.first});
    std::sort(by_time.begin(), by_time.end());
    std::map<const std::vector<uint32_t>*, uint32_t> key_id;
    for (size_t k = 0; k < by_time.size(); ++k)
        key_id[by_time[k].second] = 0xFFFFFFFFu - 1u - static_cast<uint32_t>(k);

    // Labels.
    std::vector<uint32_t> pore_id(std::max<size_t>(npores, 1));
    for (size_t k = 0; k < npores; ++k) pore_id[k] = pores[k].id;
    uint32_t* d_pid = buf<uint32_t>(ctx, "ws.pid", pore_id.size());
    PMA_CUDA(cudaMemcpyAsync(d_pid, pore_id.data(), pore_id.size() * 4, cudaMemcpyHostToDevice, s));
    ws_labels<<<G, 256, 0, s>>>(ws.claim, n, d_pid, labels);
    ctx->check_launch("ws_labels");
    if (nsh) {
        std::vector<uint32_t> sid(nsh);
        for (int64_t i = 0; i < nsh; ++i) sid[i] = key_id[final_key[i]];
        uint32_t* d_sid = buf<uint32_t>(ctx, "ws.sid", nsh);
        PMA_CUDA(cudaMemcpyAsync(d_sid, sid.data(), nsh * 4, cudaMemcpyHostToDevice, s));
        ws_shared_labels<<<grid_for(ctx, nsh), 256, 0, s>>>(sv, d_sid, nsh, labels);
        ctx->check_launch("ws_shared_labels");
    }
    ctx->sync();

    pma_table* t = new pma_table;
    for (size_t k = 0; k < npores; ++k) {
        pma_pore p = pores[k];
        p.volume = h_pvol[k];
        p.is_boundary = h_pbound[k] ? 1 : 0;
        t->pores.push_back(p);
    }
    std::vector<std::pair<uint32_t, const std::vector<uint32_t>*>> rows;
    for (auto& kv : key_id) rows.push_back({kv.second, kv.first});
    std::sort(rows.begin(), rows.end(),
              [](const std::pair<uint32_t, const std::vector<uint32_t>*>& a,
                 const std::pair<uint32_t, const std::vector<uint32_t>*>& b) { return a.first < b.first; });
    for (auto& r : rows) {
        pma_throat th;
        th.id = r.first;
        th.n_pores = static_cast<uint32_t>(r.second->size());
        th.volume = keys[*r.second].volume;
        th.pool_offset = t->pool.size();
        t->pool.insert(t->pool.end(), r.second->begin(), r.second->end());
        t->throats.push_back(th);
    }
    return t;
}

}  // namespace pma
