// CPU oracle for the pore-throat and shortest-path pipeline of PorousMediaAnalysis.
//
// TEST INFRASTRUCTURE ONLY: a sequential restatement of the reference services, used as
// the checker for the CUDA product path. Each function names the reference file:line it
// follows. Semantics are those of the reference run with "Number of threads: 1" and one
// active area covering the whole image (enough "Available memory in megabytes").
//
// Layout: [z][x][y], linear index (z*SX + x)*SY + y (DataArray.h:85-94).

#include "pma_oracle.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <stack>
#include <vector>

namespace {

struct Dims {
    int sx, sy, sz;
    size_t idx(int x, int y, int z) const {
        return (static_cast<size_t>(z) * sx + x) * static_cast<size_t>(sy) + y;
    }
    size_t count() const { return static_cast<size_t>(sx) * sy * sz; }
    bool outside(int x, int y, int z) const {  // ModelUtilities.h:309-316
        return x < 0 || x >= sx || y < 0 || y >= sy || z < 0 || z >= sz;
    }
};

// ModelUtilities.h:295-302: a neighbour differs from the centre in two or more axes.
inline bool is_diagonal(int cx, int cy, int cz, int nx, int ny, int nz) {
    return (nx != cx && ny != cy) || (nx != cx && nz != cz) || (ny != cy && nz != cz);
}

typedef std::array<int, 3> Pos;

}  // namespace

// ----------------------------------------------------------------------------------------
// a1-a4: EuclideanDistanceComputer.cpp
// ----------------------------------------------------------------------------------------
extern "C" int orc_edt(const uint8_t* solid, int sx, int sy, int sz, uint32_t* edt2,
                       uint32_t* max_edt2, uint64_t* hist, size_t hist_cap, size_t* hist_len) {
    if (sx <= 0 || sy <= 0 || sz <= 0) return -1;
    Dims d{sx, sy, sz};

    // a1, EDC.cpp:149-202. Forward then backward scan along X. The running distance
    // starts at SX-1 because BOUNDARIES_ARE_SOLID is false (EDC.h:30, EDC.cpp:164,180).
    for (int y = 0; y < sy; ++y) {
        for (int z = 0; z < sz; ++z) {
            uint32_t run = static_cast<uint32_t>(sx - 1);
            for (int x = 0; x < sx; ++x) {
                run = solid[d.idx(x, y, z)] == 0 ? run + 1 : 0;
                edt2[d.idx(x, y, z)] = run * run;
            }
            run = static_cast<uint32_t>(sx - 1);
            for (int x = sx - 1; x >= 0; --x) {
                run = solid[d.idx(x, y, z)] == 0 ? run + 1 : 0;
                uint32_t back = run * run;
                if (back < edt2[d.idx(x, y, z)]) edt2[d.idx(x, y, z)] = back;
            }
        }
    }

    // a2, EDC.cpp:204-250. Windowed minimum along Y with half-width int(sqrt(g)+1).
    std::vector<uint32_t> line(std::max(sy, sz));
    for (int x = 0; x < sx; ++x) {
        for (int z = 0; z < sz; ++z) {
            for (int y = 0; y < sy; ++y) line[y] = edt2[d.idx(x, y, z)];
            for (int y = 0; y < sy; ++y) {
                uint32_t best = line[y];
                if (best == 0) continue;
                int half = static_cast<int>(std::sqrt(static_cast<double>(best)) + 1);
                int lo = std::min(half, y);
                int hi = std::min(half, sy - y);
                for (int dy = -lo; dy < hi; ++dy) {
                    uint32_t cand = line[y + dy] + static_cast<uint32_t>(dy * dy);
                    if (cand < best) best = cand;
                }
                edt2[d.idx(x, y, z)] = best;
            }
        }
    }

    // a3, EDC.cpp:253-343. Windowed minimum along Z, running maximum and the histogram of
    // balls that do not cross the image boundary (double sqrt comparisons, :316-327).
    uint32_t maxv = 0;
    std::vector<uint64_t> counts(1, 0);
    for (int x = 0; x < sx; ++x) {
        for (int y = 0; y < sy; ++y) {
            for (int z = 0; z < sz; ++z) line[z] = edt2[d.idx(x, y, z)];
            for (int z = 0; z < sz; ++z) {
                uint32_t best = line[z];
                if (best == 0) continue;
                int half = static_cast<int>(std::sqrt(static_cast<double>(best)) + 1);
                int lo = std::min(half, z);
                int hi = std::min(half, sz - z);
                for (int dz = -lo; dz < hi; ++dz) {
                    uint32_t cand = line[z + dz] + static_cast<uint32_t>(dz * dz);
                    if (cand < best) best = cand;
                }
                edt2[d.idx(x, y, z)] = best;
                if (maxv < best) {
                    maxv = best;
                    counts.resize(static_cast<size_t>(maxv) + 1, 0);
                }
                double r = std::sqrt(static_cast<double>(best));
                bool crosses = r > x || r > y || r > z || (x + r > (sx - 1)) ||
                               (y + r > (sy - 1)) || (z + r > (sz - 1));
                if (!crosses) counts[best]++;
            }
        }
    }
    counts.resize(static_cast<size_t>(maxv) + 1, 0);
    *max_edt2 = maxv;
    *hist_len = counts.size();
    if (hist) {
        size_t n = std::min(hist_cap, counts.size());
        for (size_t i = 0; i < n; ++i) hist[i] = counts[i];
    }
    return 0;
}

// ----------------------------------------------------------------------------------------
// a5-a6: EuclideanDistanceDerivativesComputer.cpp:20-49 (float sqrt table) and
// ContainingBallsAssigner.cpp:101-183 (scatter, single-thread order x, y, z).
// ----------------------------------------------------------------------------------------
extern "C" int orc_containing_balls(const uint32_t* edt2, int sx, int sy, int sz,
                                    uint32_t max_edt2, uint32_t* crad2, uint32_t* cx,
                                    uint32_t* cy, uint32_t* cz) {
    Dims d{sx, sy, sz};
    const size_t n = d.count();
    // DataArraysGroup.cpp:21-25 defaults.
    std::fill(crad2, crad2 + n, 0u);
    std::fill(cx, cx + n, UINT_MAX);
    std::fill(cy, cy + n, UINT_MAX);
    std::fill(cz, cz + n, UINT_MAX);

    std::vector<float> root(static_cast<size_t>(max_edt2) + 1);
    for (uint32_t i = 0; i <= max_edt2; ++i) root[i] = std::sqrt(static_cast<float>(i));

    for (int x = 0; x < sx; ++x) {
        for (int y = 0; y < sy; ++y) {
            for (int z = 0; z < sz; ++z) {
                uint32_t r2 = edt2[d.idx(x, y, z)];
                if (r2 == 0) continue;
                int half = static_cast<int>(root[r2] + 1);  // CBA.cpp:142-143
                int x0 = std::max(0, x - half), x1 = std::min(sx - 1, x + half);
                int y0 = std::max(0, y - half), y1 = std::min(sy - 1, y + half);
                int z0 = std::max(0, z - half), z1 = std::min(sz - 1, z + half);
                for (int ix = x0; ix <= x1; ++ix) {
                    for (int iy = y0; iy <= y1; ++iy) {
                        for (int iz = z0; iz <= z1; ++iz) {
                            uint32_t dd = static_cast<uint32_t>((ix - x) * (ix - x) +
                                                                (iy - y) * (iy - y) +
                                                                (iz - z) * (iz - z));
                            if (dd > r2) continue;
                            size_t v = d.idx(ix, iy, iz);
                            if (edt2[v] == 0) continue;
                            if (crad2[v] < r2) {
                                crad2[v] = r2;
                                cx[v] = x;
                                cy[v] = y;
                                cz[v] = z;
                            }
                        }
                    }
                }
            }
        }
    }
    return 0;
}

// a7: ContainingBallsAssigner.cpp:190-250.
extern "C" int orc_max_ball_mask(const uint32_t* cx, const uint32_t* cy, const uint32_t* cz,
                                 int sx, int sy, int sz, uint8_t* mask, uint64_t* count) {
    Dims d{sx, sy, sz};
    for (size_t v = 0; v < d.count(); ++v) mask[v] = (cx[v] == UINT_MAX) ? 0 : 127;
    uint64_t c = 0;
    for (int x = 0; x < sx; ++x)
        for (int y = 0; y < sy; ++y)
            for (int z = 0; z < sz; ++z) {
                size_t v = d.idx(x, y, z);
                if (cx[v] == UINT_MAX) continue;
                size_t w = d.idx(cx[v], cy[v], cz[v]);
                if (mask[w] == 127) {
                    mask[w] = 255;
                    ++c;
                }
            }
    *count = c;
    return 0;
}

// ----------------------------------------------------------------------------------------
// Pores and throats: Types.h:157-195 (Pore, SharedPixelType, MaximumBall, comparer).
// ----------------------------------------------------------------------------------------
namespace {

struct Pore {
    uint32_t id;
    Pos seed;
    uint32_t seed_r2;
    size_t volume;
    bool boundary;
};

struct Throat {
    uint32_t id;
    std::vector<uint32_t> pores;
    size_t volume;
};

struct MaxBall {  // Types.h:182-186, same member layout as the reference
    Pos center;
    uint32_t r2;
};

struct MaxBallDescending {  // Types.h:188-195
    bool operator()(const MaxBall& a, const MaxBall& b) const { return a.r2 > b.r2; }
};

// Holds the maps of BasePoreAndThroatComputer (BasePoreAndThroatComputer.h) and the
// per-pixel state machine of BasePoreAndThroatComputer.cpp:37-133.
struct PoreState {
    uint32_t first_shared = UINT_MAX;  // BPTC.cpp:30
    std::map<uint32_t, Pore> pores;
    std::map<uint32_t, Throat> throats;
    std::map<std::vector<uint32_t>, uint32_t> throat_by_key;

    Throat* get_or_add(const std::vector<uint32_t>& key) {  // BPTC.cpp:112-133
        auto it = throat_by_key.find(key);
        if (it != throat_by_key.end()) return &throats[it->second];
        --first_shared;
        Throat& t = throats[first_shared];
        t.id = first_shared;
        t.volume = 0;
        t.pores = key;
        throat_by_key[key] = first_shared;
        return &t;
    }

    // BPTC.cpp:37-110. Returns "continue the propagation".
    bool update(uint32_t* labels, size_t v, Pore& pore, bool continue_after_shared) {
        uint32_t cur = labels[v];
        if (cur == pore.id) return false;
        if (cur == 0) {
            labels[v] = pore.id;
            pore.volume++;
            return true;
        }
        if (cur < first_shared) {
            std::vector<uint32_t> key{pore.id, cur};
            Throat* t = get_or_add(key);
            labels[v] = t->id;
            t->volume++;
            pores[cur].volume--;
            return continue_after_shared;
        }
        Throat& old = throats[cur];
        if (std::find(old.pores.begin(), old.pores.end(), pore.id) != old.pores.end())
            return false;
        std::vector<uint32_t> key = old.pores;
        key.push_back(pore.id);
        Throat* t = get_or_add(key);
        labels[v] = t->id;
        old.volume--;
        t->volume++;
        return continue_after_shared;
    }
};

}  // namespace

struct orc_table {
    std::vector<orc_pore> pores;
    std::vector<orc_throat> throats;
    std::vector<uint32_t> pool;
};

static orc_table* make_table(const std::map<uint32_t, Pore>& pores,
                             const std::map<uint32_t, Throat>& throats) {
    orc_table* t = new orc_table;
    for (const auto& kv : pores) {
        const Pore& p = kv.second;
        orc_pore o{p.id, p.seed[0], p.seed[1], p.seed[2], p.seed_r2, p.boundary ? 1 : 0,
                   static_cast<uint64_t>(p.volume)};
        t->pores.push_back(o);
    }
    for (const auto& kv : throats) {
        const Throat& th = kv.second;
        orc_throat o{th.id, static_cast<uint32_t>(th.pores.size()),
                     static_cast<uint64_t>(th.volume), static_cast<uint64_t>(t->pool.size())};
        t->throats.push_back(o);
        t->pool.insert(t->pool.end(), th.pores.begin(), th.pores.end());
    }
    return t;
}

static void table_to_maps(const orc_table* t, std::map<uint32_t, Pore>* pores,
                          std::map<uint32_t, Throat>* throats) {
    pores->clear();
    if (throats) throats->clear();
    for (const orc_pore& o : t->pores) {
        Pore p;
        p.id = o.id;
        p.seed = {o.seed_x, o.seed_y, o.seed_z};
        p.seed_r2 = o.seed_r2;
        p.volume = o.volume;
        p.boundary = o.is_boundary != 0;
        (*pores)[p.id] = p;
    }
    if (!throats) return;
    for (const orc_throat& o : t->throats) {
        Throat th;
        th.id = o.id;
        th.volume = o.volume;
        th.pores.assign(t->pool.begin() + o.pool_offset,
                        t->pool.begin() + o.pool_offset + o.n_pores);
        (*throats)[th.id] = th;
    }
}

// a8-a10: PoreAndThroatComputer.cpp:93-269.
extern "C" orc_table* orc_pores(const uint8_t* mask, const uint32_t* edt2,
                                const uint32_t* crad2, int sx, int sy, int sz, int d3q7,
                                uint32_t* labels) {
    Dims d{sx, sy, sz};
    // PTC.cpp:93-123: outer balls in z, x, y scan order, radius from the EDT, std::sort.
    std::vector<MaxBall> balls;
    for (int z = 0; z < sz; ++z)
        for (int x = 0; x < sx; ++x)
            for (int y = 0; y < sy; ++y) {
                size_t v = d.idx(x, y, z);
                if (mask[v] != 255) continue;
                MaxBall b;
                b.center = {x, y, z};
                b.r2 = edt2[v];
                balls.push_back(b);
            }
    std::sort(balls.begin(), balls.end(), MaxBallDescending());

    PoreState st;
    uint32_t pore_id = 127;  // PTC.cpp:60
    for (const MaxBall& b : balls) {  // PTC.cpp:125-163
        if (labels[d.idx(b.center[0], b.center[1], b.center[2])] != 0) continue;
        Pore& pore = st.pores[pore_id];
        pore.seed = b.center;
        pore.seed_r2 = b.r2;
        pore.id = pore_id;
        pore.volume = 0;
        pore.boundary = false;
        pore_id += (pore_id % 255 == 0) ? 127 : 1;

        // PTC.cpp:192-217: explicit-stack depth-first search.
        std::stack<Pos> todo;
        todo.push(pore.seed);
        while (!todo.empty()) {
            Pos node = todo.top();
            todo.pop();
            size_t nv = d.idx(node[0], node[1], node[2]);
            if (!st.update(labels, nv, pore, true)) continue;
            // PTC.cpp:219-269
            uint32_t node_r2 = crad2[nv];
            for (int nx = node[0] - 1; nx <= node[0] + 1; ++nx)
                for (int ny = node[1] - 1; ny <= node[1] + 1; ++ny)
                    for (int nz = node[2] - 1; nz <= node[2] + 1; ++nz) {
                        if (nx == node[0] && ny == node[1] && nz == node[2]) continue;
                        if (d3q7 && is_diagonal(node[0], node[1], node[2], nx, ny, nz)) continue;
                        if (d.outside(nx, ny, nz)) {
                            pore.boundary = true;
                            continue;
                        }
                        uint32_t r2 = crad2[d.idx(nx, ny, nz)];
                        if (r2 > 0 && r2 <= node_r2) todo.push(Pos{nx, ny, nz});
                    }
        }

        // PTC.cpp:168-189: drop shared types left with zero volume.
        std::vector<uint32_t> empty;
        for (const auto& kv : st.throats)
            if (kv.second.volume == 0) empty.push_back(kv.second.id);
        for (uint32_t id : empty) {
            st.throat_by_key.erase(st.throats[id].pores);
            st.throats.erase(id);
        }
    }
    return make_table(st.pores, st.throats);
}

// The std::sort order of a8 (PoreAndThroatComputer.cpp:93-123): writes the linear index of
// each maximum ball in sorted order; returns their number.
extern "C" size_t orc_sorted_balls(const uint8_t* mask, const uint32_t* edt2, int sx, int sy, int sz,
                                   uint32_t* out, size_t cap) {
    Dims d{sx, sy, sz};
    std::vector<MaxBall> balls;
    for (int z = 0; z < sz; ++z)
        for (int x = 0; x < sx; ++x)
            for (int y = 0; y < sy; ++y) {
                size_t v = d.idx(x, y, z);
                if (mask[v] != 255) continue;
                MaxBall b;
                b.center = {x, y, z};
                b.r2 = edt2[v];
                balls.push_back(b);
            }
    std::sort(balls.begin(), balls.end(), MaxBallDescending());
    for (size_t i = 0; i < balls.size() && i < cap; ++i)
        out[i] = static_cast<uint32_t>(d.idx(balls[i].center[0], balls[i].center[1], balls[i].center[2]));
    return balls.size();
}

// a11: EmptyPoresRemover.cpp:31-244.
extern "C" int orc_remove_empty_pores(orc_table* t, uint32_t* labels, int sx, int sy, int sz) {
    std::map<uint32_t, Pore> pores;
    std::map<uint32_t, Throat> throats;
    table_to_maps(t, &pores, &throats);
    std::map<uint32_t, uint32_t> remap;

    // EPR.cpp:193-244
    std::vector<uint32_t> empty;
    for (const auto& kv : pores)
        if (kv.second.volume == 0) empty.push_back(kv.second.id);
    for (uint32_t id : empty) pores.erase(id);
    std::sort(empty.begin(), empty.end());
    for (auto& kv : throats) {
        std::vector<uint32_t>& p = kv.second.pores;
        std::sort(p.begin(), p.end());
        std::vector<uint32_t> kept;
        std::set_difference(p.begin(), p.end(), empty.begin(), empty.end(),
                            std::back_inserter(kept));
        p = kept;
    }
    // EPR.cpp:167-191
    std::vector<uint32_t> few;
    for (const auto& kv : throats)
        if (kv.second.pores.size() < 2) few.push_back(kv.second.id);
    for (uint32_t id : few) {
        const Throat& th = throats[id];
        if (th.pores.size() == 1) remap[th.id] = th.pores[0];
        throats.erase(id);
    }
    // EPR.cpp:126-165
    std::map<std::vector<uint32_t>, std::vector<uint32_t>> ids_by_pores;
    for (const auto& kv : throats) ids_by_pores[kv.second.pores].push_back(kv.second.id);
    for (const auto& kv : ids_by_pores) {
        const std::vector<uint32_t>& ids = kv.second;
        if (ids.size() == 1) continue;
        uint32_t keep = *std::max_element(ids.begin(), ids.end());
        for (uint32_t id : ids)
            if (id != keep) {
                throats.erase(id);
                remap[id] = keep;
            }
    }

    orc_table* nt = make_table(pores, throats);
    t->pores.swap(nt->pores);
    t->throats.swap(nt->throats);
    t->pool.swap(nt->pool);
    delete nt;

    // EPR.cpp:74-99 (skipped entirely when the mapping is empty, :54-57).
    if (remap.empty()) return 0;
    Dims d{sx, sy, sz};
    for (size_t v = 0; v < d.count(); ++v) {
        if (labels[v] == 0) continue;
        auto it = remap.find(labels[v]);
        if (it != remap.end()) labels[v] = it->second;
    }
    return 0;
}

// a12: WatershedComputer.cpp:80-219.
extern "C" orc_table* orc_watershed(const orc_table* pores_after_removal, const uint32_t* crad2,
                                    int sx, int sy, int sz, int d3q7, uint32_t max_edt2,
                                    uint32_t* labels) {
    Dims d{sx, sy, sz};
    PoreState st;  // ClearCache, BPTC.cpp:22-28
    table_to_maps(pores_after_removal, &st.pores, nullptr);

    struct Node {
        Pos pos;
        uint32_t depth;
        Pore* pore;
    };
    std::vector<std::queue<Node>> buckets(static_cast<size_t>(max_edt2) + 1);
    for (auto& kv : st.pores) {  // WC.cpp:183-219
        Pore& p = kv.second;
        p.boundary = false;
        p.volume = 0;
        Node n{p.seed, p.seed_r2, &p};
        buckets[p.seed_r2].push(n);
        st.update(labels, d.idx(p.seed[0], p.seed[1], p.seed[2]), p, false);
    }
    for (int depth = static_cast<int>(buckets.size()) - 1; depth >= 0; --depth) {  // WC.cpp:80-102
        std::queue<Node>& q = buckets[depth];
        while (!q.empty()) {
            Node n = q.front();
            q.pop();
            for (int nx = n.pos[0] - 1; nx <= n.pos[0] + 1; ++nx)
                for (int ny = n.pos[1] - 1; ny <= n.pos[1] + 1; ++ny)
                    for (int nz = n.pos[2] - 1; nz <= n.pos[2] + 1; ++nz) {
                        if (nx == n.pos[0] && ny == n.pos[1] && nz == n.pos[2]) continue;
                        // WC.cpp:130-176
                        if (d3q7 && is_diagonal(n.pos[0], n.pos[1], n.pos[2], nx, ny, nz)) continue;
                        if (d.outside(nx, ny, nz)) {
                            n.pore->boundary = true;
                            continue;
                        }
                        size_t w = d.idx(nx, ny, nz);
                        uint32_t r2 = crad2[w];
                        if (r2 == 0 || r2 > n.depth) continue;
                        if (st.update(labels, w, *n.pore, false))
                            buckets[r2].push(Node{Pos{nx, ny, nz}, r2, n.pore});
                    }
        }
    }
    return make_table(st.pores, st.throats);
}

// A pores table from rows (a pores.txt read back, Serializer.cpp:104-128), for watershed runs
// on hand-made seeds.
extern "C" orc_table* orc_table_from_pores(const orc_pore* pores, size_t n) {
    orc_table* t = new orc_table;
    t->pores.assign(pores, pores + n);
    return t;
}

extern "C" size_t orc_table_npores(const orc_table* t) { return t->pores.size(); }
extern "C" const orc_pore* orc_table_pores(const orc_table* t) { return t->pores.data(); }
extern "C" size_t orc_table_nthroats(const orc_table* t) { return t->throats.size(); }
extern "C" const orc_throat* orc_table_throats(const orc_table* t) { return t->throats.data(); }
extern "C" size_t orc_table_pool_size(const orc_table* t) { return t->pool.size(); }
extern "C" const uint32_t* orc_table_pool(const orc_table* t) { return t->pool.data(); }
extern "C" void orc_table_free(orc_table* t) { delete t; }

// ----------------------------------------------------------------------------------------
// a13-a15: ShortestPathComputer.cpp. The reference keeps every voxel in an indexed binary
// heap (HeapUtilities.h:26-101) and settles the minimum each step. Here the same Dijkstra
// runs on a lazy-deletion binary heap. Settled distances do not depend on the heap's tie
// order: each equals min over void neighbours u of fl(d(u) + w), the unique fixed point
// reached from above, so both heaps give identical bits.
// ----------------------------------------------------------------------------------------
namespace {

template <class T>
struct Geodesic {
    Dims d{0, 0, 0};
    bool d3q7 = false;
    const uint8_t* solid = nullptr;
    T* dist = nullptr;
    uint32_t* cavity = nullptr;
    T unknown = std::numeric_limits<T>::max();  // Constants.h:266
    T step[4];
    std::vector<char> settled;
    std::vector<std::pair<int, int>> walls_reached;  // (axis, coordinate)
    size_t processed = 0;

    Pos center() const {  // SPC.cpp:443-453 with Math::Round (Math.h:29-39)
        int s[3] = {d.sx, d.sy, d.sz};
        Pos c;
        for (int i = 0; i < 3; ++i) {
            double h = s[i] * 0.5;
            int r = static_cast<int>(h + 0.5);
            c[i] = std::min(r, s[i] - 1);
        }
        return c;
    }

    bool is_void(const Pos& p) const { return solid[d.idx(p[0], p[1], p[2])] == 0; }
    bool unreached(const Pos& p) const { return dist[d.idx(p[0], p[1], p[2])] == unknown; }

    int walls_count() const {  // SPC.cpp:229-261
        int s[3] = {d.sx, d.sy, d.sz};
        int n = 0;
        for (int i = 0; i < 3; ++i) n += (s[i] - 1 == 0) ? 1 : 2;
        return n;
    }

    // SPC.cpp:460-511
    bool find_on_shell(const Pos& c, int h, Pos* out) const {
        int s[3] = {d.sx, d.sy, d.sz};
        for (int k = 0; k < 3; ++k) {
            int a = (k == 0) ? 1 : 0;
            int b = (k == 2) ? 1 : 2;
            int a0 = std::max(c[a] - h, 0), a1 = std::min(c[a] + h, s[a] - 1);
            int b0 = std::max(c[b] - h, 0), b1 = std::min(c[b] + h, s[b] - 1);
            int fixed[2] = {std::max(c[k] - h, 0), std::min(c[k] + h, s[k] - 1)};
            int nfixed = (fixed[0] == fixed[1]) ? 1 : 2;
            for (int f = 0; f < nfixed; ++f)
                for (int i = a0; i <= a1; ++i)
                    for (int j = b0; j <= b1; ++j) {
                        Pos p;
                        p[a] = i;
                        p[b] = j;
                        p[k] = fixed[f];
                        if (is_void(p) && unreached(p)) {
                            *out = p;
                            return true;
                        }
                    }
        }
        return false;
    }

    // SPC.cpp:396-441
    bool select_start(Pos* out, int* half) const {
        Pos c = center();
        if (is_void(c) && unreached(c)) {
            *out = c;
            return true;
        }
        int s[3] = {d.sx, d.sy, d.sz};
        int maxh = 0;
        for (int i = 0; i < 3; ++i) maxh = std::max(maxh, std::max(s[i] - 1 - c[i], c[i]));
        for (*half = *half; *half < maxh; ++*half)
            if (find_on_shell(c, *half, out)) return true;
        return false;
    }

    void note_walls(const Pos& p) {  // SPC.cpp:210-227
        int s[3] = {d.sx, d.sy, d.sz};
        for (int i = 0; i < 3; ++i)
            if (p[i] == 0 || p[i] == s[i] - 1) {
                std::pair<int, int> w(i, p[i]);
                if (std::find(walls_reached.begin(), walls_reached.end(), w) == walls_reached.end())
                    walls_reached.push_back(w);
            }
    }

    // SPC.cpp:167-208 and :263-337
    void dijkstra(const Pos& start, uint32_t cavity_id) {
        typedef std::pair<T, size_t> Item;
        std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
        size_t s0 = d.idx(start[0], start[1], start[2]);
        dist[s0] = 0;
        heap.push(Item(0, s0));
        while (!heap.empty()) {
            Item it = heap.top();
            heap.pop();
            size_t v = it.second;
            if (settled[v] || it.first != dist[v]) continue;
            settled[v] = 1;
            cavity[v] = cavity_id;
            ++processed;
            int z = static_cast<int>(v / (static_cast<size_t>(d.sx) * d.sy));
            int rem = static_cast<int>(v % (static_cast<size_t>(d.sx) * d.sy));
            int x = rem / d.sy, y = rem % d.sy;
            note_walls(Pos{x, y, z});
            T dv = dist[v];
            for (int nx = x - 1; nx <= x + 1; ++nx)
                for (int ny = y - 1; ny <= y + 1; ++ny)
                    for (int nz = z - 1; nz <= z + 1; ++nz) {
                        if (nx == x && ny == y && nz == z) continue;
                        if (d3q7 && is_diagonal(x, y, z, nx, ny, nz)) continue;
                        if (d.outside(nx, ny, nz)) continue;
                        size_t w = d.idx(nx, ny, nz);
                        if (solid[w] != 0) continue;
                        int k = std::abs(nx - x) + std::abs(ny - y) + std::abs(nz - z);
                        T nd = dv + (d3q7 ? static_cast<T>(1.0) : step[k]);
                        if (nd < dist[w]) {
                            dist[w] = nd;
                            heap.push(Item(nd, w));
                        }
                    }
        }
    }

    int run(orc_cavity* cav, int cav_cap) {
        const size_t n = d.count();
        for (int k = 0; k < 4; ++k) step[k] = std::sqrt(static_cast<T>(k));  // SPC.cpp:31-36
        settled.assign(n, 0);
        for (size_t v = 0; v < n; ++v) {  // SPC.cpp:339-383
            bool s = solid[v] != 0;
            dist[v] = s ? static_cast<T>(-1) : unknown;
            cavity[v] = s ? 0u : UINT_MAX;
            if (s) settled[v] = 1;
        }
        int half = 0;
        int walls = walls_count();
        uint32_t cavity_id = 0;
        size_t previous = 0;
        int ncav = 0;
        Pos c = center();
        while (true) {  // SPC.cpp:78-141
            Pos start;
            ++half;
            if (!select_start(&start, &half)) break;
            walls_reached.clear();
            cavity_id += 127;
            dijkstra(start, cavity_id);
            if (ncav < cav_cap && cav) {  // SPC.cpp:143-164 (every cavity is counted)
                orc_cavity& o = cav[ncav];
                std::memset(&o, 0, sizeof(o));
                o.id = cavity_id;
                o.seed_x = start[0];
                o.seed_y = start[1];
                o.seed_z = start[2];
                o.reached_walls = static_cast<int32_t>(walls_reached.size());
                o.reaches_all_walls = static_cast<int>(walls_reached.size()) == walls ? 1 : 0;
                o.void_count = processed - previous;
                int dx = start[0] - c[0], dy = start[1] - c[1], dz = start[2] - c[2];
                o.distance_to_center =
                    static_cast<float>(std::sqrt(static_cast<double>(dx * dx + dy * dy + dz * dz)));
            }
            ++ncav;
            previous = processed;
            if (static_cast<int>(walls_reached.size()) == walls) break;
        }
        return ncav;  // the number of cavities; rows beyond cav_cap are not stored
    }
};

}  // namespace

extern "C" int orc_geodesic_f32(const uint8_t* solid, int sx, int sy, int sz, int d3q7,
                                float* dist, uint32_t* cavity, orc_cavity* cav, int cav_cap) {
    if (sx <= 0 || sy <= 0 || sz <= 0) return -1;
    Geodesic<float> g;
    g.d = Dims{sx, sy, sz};
    g.d3q7 = d3q7 != 0;
    g.solid = solid;
    g.dist = dist;
    g.cavity = cavity;
    return g.run(cav, cav_cap);
}

extern "C" int orc_geodesic_f64(const uint8_t* solid, int sx, int sy, int sz, int d3q7,
                                double* dist, uint32_t* cavity, orc_cavity* cav, int cav_cap) {
    if (sx <= 0 || sy <= 0 || sz <= 0) return -1;
    Geodesic<double> g;
    g.d = Dims{sx, sy, sz};
    g.d3q7 = d3q7 != 0;
    g.solid = solid;
    g.dist = dist;
    g.cavity = cavity;
    return g.run(cav, cav_cap);
}
