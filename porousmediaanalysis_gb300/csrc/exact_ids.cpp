// Shared-type ids of the initial pore propagation in the reference's own numbering
// (PoreAndThroatComputer.cpp:125-269, BasePoreAndThroatComputer.cpp:37-133).
//
// The reference runs one depth-first search per pore, in pore order, and gives a shared
// type the next id (counting down from UINT32_MAX - 1) at the first voxel where its pore-id
// key appears. Keys of types that later lose all their voxels also consumed ids (the types
// are deleted after each pore, :155-189), so the ids of the surviving types depend on the
// creation order of every key ever formed.
//
// Replay. A pore's search visits exactly its reach set (the voxels reachable from its seed
// along stencil steps of non-increasing containing radius), whatever earlier pores did: a
// visit stops only where the voxel already holds this pore. So the visit order of each
// pore's search is a function of the radii and the seed alone, and the searches can run
// independently (one host thread per pore at a time). At a visited voxel whose final pore
// set is q1 < q2 < ... < qk (pore ids, i.e. processing order) and whose pore X = qj, j >= 2,
// the key formed is the prefix [q2, q1, q3, ..., qj]; it is formed only during qj's search,
// so its creation time is (qj, the rank of its first formation in qj's search). All keys
// are prefixes of the final keys: they are the nodes of a trie over the final pore lists.
// A search stops as soon as every key its pore creates has been seen.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <system_error>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pma_internal.h"

namespace pma {
namespace {

struct Box {  // [z][x][y] volume geometry, y fastest
    int SX, SY, SZ;
    size_t idx(int x, int y, int z) const { return (static_cast<size_t>(z) * SX + x) * SY + y; }
    void coords(uint32_t v, int& x, int& y, int& z) const {
        const uint32_t zx = v / static_cast<uint32_t>(SY);
        y = static_cast<int>(v - zx * static_cast<uint32_t>(SY));
        z = static_cast<int>(zx / static_cast<uint32_t>(SX));
        x = static_cast<int>(zx - static_cast<uint32_t>(z) * static_cast<uint32_t>(SX));
    }
    bool inside(int x, int y, int z) const { return x >= 0 && x < SX && y >= 0 && y < SY && z >= 0 && z < SZ; }
};

}  // namespace

std::vector<uint32_t> replay_type_ids(const uint32_t* crad, const uint32_t* labels, pma_dims d, bool d3q7,
                                      const std::vector<pma_pore>& pores,
                                      const std::vector<std::vector<uint32_t>>& lists,
                                      const std::vector<uint32_t>& fast_ids) {
    const size_t ng = lists.size();
    const size_t npores = pores.size();
    std::vector<uint32_t> pore_ids(npores);
    for (size_t k = 0; k < npores; ++k) pore_ids[k] = pores[k].id;
    PMA_REQUIRE(std::is_sorted(pore_ids.begin(), pore_ids.end()), PMA_ERR_INTERNAL,
                "exact type ids: pores are not in id order");
    auto pore_index = [&](uint32_t id) -> int64_t {
        auto it = std::lower_bound(pore_ids.begin(), pore_ids.end(), id);
        return (it != pore_ids.end() && *it == id) ? it - pore_ids.begin() : -1;
    };

    // Trie of the sorted pore lists: node per prefix of length >= 2, its creator (the prefix's
    // last pore) and, per list, the node of each prefix length.
    std::unordered_map<unsigned long long, uint32_t> child;
    std::vector<uint32_t> node_creator;  // pore index
    std::vector<std::vector<uint32_t>> path(ng);  // path[g][j] = node of prefix length j + 1 (j >= 1)
    std::vector<uint32_t> first_node(npores, 0xFFFFFFFFu);  // depth-1 pseudo nodes per pore
    uint32_t pseudo = 0;
    for (size_t g = 0; g < ng; ++g) {
        const std::vector<uint32_t>& L = lists[g];
        PMA_REQUIRE(L.size() >= 2, PMA_ERR_INTERNAL, "exact type ids: a type with fewer than two pores");
        path[g].assign(L.size(), 0xFFFFFFFFu);
        const int64_t p0 = pore_index(L[0]);
        PMA_REQUIRE(p0 >= 0, PMA_ERR_INTERNAL, "exact type ids: unknown pore in a type");
        if (first_node[p0] == 0xFFFFFFFFu) first_node[p0] = 0x80000000u | pseudo++;
        uint32_t cur = first_node[p0];
        for (size_t j = 1; j < L.size(); ++j) {
            const int64_t pj = pore_index(L[j]);
            PMA_REQUIRE(pj >= 0 && L[j] > L[j - 1], PMA_ERR_INTERNAL, "exact type ids: bad pore list");
            const unsigned long long key = (static_cast<unsigned long long>(cur) << 32) | L[j];
            auto it = child.find(key);
            if (it == child.end()) {
                const uint32_t nn = static_cast<uint32_t>(node_creator.size());
                node_creator.push_back(static_cast<uint32_t>(pj));
                it = child.emplace(key, nn).first;
            }
            cur = it->second;
            path[g][j] = cur;
        }
    }
    const size_t nn = node_creator.size();
    std::vector<uint32_t> expected(npores, 0);
    for (uint32_t c : node_creator) expected[c]++;

    // type label -> list index
    std::vector<std::pair<uint32_t, uint32_t>> by_fast(ng);
    for (size_t g = 0; g < ng; ++g) by_fast[g] = {fast_ids[g], static_cast<uint32_t>(g)};
    std::sort(by_fast.begin(), by_fast.end());
    auto group_of = [&](uint32_t label) -> int64_t {
        auto it = std::lower_bound(by_fast.begin(), by_fast.end(), std::make_pair(label, 0u));
        return (it != by_fast.end() && it->first == label) ? it->second : -1;
    };

    const Box gr{d.sx, d.sy, d.sz};
    const size_t n = voxels(d);
    std::vector<uint32_t> local(nn, 0xFFFFFFFFu);  // rank of first formation in the creator's search
    std::atomic<size_t> next{0};
    std::atomic<int> failed{0};
    auto worker = [&]() {
        std::vector<uint64_t> visited((n + 63) / 64, 0);
        std::vector<uint32_t> touched;
        std::vector<uint32_t> stack;
        for (;;) {
            const size_t xi = next.fetch_add(1);
            if (xi >= npores) break;
            if (expected[xi] == 0) continue;  // this pore is the first of every key it joins
            const pma_pore& P = pores[xi];
            const uint32_t X = P.id;
            uint32_t seen = 0;
            stack.clear();
            stack.push_back(static_cast<uint32_t>(gr.idx(P.seed_x, P.seed_y, P.seed_z)));
            while (!stack.empty() && seen < expected[xi]) {  // PoreAndThroatComputer.cpp:192-217
                const uint32_t v = stack.back();
                stack.pop_back();
                uint64_t& word = visited[v >> 6];
                const uint64_t bit = 1ull << (v & 63);
                if (word & bit) continue;
                word |= bit;
                touched.push_back(v);
                const uint32_t lab = labels[v];
                if (lab >= 0x80000000u) {  // a shared voxel: the key it takes now
                    const int64_t g = group_of(lab);
                    if (g < 0) {
                        failed = 1;
                        break;
                    }
                    const std::vector<uint32_t>& L = lists[g];
                    const size_t j = std::lower_bound(L.begin(), L.end(), X) - L.begin();
                    if (j >= 1 && j < L.size() && L[j] == X) {
                        const uint32_t node = path[g][j];
                        if (local[node] == 0xFFFFFFFFu) local[node] = seen++;
                    }
                }
                // AddNeighborsToStack, PoreAndThroatComputer.cpp:219-269: x, y, z loops
                const uint32_t r = crad[v];
                int x, y, z;
                gr.coords(v, x, y, z);
                for (int dx = -1; dx <= 1; ++dx)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dz = -1; dz <= 1; ++dz) {
                            if (!dx && !dy && !dz) continue;
                            if (d3q7 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
                            const int nx = x + dx, ny = y + dy, nz = z + dz;
                            if (!gr.inside(nx, ny, nz)) continue;
                            const size_t w = gr.idx(nx, ny, nz);
                            const uint32_t rw = crad[w];
                            if (rw > 0 && rw <= r) stack.push_back(static_cast<uint32_t>(w));
                        }
            }
            if (seen < expected[xi]) failed = 1;
            for (uint32_t v : touched) visited[v >> 6] = 0;
            touched.clear();
        }
    };
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    nt = static_cast<unsigned>(std::min<size_t>(nt, std::max<size_t>(npores, 1)));
    std::vector<std::thread> th;
    for (unsigned i = 1; i < nt; ++i) {
        try {
            th.emplace_back(worker);
        } catch (const std::system_error&) {
            break;  // fewer threads: the running ones take the remaining pores
        }
    }
    worker();
    for (std::thread& t : th) t.join();
    PMA_REQUIRE(!failed, PMA_ERR_INTERNAL, "exact type ids: a pore's search did not form the keys it should");

    // creation order: (creator, rank in its search) -> ids UINT32_MAX - 1, - 2, ...
    std::vector<uint32_t> order(nn);
    for (uint32_t k = 0; k < nn; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return node_creator[a] != node_creator[b] ? node_creator[a] < node_creator[b] : local[a] < local[b];
    });
    std::vector<uint32_t> node_id(nn);
    for (size_t k = 0; k < nn; ++k) node_id[order[k]] = 0xFFFFFFFFu - 1u - static_cast<uint32_t>(k);
    std::vector<uint32_t> out(ng);
    for (size_t g = 0; g < ng; ++g) out[g] = node_id[path[g][lists[g].size() - 1]];
    return out;
}

}  // namespace pma
