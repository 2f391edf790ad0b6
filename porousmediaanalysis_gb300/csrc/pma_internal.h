// Internal runtime of the pma library: context, errors, scratch cache, launch accounting.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pma.h"

namespace pma {

// Error carried through the C++ layer and turned into a pma_status at the C boundary.
struct Error : std::runtime_error {
    pma_status status;
    Error(pma_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string& msg);

#define PMA_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            throw ::pma::Error(PMA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define PMA_REQUIRE(cond, status, msg)                                                      \
    do {                                                                                    \
        if (!(cond)) throw ::pma::Error(status, msg);                                       \
    } while (0)

// Runs a C++ body and maps exceptions onto the C ABI status codes.
template <class F>
int guarded(F&& f) {
    try {
        f();
        return PMA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return PMA_ERR_MEMORY;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return PMA_ERR_IO;
    } catch (...) {
        set_last_error("unknown error");
        return PMA_ERR_INTERNAL;
    }
}

}  // namespace pma

// Device buffers cached by name; grow-only until trimmed. They come from a stream-ordered
// memory pool of the context: growing one never synchronises the device, so batch lanes and
// serving lanes do not stall each other.
struct pma_ctx {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::atomic<uint64_t> launches{0};
    struct Buf {
        void* ptr = nullptr;
        size_t bytes = 0;
    };
    std::map<std::string, Buf> cache;
    cudaMemPool_t pool = nullptr;  // stream-ordered pool of the scratch buffers
    bool blocking_sync = false;    // sync() sleeps on an event instead of spinning
    cudaEvent_t sync_event = nullptr;
    void* pinned = nullptr;       // small pinned host staging area
    size_t pinned_bytes = 0;
    bool timing = false;          // bracket hot kernels with events
    struct Timed {
        std::string name;
        cudaEvent_t start, stop;
    };
    std::vector<Timed> timed;
    // Work counters of the timed calls (reported with the timings as [sum, increments]).
    std::map<std::string, std::pair<double, long long>> counters;
    void count(const std::string& name, double v) {
        if (!timing) return;
        auto& c = counters[name];
        c.first += v;
        c.second += 1;
    }
    std::vector<pma_ctx*> lanes;  // child contexts of batch calls (own stream and scratch)
    pma_limits limits{1 << 20, 1 << 22, (1ull << 23) - 1, 0};  // device loop bounds
    bool reference_throat_ids = false;  // pma_pores numbers shared types as the reference does
    // Demand: the largest size each named buffer was asked for since reset_demand(), summed;
    // what one request needs, whatever earlier requests left in the cache.
    std::map<std::string, size_t> demand;
    size_t demand_bytes = 0;
    void reset_demand() {
        demand.clear();
        demand_bytes = 0;
    }

    void* scratch(const std::string& tag, size_t bytes);
    size_t cached_bytes(const std::string& tag) const {  // capacity held under tag (0 = none)
        auto it = cache.find(tag);
        return it == cache.end() ? 0 : it->second.bytes;
    }
    void release(const std::string& tag);  // frees one scratch buffer (after the stream's work)
    void* host_staging(size_t bytes);
    // Page-locked host buffers by name, grow-only until trimmed (host copies of large device
    // arrays that the host works on, moved by the streaming copy kernel).
    std::map<std::string, Buf> host_cache;
    void* host_buffer(const std::string& tag, size_t bytes);
    void free_host_buffers();
    int64_t* pinned_count();  // a pinned word of its own for counts read back after CUB calls
    int64_t* count_word = nullptr;
    void sync();
    void check_launch(const char* what);
    void count_launch(uint64_t n = 1) { launches.fetch_add(n, std::memory_order_relaxed); }
};

struct pma_table {
    std::vector<pma_pore> pores;
    std::vector<pma_throat> throats;
    std::vector<uint32_t> pool;
};

namespace pma {

// Brackets the launches of its scope with CUDA events when the context's timing is on.
struct KernelTimer {
    pma_ctx* ctx;
    const char* name;
    cudaEvent_t start = nullptr;
    KernelTimer(pma_ctx* c, const char* n) : ctx(c), name(n) {
        if (ctx->timing && cudaEventCreate(&start) == cudaSuccess) cudaEventRecord(start, ctx->stream);
    }
    ~KernelTimer() {
        if (!start) return;
        cudaEvent_t stop;
        if (cudaEventCreate(&stop) != cudaSuccess) return;
        cudaEventRecord(stop, ctx->stream);
        ctx->timed.push_back(pma_ctx::Timed{name, start, stop});
    }
};

inline unsigned div_up(size_t a, size_t b) { return static_cast<unsigned>((a + b - 1) / b); }

inline void check_dims(pma_dims d) {
    PMA_REQUIRE(d.sx > 0 && d.sy > 0 && d.sz > 0, PMA_ERR_ARGUMENT, "volume dimensions must be positive");
    unsigned long long n = 1ull * d.sx * d.sy * d.sz;
    PMA_REQUIRE(n < (1ull << 32), PMA_ERR_ARGUMENT, "volume must hold fewer than 2^32 voxels");
}

inline size_t voxels(pma_dims d) { return static_cast<size_t>(d.sx) * d.sy * d.sz; }

// Stage implementations (device pointers, ctx stream).
void edt(pma_ctx* ctx, const uint8_t* solid, pma_dims d, uint32_t* edt2, pma_edt_stats* stats,
         uint64_t* h_hist, size_t hist_cap);
void edt_noalloc(const uint8_t* solid, pma_dims d, uint32_t* edt2, pma_edt_stats* stats,
                 uint64_t* h_hist, size_t hist_cap, cudaStream_t s);
void containing_balls(pma_ctx* ctx, const uint32_t* edt2, pma_dims d, uint32_t max_edt2,
                      uint32_t* crad2, uint32_t* cx, uint32_t* cy, uint32_t* cz, uint8_t* mask,
                      uint64_t* count);
// Returns every cavity's row, in the order the cavities were flooded.
template <class T>
std::vector<pma_cavity> geodesic(pma_ctx* ctx, const uint8_t* solid, pma_dims d, pma_stencil st, T* dist,
                                 uint32_t* cavity);
pma_table* pores(pma_ctx* ctx, const uint8_t* mask, const uint32_t* edt2, const uint32_t* crad2,
                 pma_dims d, pma_stencil st, uint32_t* labels);
void remove_empty_pores(pma_ctx* ctx, pma_table* t, uint32_t* labels, pma_dims d);
pma_table* watershed(pma_ctx* ctx, const pma_table* pores, const uint32_t* crad2, pma_dims d,
                     pma_stencil st, uint32_t max_edt2, uint32_t* labels);
void wait_selftest(pma_ctx* ctx, int* timed_out);
// Whole-field transfers on the context's stream: a streaming kernel through the mapped address
// of a page-locked host buffer, cudaMemcpyAsync for pageable ones (transfer.cu).
void copy_to_host(pma_ctx* ctx, void* host, const void* dev, size_t bytes);
void copy_from_host(pma_ctx* ctx, void* dev, const void* host, size_t bytes);
// resample.cu: 8-bit slices [nz][sx][sy] (host) upsampled in plane to [nz][dx][dy] as the
// reference's image rescale does.
std::vector<uint8_t> resample_slices(pma_ctx* ctx, const std::vector<uint8_t>& src, int nz, int sx, int sy, int dx,
                                     int dy);
// exact_ids.cpp: the reference's shared-type ids of the initial propagation, per type row.
std::vector<uint32_t> replay_type_ids(const uint32_t* crad, const uint32_t* labels, pma_dims d, bool d3q7,
                                      const std::vector<pma_pore>& pores,
                                      const std::vector<std::vector<uint32_t>>& lists,
                                      const std::vector<uint32_t>& fast_ids);

// Copies the first `cap` cavity rows to `out` and reports how many there are in all.
inline void copy_cavities(const std::vector<pma_cavity>& rows, pma_cavity* out, int cap, int* n) {
    const size_t k = std::min(rows.size(), static_cast<size_t>(cap > 0 ? cap : 0));
    for (size_t i = 0; i < k; ++i) out[i] = rows[i];
    if (n) *n = static_cast<int>(rows.size());
}

// Whole chain of one volume on ctx's stream (pipeline.cpp): from host buffers, or on device
// buffers (output field pointers of `out` are device pointers, NULL = context scratch).
void run_pipeline_host(pma_ctx* ctx, const uint8_t* h_solid, pma_dims dims, const pma_options& o,
                       pma_outputs* out);
void run_pipeline_device(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, const pma_options& o,
                         pma_outputs* out);

}  // namespace pma
