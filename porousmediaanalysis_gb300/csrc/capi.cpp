// C ABI of the pma library (include/pma.h): context, errors, tables and stage wrappers.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

#include "pma_internal.h"
#include "pma_io.h"

namespace pma {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

}  // namespace pma

using pma::Error;
using pma::guarded;

static cudaMemPool_t ensure_pool(pma_ctx* c) {
    if (c->pool) return c->pool;
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = c->device;
    PMA_CUDA(cudaMemPoolCreate(&c->pool, &props));
    // Freed blocks stay in the pool for reuse until pma_ctx_trim: buffers that grow inside a
    // call (e.g. the watershed's shared-voxel records) would otherwise go back to the driver
    // at every synchronisation and be mapped afresh, gigabytes at a time, on the next call.
    unsigned long long keep = ~0ull;
    PMA_CUDA(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    return c->pool;
}

void* pma_ctx::scratch(const std::string& tag, size_t bytes) {
    size_t& d = demand[tag];
    if (bytes > d) {
        demand_bytes += bytes - d;
        d = bytes;
    }
    Buf& b = cache[tag];
    if (b.bytes >= bytes && b.ptr) return b.ptr;
    cudaMemPool_t mp = ensure_pool(this);
    if (b.ptr) {  // stream-ordered: freed after the work already queued on the stream
        PMA_CUDA(cudaFreeAsync(b.ptr, stream));
        b.ptr = nullptr;
        b.bytes = 0;
    }
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMallocFromPoolAsync(&b.ptr, want, mp, stream);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        (void)cudaGetLastError();
        throw Error(PMA_ERR_MEMORY, "device allocation of " + std::to_string(want) + " bytes for " +
                                        tag + " failed: " + cudaGetErrorString(e));
    }
    b.bytes = want;
    return b.ptr;
}

void pma_ctx::release(const std::string& tag) {
    auto it = cache.find(tag);
    if (it == cache.end()) return;
    if (it->second.ptr) PMA_CUDA(cudaFreeAsync(it->second.ptr, stream));
    cache.erase(it);
}

void* pma_ctx::host_staging(size_t bytes) {
    if (pinned_bytes >= bytes && pinned) return pinned;
    if (pinned) {
        PMA_CUDA(cudaStreamSynchronize(stream));
        PMA_CUDA(cudaFreeHost(pinned));
        pinned = nullptr;
    }
    PMA_CUDA(cudaMallocHost(&pinned, bytes));
    pinned_bytes = bytes;
    return pinned;
}

void* pma_ctx::host_buffer(const std::string& tag, size_t bytes) {
    Buf& b = host_cache[tag];
    if (b.ptr && b.bytes >= bytes) return b.ptr;
    if (b.ptr) {
        PMA_CUDA(cudaFreeHost(b.ptr));
        b.ptr = nullptr;
        b.bytes = 0;
    }
    const size_t want = std::max<size_t>(bytes + bytes / 8, 4096);
    PMA_CUDA(cudaMallocHost(&b.ptr, want));
    b.bytes = want;
    return b.ptr;
}

void pma_ctx::free_host_buffers() {
    for (auto& kv : host_cache)
        if (kv.second.ptr) cudaFreeHost(kv.second.ptr);
    host_cache.clear();
}

int64_t* pma_ctx::pinned_count() {
    if (!count_word) {
        void* p = nullptr;
        PMA_CUDA(cudaMallocHost(&p, 64));
        count_word = static_cast<int64_t*>(p);
    }
    return count_word;
}

void pma_ctx::sync() {
    if (!blocking_sync) {
        PMA_CUDA(cudaStreamSynchronize(stream));
        return;
    }
    // lanes of a batch or a server: the host thread sleeps instead of spinning, leaving the
    // CPU cores to the other lanes' host work
    if (!sync_event) PMA_CUDA(cudaEventCreateWithFlags(&sync_event, cudaEventBlockingSync | cudaEventDisableTiming));
    PMA_CUDA(cudaEventRecord(sync_event, stream));
    PMA_CUDA(cudaEventSynchronize(sync_event));
}

void pma_ctx::check_launch(const char* what) {
    count_launch(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(PMA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

extern "C" {

size_t pma_last_error(char* buf, size_t cap) {
    const std::string& m = pma::g_last_error;
    if (buf && cap) {
        size_t n = std::min(cap - 1, m.size());
        std::memcpy(buf, m.data(), n);
        buf[n] = 0;
    }
    return m.size();
}

int pma_abi_version(void) { return PMA_ABI_VERSION; }

int pma_ctx_create(int device, pma_ctx** out) {
    return guarded([&] {
        PMA_REQUIRE(out, PMA_ERR_ARGUMENT, "pma_ctx_create: null output");
        int n = 0;
        PMA_CUDA(cudaGetDeviceCount(&n));
        PMA_REQUIRE(device >= 0 && device < n, PMA_ERR_CUDA, "pma_ctx_create: no such CUDA device");
        PMA_CUDA(cudaSetDevice(device));
        pma_ctx* c = new pma_ctx;
        c->device = device;
        cudaDeviceProp p;
        PMA_CUDA(cudaGetDeviceProperties(&p, device));
        c->num_sms = p.multiProcessorCount;
        c->smem_optin = p.sharedMemPerBlockOptin;
        PMA_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
        *out = c;
    });
}

int pma_ctx_destroy(pma_ctx* ctx) {
    if (!ctx) return PMA_OK;
    return guarded([&] {
        for (pma_ctx* lane : ctx->lanes) pma_ctx_destroy(lane);
        ctx->lanes.clear();
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        for (auto& kv : ctx->cache)
            if (kv.second.ptr) cudaFreeAsync(kv.second.ptr, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
        if (ctx->sync_event) cudaEventDestroy(ctx->sync_event);
        if (ctx->pinned) cudaFreeHost(ctx->pinned);
        if (ctx->count_word) cudaFreeHost(ctx->count_word);
        ctx->free_host_buffers();
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
    });
}

int pma_ctx_set_stream(pma_ctx* ctx, void* stream) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        PMA_CUDA(cudaSetDevice(ctx->device));
        // scratch buffers are stream-ordered: finish the old stream's work before switching
        PMA_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ctx->own_stream) {
            PMA_CUDA(cudaStreamDestroy(ctx->stream));
            ctx->own_stream = false;
        }
        if (stream) {
            ctx->stream = static_cast<cudaStream_t>(stream);
        } else {
            PMA_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
    });
}

uint64_t pma_ctx_launch_count(const pma_ctx* ctx) {
    if (!ctx) return 0;
    uint64_t total = ctx->launches.load();
    for (const pma_ctx* lane : ctx->lanes) total += pma_ctx_launch_count(lane);
    return total;
}

int pma_ctx_get_limits(const pma_ctx* ctx, pma_limits* out) {
    return guarded([&] {
        PMA_REQUIRE(ctx && out, PMA_ERR_ARGUMENT, "pma_ctx_get_limits: null argument");
        *out = ctx->limits;
    });
}

int pma_ctx_set_limits(pma_ctx* ctx, const pma_limits* limits) {
    return guarded([&] {
        PMA_REQUIRE(ctx && limits, PMA_ERR_ARGUMENT, "pma_ctx_set_limits: null argument");
        PMA_REQUIRE(limits->spin_limit >= 0 && limits->union_limit >= 0, PMA_ERR_ARGUMENT,
                    "pma_ctx_set_limits: negative limit");
        PMA_REQUIRE(limits->watershed_generations >= 1, PMA_ERR_ARGUMENT,
                    "pma_ctx_set_limits: watershed_generations must be at least 1");
        ctx->limits = *limits;
    });
}

int pma_ctx_set_throat_numbering(pma_ctx* ctx, int reference_order) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "pma_ctx_set_throat_numbering: null context");
        ctx->reference_throat_ids = reference_order != 0;
    });
}

int pma_selftest_bounded_wait(pma_ctx* ctx, int* timed_out) {
    return guarded([&] {
        PMA_REQUIRE(ctx && timed_out, PMA_ERR_ARGUMENT, "pma_selftest_bounded_wait: null argument");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma::wait_selftest(ctx, timed_out);
    });
}

int pma_ctx_set_timing(pma_ctx* ctx, int enable) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        ctx->timing = enable != 0;
    });
}

size_t pma_ctx_timing_report(pma_ctx* ctx, char* buf, size_t cap) {
    std::string out = "{";
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        std::map<std::string, std::pair<double, long long>> acc;
        for (auto& t : ctx->timed) {
            float ms = 0;
            if (cudaEventElapsedTime(&ms, t.start, t.stop) == cudaSuccess) {
                acc[t.name].first += ms;
                acc[t.name].second += 1;
            }
            cudaEventDestroy(t.start);
            cudaEventDestroy(t.stop);
        }
        ctx->timed.clear();
        for (auto& kv : ctx->counters) acc["count." + kv.first] = kv.second;
        ctx->counters.clear();
        bool first = true;
        char item[256];
        for (auto& kv : acc) {
            std::snprintf(item, sizeof(item), "%s\"%s\": [%.6f, %lld]", first ? "" : ", ", kv.first.c_str(),
                          kv.second.first, kv.second.second);
            out += item;
            first = false;
        }
    }
    out += "}";
    if (buf && cap) {
        size_t n = std::min(cap - 1, out.size());
        std::memcpy(buf, out.data(), n);
        buf[n] = 0;
    }
    return out.size();
}

size_t pma_ctx_scratch_bytes(const pma_ctx* ctx) {
    size_t s = 0;
    if (ctx) {
        for (auto& kv : ctx->cache) s += kv.second.bytes;
        // the pool also holds freed blocks kept for reuse
        unsigned long long reserved = 0;
        if (ctx->pool && cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess)
            s = std::max<size_t>(s, static_cast<size_t>(reserved));
        for (const pma_ctx* lane : ctx->lanes) s += pma_ctx_scratch_bytes(lane);
    }
    return s;
}

int pma_ctx_trim(pma_ctx* ctx) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        for (pma_ctx* lane : ctx->lanes) PMA_REQUIRE(pma_ctx_trim(lane) == PMA_OK, PMA_ERR_CUDA, "pma_ctx_trim: lane");
        PMA_CUDA(cudaSetDevice(ctx->device));
        PMA_CUDA(cudaStreamSynchronize(ctx->stream));
        for (auto& kv : ctx->cache)
            if (kv.second.ptr) PMA_CUDA(cudaFreeAsync(kv.second.ptr, ctx->stream));
        ctx->cache.clear();
        PMA_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ctx->pool) PMA_CUDA(cudaMemPoolTrimTo(ctx->pool, 0));
        ctx->free_host_buffers();
    });
}

int pma_edt(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, uint32_t* d_edt2,
            pma_edt_stats* stats, uint64_t* h_hist, size_t hist_cap) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma::edt(ctx, d_solid, dims, d_edt2, stats, h_hist, hist_cap);
    });
}

int pma_edt_noalloc(const uint8_t* d_solid, pma_dims dims, uint32_t* d_edt2, pma_edt_stats* stats,
                    uint64_t* h_hist, size_t hist_cap, void* cuda_stream) {
    return guarded([&] {
        pma::edt_noalloc(d_solid, dims, d_edt2, stats, h_hist, hist_cap,
                         static_cast<cudaStream_t>(cuda_stream));
    });
}

int pma_containing_balls(pma_ctx* ctx, const uint32_t* d_edt2, pma_dims dims, uint32_t max_edt2,
                         uint32_t* d_crad2, uint32_t* d_cx, uint32_t* d_cy, uint32_t* d_cz,
                         uint8_t* d_mask, uint64_t* h_count) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma::containing_balls(ctx, d_edt2, dims, max_edt2, d_crad2, d_cx, d_cy, d_cz, d_mask, h_count);
    });
}

int pma_table_create(const pma_pore* pores, size_t n_pores, const pma_throat* throats,
                     size_t n_throats, const uint32_t* pool, size_t pool_size, pma_table** out) {
    return guarded([&] {
        PMA_REQUIRE(out, PMA_ERR_ARGUMENT, "pma_table_create: null output");
        PMA_REQUIRE(n_pores == 0 || pores, PMA_ERR_ARGUMENT, "pma_table_create: null pores");
        PMA_REQUIRE(n_throats == 0 || throats, PMA_ERR_ARGUMENT, "pma_table_create: null throats");
        PMA_REQUIRE(pool_size == 0 || pool, PMA_ERR_ARGUMENT, "pma_table_create: null pool");
        for (size_t i = 0; i < n_throats; ++i)
            PMA_REQUIRE(throats[i].pool_offset + throats[i].n_pores <= pool_size, PMA_ERR_ARGUMENT,
                        "pma_table_create: throat pore list outside the pool");
        pma_table* t = new pma_table;
        t->pores.assign(pores, pores + n_pores);
        t->throats.assign(throats, throats + n_throats);
        t->pool.assign(pool, pool + pool_size);
        *out = t;
    });
}

size_t pma_table_npores(const pma_table* t) { return t ? t->pores.size() : 0; }
const pma_pore* pma_table_pores(const pma_table* t) { return t ? t->pores.data() : nullptr; }
size_t pma_table_nthroats(const pma_table* t) { return t ? t->throats.size() : 0; }
const pma_throat* pma_table_throats(const pma_table* t) { return t ? t->throats.data() : nullptr; }
size_t pma_table_pool_size(const pma_table* t) { return t ? t->pool.size() : 0; }
const uint32_t* pma_table_pool(const pma_table* t) { return t ? t->pool.data() : nullptr; }
void pma_table_free(pma_table* t) { delete t; }

int pma_pores(pma_ctx* ctx, const uint8_t* d_mask, const uint32_t* d_edt2, const uint32_t* d_crad2,
              pma_dims dims, pma_stencil stencil, uint32_t* d_labels, pma_table** out) {
    return guarded([&] {
        PMA_REQUIRE(ctx && out, PMA_ERR_ARGUMENT, "pma_pores: null context or output");
        PMA_CUDA(cudaSetDevice(ctx->device));
        *out = pma::pores(ctx, d_mask, d_edt2, d_crad2, dims, stencil, d_labels);
    });
}

int pma_remove_empty_pores(pma_ctx* ctx, pma_table* table, uint32_t* d_labels, pma_dims dims) {
    return guarded([&] {
        PMA_REQUIRE(ctx && table, PMA_ERR_ARGUMENT, "pma_remove_empty_pores: null context or table");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma::remove_empty_pores(ctx, table, d_labels, dims);
    });
}

int pma_watershed(pma_ctx* ctx, const pma_table* pores, const uint32_t* d_crad2, pma_dims dims,
                  pma_stencil stencil, uint32_t max_edt2, uint32_t* d_labels_ws, pma_table** out) {
    return guarded([&] {
        PMA_REQUIRE(ctx && pores && out, PMA_ERR_ARGUMENT, "pma_watershed: null argument");
        PMA_CUDA(cudaSetDevice(ctx->device));
        *out = pma::watershed(ctx, pores, d_crad2, dims, stencil, max_edt2, d_labels_ws);
    });
}

int pma_geodesic_f32(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, pma_stencil stencil,
                     float* d_dist, uint32_t* d_cavity, pma_cavity* h_cav, int cap, int* n_cav) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        PMA_CUDA(cudaSetDevice(ctx->device));
        PMA_REQUIRE(cap >= 0 && (cap == 0 || h_cav), PMA_ERR_ARGUMENT, "pma_geodesic_f32: bad cavity buffer");
        const std::vector<pma_cavity> rows = pma::geodesic<float>(ctx, d_solid, dims, stencil, d_dist, d_cavity);
        pma::copy_cavities(rows, h_cav, cap, n_cav);
    });
}

int pma_geodesic_f64(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, pma_stencil stencil,
                     double* d_dist, uint32_t* d_cavity, pma_cavity* h_cav, int cap, int* n_cav) {
    return guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "null context");
        PMA_CUDA(cudaSetDevice(ctx->device));
        PMA_REQUIRE(cap >= 0 && (cap == 0 || h_cav), PMA_ERR_ARGUMENT, "pma_geodesic_f64: bad cavity buffer");
        const std::vector<pma_cavity> rows = pma::geodesic<double>(ctx, d_solid, dims, stencil, d_dist, d_cavity);
        pma::copy_cavities(rows, h_cav, cap, n_cav);
    });
}

int pma_read_tiff_stack(const char* folder, int bpv, pma_dims* dims, void* out, size_t out_bytes) {
    return guarded([&] {
        PMA_REQUIRE(folder && dims, PMA_ERR_ARGUMENT, "pma_read_tiff_stack: null argument");
        PMA_REQUIRE(bpv == 1 || bpv == 4, PMA_ERR_ARGUMENT, "pma_read_tiff_stack: 1 or 4 bytes per voxel");
        pma::Dims d;
        std::vector<uint8_t> v = pma::read_stack(folder, bpv, &d);
        dims->sx = d.sx;
        dims->sy = d.sy;
        dims->sz = d.sz;
        if (out) {
            PMA_REQUIRE(out_bytes >= v.size(), PMA_ERR_ARGUMENT, "pma_read_tiff_stack: output too small");
            std::memcpy(out, v.data(), v.size());
        }
    });
}

int pma_read_config(const char* path, pma_run_config* out) {
    return guarded([&] {
        PMA_REQUIRE(path && out, PMA_ERR_ARGUMENT, "pma_read_config: null argument");
        const pma::RunConfig c = pma::read_config(path);
        std::memset(out, 0, sizeof(*out));
        for (int i = 0; i < 3; ++i) out->resolution[i] = c.resolution[i];
        out->max_pore_radius_ratio = c.max_pore_radius_ratio;
        out->available_memory_mb = c.available_memory_mb;
        out->use_d3q7 = c.use_d3q7;
        out->threads = c.threads;
    });
}

int pma_write_tiff_stack(const char* folder, int bpv, pma_dims dims, const void* data) {
    return guarded([&] {
        PMA_REQUIRE(folder && data, PMA_ERR_ARGUMENT, "pma_write_tiff_stack: null argument");
        PMA_REQUIRE(bpv == 1 || bpv == 4, PMA_ERR_ARGUMENT, "pma_write_tiff_stack: 1 or 4 bytes per voxel");
        pma::Dims d;
        d.sx = dims.sx;
        d.sy = dims.sy;
        d.sz = dims.sz;
        // zero-padded names: the reference (and read_stack) orders slices by name
        std::vector<std::string> names;
        const int width = static_cast<int>(std::to_string(std::max(d.sz, 1)).size());
        for (int z = 0; z < d.sz; ++z) {
            std::string s = std::to_string(z + 1);
            names.push_back(std::string(width - s.size(), '0') + s + ".tif");
        }
        pma::write_stack(folder, names, data, bpv, d);
    });
}

}  // extern "C"
