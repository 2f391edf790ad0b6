// Batched pipeline: many independent volumes of uneven sizes in flight at once.
//
// The chain of one small volume is bound by launch latency and by the host round trips of
// its data-dependent loops (level sweeps, watershed generations, geodesic buckets), not by
// HBM: a 100^3 volume keeps the GPU mostly idle. The batch therefore runs several volumes
// concurrently, each on its own lane - a child context with its own stream, scratch cache
// and host thread - so that one lane's kernels fill the gaps of the others. Lanes take the
// largest remaining volume next (longest-processing-time order), and keep their scratch
// for later batches. Every volume's results are those of a separate pma_pipeline_host call:
// the lanes share no device state.
#include <algorithm>
#include <atomic>
#include <numeric>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "pma_internal.h"

using pma::guarded;

namespace pma {
namespace {

pma_ctx* make_lane(const pma_ctx* parent) {
    pma_ctx* c = new pma_ctx;
    c->device = parent->device;
    c->num_sms = parent->num_sms;
    c->smem_optin = parent->smem_optin;
    c->timing = false;
    c->limits = parent->limits;
    c->reference_throat_ids = parent->reference_throat_ids;
    const cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        throw Error(PMA_ERR_CUDA, std::string("pma_pipeline_batch: stream creation failed: ") +
                                      cudaGetErrorString(e));
    }
    c->own_stream = true;
    return c;
}

}  // namespace
}  // namespace pma

extern "C" int pma_pipeline_batch(pma_ctx* ctx, pma_batch_item* items, size_t n, const pma_options* opts,
                                  int resident, int lanes) {
    std::string first_error;
    int first_status = PMA_OK;
    const int rc = guarded([&] {
        PMA_REQUIRE(ctx, PMA_ERR_ARGUMENT, "pma_pipeline_batch: null context");
        PMA_REQUIRE(items || n == 0, PMA_ERR_ARGUMENT, "pma_pipeline_batch: null items");
        PMA_REQUIRE(lanes >= 0 && lanes <= 64, PMA_ERR_ARGUMENT, "pma_pipeline_batch: lanes must be 0..64");
        PMA_CUDA(cudaSetDevice(ctx->device));
        pma_options o{PMA_D3Q27, 1, 1, 0};
        if (opts) o = *opts;
        for (size_t i = 0; i < n; ++i) {
            pma::check_dims(items[i].dims);
            PMA_REQUIRE(items[i].solid && items[i].out, PMA_ERR_ARGUMENT, "pma_pipeline_batch: null item buffer");
            items[i].status = -1;
        }
        if (n == 0) return;
        const size_t want = std::min<size_t>(lanes ? static_cast<size_t>(lanes) : 8, n);
        while (ctx->lanes.size() < want) ctx->lanes.push_back(pma::make_lane(ctx));
        // several lanes: host threads sleep in their synchronisations, leaving CPU cores to
        // each other; a single lane spins like a plain call
        for (size_t l = 0; l < want; ++l) ctx->lanes[l]->blocking_sync = want > 1;
        // Inputs produced on the caller's stream must be complete before the lanes read them.
        PMA_CUDA(cudaStreamSynchronize(ctx->stream));

        std::vector<size_t> order(n);
        std::iota(order.begin(), order.end(), size_t(0));
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return pma::voxels(items[a].dims) > pma::voxels(items[b].dims);
        });
        std::atomic<size_t> next{0};
        std::vector<std::string> messages(n);
        auto work = [&](pma_ctx* lane) {
            cudaSetDevice(lane->device);
            for (size_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
                pma_batch_item& it = items[order[k]];
                it.status = guarded([&] {
                    if (resident) pma::run_pipeline_device(lane, it.solid, it.dims, o, it.out);
                    else pma::run_pipeline_host(lane, it.solid, it.dims, o, it.out);
                });
                if (it.status != PMA_OK) {
                    char buf[1024];
                    pma_last_error(buf, sizeof(buf));
                    messages[order[k]] = buf;
                }
            }
        };
        std::vector<std::thread> threads;
        for (size_t l = 1; l < want; ++l) {
            try {
                threads.emplace_back(work, ctx->lanes[l]);
            } catch (const std::system_error&) {
                break;  // fewer host threads: the lanes that run take the remaining volumes
            }
        }
        work(ctx->lanes[0]);
        for (std::thread& t : threads) t.join();
        for (size_t i = 0; i < n; ++i)
            if (items[i].status != PMA_OK) {
                first_status = items[i].status;
                first_error = "pma_pipeline_batch: volume " + std::to_string(i) + ": " + messages[i];
                break;
            }
    });
    if (rc != PMA_OK) return rc;
    if (first_status != PMA_OK) pma::set_last_error(first_error);
    return first_status;
}
