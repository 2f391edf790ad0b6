// Whole-field transfers between device memory and the caller's host buffers.
//
// A page-locked host buffer is device-accessible through its mapped address, so a field moves
// with a streaming kernel (16-byte loads and stores over every SM) instead of a copy engine.
// On the GB300 machine (Grace host, NVLink-C2C) both reach 193 GB/s device-to-host at best,
// but copy-engine transfers into a pinned buffer fell to 24-98 GB/s on many calls (after the
// host or a kernel had touched the buffer, and at random on repeats), while the kernel held
// 191-193 GB/s in every case measured. Pageable buffers, and pairs of addresses whose
// alignments differ, go through cudaMemcpyAsync.
#include "devutil.cuh"

namespace pma {
namespace {

__global__ void __launch_bounds__(256) stream_copy16(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                     size_t n16) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n16;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

// The device-side address of a page-locked host buffer, or null for pageable memory.
void* mapped_address(const void* host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();  // an unknown pointer leaves a (non-sticky) error: clear it
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void transfer(pma_ctx* ctx, void* dst, const void* src, size_t bytes, bool to_host) {
    if (!bytes || !dst || !src) return;
    const cudaMemcpyKind kind = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
    void* hd = mapped_address(to_host ? dst : src);
    const char* s = static_cast<const char*>(to_host ? src : hd);
    char* d = static_cast<char*>(to_host ? hd : dst);
    if (!hd || (reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d)) % 16 != 0) {
        PMA_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
        return;
    }
    const size_t n16 = bytes / 16;
    if (n16) {
        const unsigned grid = static_cast<unsigned>(std::min<size_t>((n16 + 255) / 256, ctx->num_sms * 8ull));
        stream_copy16<<<grid, 256, 0, ctx->stream>>>(reinterpret_cast<const uint4*>(s), reinterpret_cast<uint4*>(d),
                                                     n16);
        ctx->count_launch();
        ctx->check_launch("stream_copy16");
    }
    const size_t done = n16 * 16;
    if (done < bytes)
        PMA_CUDA(cudaMemcpyAsync(static_cast<char*>(dst) + done, static_cast<const char*>(src) + done, bytes - done,
                                 kind, ctx->stream));
}

}  // namespace

void copy_to_host(pma_ctx* ctx, void* host, const void* dev, size_t bytes) { transfer(ctx, host, dev, bytes, true); }

void copy_from_host(pma_ctx* ctx, void* dev, const void* host, size_t bytes) {
    transfer(ctx, dev, host, bytes, false);
}

}  // namespace pma
