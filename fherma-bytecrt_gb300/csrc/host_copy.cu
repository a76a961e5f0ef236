// Copies between device memory and pageable host memory with SM loads and
// stores, for systems where the GPU reads and writes host memory through the
// host's page tables (Grace-based systems such as the GB300: device attribute
// cudaDevAttrPageableMemoryAccessUsesHostPageTables).  There a copy-engine
// copy from pageable memory holds the calling thread for the whole transfer
// and page locking costs about 1.6 us per 64 KiB page, while a copy kernel is
// asynchronous and needs neither (measured on a GB300 host: 199 GB/s reading
// and 170 GB/s writing pageable memory).  The host path uses it for calls too
// small to pipeline, where the SMs are idle while the operands arrive.
#include "kernels.hpp"

#include <algorithm>

namespace bcg {

namespace {

constexpr uint32_t kCopyThreads = 512;

__global__ void __launch_bounds__(kCopyThreads) copy_words16(uint4* __restrict__ dst, const uint4* __restrict__ src,
                                                             size_t n16) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += size_t(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

__global__ void __launch_bounds__(kCopyThreads) copy_words4(uint32_t* __restrict__ dst,
                                                            const uint32_t* __restrict__ src, size_t n) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

int sms() {
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

}  // namespace

cudaError_t launch_host_copy(uint32_t* dst, const uint32_t* src, size_t words, cudaStream_t st) {
    if (words == 0) return cudaSuccess;
    // Four 512-thread CTAs per SM keep enough loads in flight to cover the
    // link's latency; a grid-stride loop covers any size.
    const bool wide = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0 &&
                      words % 4 == 0;
    const size_t units = wide ? words / 4 : words;
    const size_t need = (units + kCopyThreads - 1) / kCopyThreads;
    const uint32_t grid = uint32_t(std::min<size_t>(need, size_t(sms()) * 4));
    if (wide)
        copy_words16<<<grid, kCopyThreads, 0, st>>>(reinterpret_cast<uint4*>(dst), reinterpret_cast<const uint4*>(src),
                                                     units);
    else
        copy_words4<<<grid, kCopyThreads, 0, st>>>(dst, src, units);
    return cudaGetLastError();
}

}  // namespace bcg
