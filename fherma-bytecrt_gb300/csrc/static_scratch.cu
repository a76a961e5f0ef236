// Allocation-free product entry point: bcg_multiply_device_static.
//
// Some callers cannot allocate device memory at call time: code running
// under a memory pool they do not own, inside a framework that forbids
// cudaMalloc on its hot path, or in a process whose allocator is already at
// its limit.  bcg_multiply_device allocates its residue-plane workspace on
// first use; this entry point instead uses a fixed scratch array compiled into
// the library, so a call performs no cudaMalloc, cudaFree or other allocation.
//
// The scratch is a file-scope __device__ array of kStaticScratchWords uint32
// (16 MiB).  Every GPU that loads the library holds it until the process
// exits.  One product needs 2 * P * N words of it, so it fits points up to
// N = 32768 with W around 868 bits (P = 57); a larger point is rejected with
// BCG_ERR_INVALID.  Several products fitting at once run in one launch chain.
//
// Set-up: host code cannot use the array's name as a device address, so the
// first call on each device looks up the address with cudaGetSymbolAddress,
// with that device current, and keeps it.  Make that first call before any
// stream capture.  The address stays valid for the life of the device's
// primary context: after cudaDeviceReset the library's module is loaded
// again elsewhere, so do not call this entry point across a device reset.
// All calls share the array: calls that overlap on the GPU (different
// streams, contexts or threads) race on it.  Nothing in it needs to start at
// zero; every word a call reads was written earlier by the same call.
#include "../../include/bytecrt_gb300.h"
#include "capi_internal.hpp"

#include <algorithm>
#include <mutex>

namespace {

constexpr size_t kStaticScratchWords = size_t(4) << 20;   // 16 MiB

__device__ __align__(256) uint32_t g_static_scratch[kStaticScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (set-up on first use).
uint32_t* scratch_address(int device) {
    if (device < 0 || device >= kMaxDevices) throw std::invalid_argument("device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[device]) {
        int previous = 0;
        bcg::check(cudaGetDevice(&previous), "current device");
        bcg::check(cudaSetDevice(device), "select device");
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        cudaSetDevice(previous);
        bcg::check(e, "static scratch address");
        g_scratch_ptr[device] = static_cast<uint32_t*>(p);
    }
    return g_scratch_ptr[device];
}

}  // namespace

extern "C" int bcg_multiply_device_static(bcg_context* ctx, const uint32_t* a, const uint32_t* b, uint32_t* c,
                                          uint32_t count, void* stream) {
    try {
        if (!ctx) throw std::invalid_argument("null context");
        if (count == 0) return BCG_OK;
        if (!a || !b || !c) throw std::invalid_argument("null buffer");
        bcg::Context& x = *ctx->ctx;
        const size_t pw = x.plane_words();
        const size_t per_product = 2 * pw;
        if (per_product > kStaticScratchWords)
            throw std::invalid_argument("point needs " + std::to_string(per_product) +
                                        " scratch words per product; the static scratch holds " +
                                        std::to_string(kStaticScratchWords));
        uint32_t* ws = scratch_address(x.device());
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : x.stream();
        // Products per launch chain: as many as the scratch holds, but no more
        // than the context's own chain length (the allocating path's group),
        // which keeps every stage's grid within its limits (the column pass
        // puts 2 x products on grid.z).
        const uint32_t fit = uint32_t(std::min<size_t>(kStaticScratchWords / per_product,
                                                       std::max<uint32_t>(1u, x.group())));
        const size_t cw = x.coeff_words();
        const bcg::NttArgs ntt = x.ntt_args();
        for (uint32_t done = 0; done < count; done += fit) {
            const uint32_t n = count - done < fit ? count - done : fit;
            // Same stages as the allocating path, on the static planes.
            uint32_t* pa = ws;
            uint32_t* pb = ws + pw;
            x.encode(a + done * cw, b + done * cw, pa, pb, per_product, n, st);
            if (x.geom().C > 1) bcg::check(bcg::launch_col_forward(ntt, pa, pw, 2 * n, st), "column pass launch");
            bcg::check(bcg::launch_row_product(ntt, pa, per_product, pb, per_product, pa, per_product, n, false, st),
                       "row pass launch");
            if (x.geom().C > 1) bcg::check(bcg::launch_col_inverse(ntt, pa, per_product, n, st), "inverse column pass launch");
            x.crt(pa, per_product, c + done * cw, n, st);
        }
        return BCG_OK;
    } catch (const std::invalid_argument& e) {
        bcg::set_last_error(e.what());
        return BCG_ERR_INVALID;
    } catch (const bcg::CudaError& e) {
        bcg::set_last_error(e.what());
        return BCG_ERR_CUDA;
    } catch (const std::exception& e) {
        bcg::set_last_error(e.what());
        return BCG_ERR_INVALID;
    }
}
