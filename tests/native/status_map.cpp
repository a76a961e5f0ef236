// Host-only check of how a kernel's device status word reaches a C ABI
// caller: the word the host reads back (engine.hpp raise_device_status) is
// turned into an exception, and the C ABI boundary (capi_internal.hpp
// guarded) maps it to its status code and message.  Exits non-zero on the
// first mismatch.
#include "capi_internal.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>

#define REQUIRE(cond)                                                      \
    do {                                                                   \
        if (!(cond)) {                                                     \
            std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #cond); \
            std::exit(1);                                                  \
        }                                                                  \
    } while (0)

int main() {
    // Status 0: no error, the call succeeds.
    REQUIRE(bcg::guarded([] { bcg::raise_device_status(0); }) == BCG_OK);
    // A wait that ran out (kStatusWaitTimeout = 1) and any other non-zero word.
    for (uint32_t st : {1u, 2u, 0xffffffffu}) {
        const int rc = bcg::guarded([st] { bcg::raise_device_status(st); });
        REQUIRE(rc == BCG_ERR_DEVICE_TIMEOUT);
        REQUIRE(std::strstr(bcg::last_error(), "bounded wait ran out") != nullptr);
        REQUIRE(std::strstr(bcg::last_error(), std::to_string(st).c_str()) != nullptr);
    }
    // The other exception kinds keep their own codes.
    REQUIRE(bcg::guarded([] { throw std::invalid_argument("x"); }) == BCG_ERR_INVALID);
    REQUIRE(bcg::guarded([] { throw bcg::Busy("x"); }) == BCG_ERR_BUSY);
    REQUIRE(bcg::guarded([] { throw bcg::CudaError("x", cudaErrorLaunchFailure); }) == BCG_ERR_CUDA);
    REQUIRE(bcg::guarded([] { throw bcg::CudaError("x", cudaErrorMemoryAllocation); }) == BCG_ERR_NOMEM);
    std::printf("ok\n");
    return 0;
}
