// Definitions behind the opaque C ABI handles, shared by the C ABI sources.
#pragma once

#include <memory>
#include <new>
#include <stdexcept>

#include "engine.hpp"
#include "plan.hpp"
#include "../../include/bytecrt_gb300.h"

struct bcg_plan {
    bcg::HostPlan plan;
};

struct bcg_context {
    std::unique_ptr<bcg::Context> ctx;
};

namespace bcg {

// Runs f and maps the exception it throws to a BCG_* status code, keeping the
// message for bcg_last_error().  Exceptions never cross the C ABI.
template <class F>
inline int guarded(F&& f) {
    try {
        f();
        return BCG_OK;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return BCG_ERR_INVALID;
    } catch (const DeviceTimeout& e) {
        set_last_error(e.what());
        return BCG_ERR_DEVICE_TIMEOUT;
    } catch (const Busy& e) {
        set_last_error(e.what());
        return BCG_ERR_BUSY;
    } catch (const CudaError& e) {
        set_last_error(e.what());
        return (e.code == cudaErrorMemoryAllocation) ? BCG_ERR_NOMEM : BCG_ERR_CUDA;
    } catch (const std::bad_alloc& e) {
        set_last_error("host allocation failed");
        return BCG_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return BCG_ERR_INVALID;
    }
}

inline void require(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
}

}  // namespace bcg
