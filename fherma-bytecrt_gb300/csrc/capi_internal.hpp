// Definitions behind the opaque C ABI handles, shared by the C ABI sources.
#pragma once

#include <memory>

#include "engine.hpp"
#include "plan.hpp"

struct bcg_plan {
    bcg::HostPlan plan;
};

struct bcg_context {
    std::unique_ptr<bcg::Context> ctx;
};
