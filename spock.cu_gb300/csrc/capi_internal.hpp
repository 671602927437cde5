// Helpers shared by the C ABI translation units (not part of the public interface).
#pragma once

#include <functional>

#include "../../include/spock_gb300.h"
#include "engine.cuh"

namespace spock {
EngineBase *engineOf(spock_solver s);               // throws std::invalid_argument on a null handle
int guardedCall(const std::function<void()> &f);    // exceptions -> SPOCK_E_* codes + spock_last_error()
}  // namespace spock
