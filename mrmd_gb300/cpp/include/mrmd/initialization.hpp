// Drop-in mrmd::initialize / mrmd::finalize (initialization.hpp,
// initialization.cpp:23-44).  The reference starts and stops Kokkos there;
// here initialize() creates the process-wide context on device 0 (every
// drop-in call would create it on first use anyway) and finalize() waits for
// the context's stream.  The context itself lives until the process exits,
// as the drop-in objects that a driver still holds release through it.
#pragma once

#include "datatypes.hpp"

namespace mrmd
{
inline void initialize(int /*argc*/, char** /*argv*/) { (void)gb300::context(); }
inline void initialize() { (void)gb300::context(); }
inline void finalize() { gb300::check(mrmd_ctx_sync(gb300::context()), "finalize"); }
}  // namespace mrmd
