// No-op stand-in for Kokkos::Profiling::ScopedRegion (TEST INFRASTRUCTURE ONLY; see
// Kokkos_Core.hpp).
#pragma once

#include <string>

namespace Kokkos::Profiling
{
struct ScopedRegion {
    explicit ScopedRegion(const std::string&) {}
    ScopedRegion(const ScopedRegion&) = delete;
};
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
} // namespace Kokkos::Profiling
