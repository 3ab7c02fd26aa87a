// Minimal no-op stand-in for spdlog, used only to compile a few of the reference's own
// translation units (stencils, sphere) into oracle/_ref for pinning the oracle.
#pragma once
#include <memory>
#include <utility>
#include <optional>
#include <vector>
#include <functional>
#include <string>
namespace spdlog
{
namespace level
{
enum level_enum { trace, debug, info, warn, err, critical, off };
}
struct logger {
    template <typename... A>
    void log(A&&...)
    {
    }
};
} // namespace spdlog
