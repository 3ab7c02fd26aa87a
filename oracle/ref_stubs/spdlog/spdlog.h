// Minimal no-op stand-in for spdlog, used only to compile the reference's own translation
// units into oracle/_ref for pinning the oracle (TEST INFRASTRUCTURE ONLY).  Loggers are
// constructible and accept messages; nothing is written.
#pragma once
#include <functional>
#include <memory>
#include <optional>
#include <string>
#include <utility>
#include <vector>
namespace spdlog
{
namespace level
{
enum level_enum { trace, debug, info, warn, err, critical, off };
}
namespace sinks
{
struct sink {
    virtual ~sink() = default;
};
} // namespace sinks
using sink_ptr = std::shared_ptr<sinks::sink>;
struct logger {
    logger() = default;
    template <typename... S>
    logger(const std::string&, S&&...)
    {
    }
    template <typename... A>
    void log(A&&...)
    {
    }
    template <typename... A>
    void info(A&&...)
    {
    }
    template <typename... A>
    void error(A&&...)
    {
    }
    void set_pattern(const std::string&) {}
    void flush() {}
};
template <typename... A>
void info(A&&...)
{
}
inline std::shared_ptr<logger> get(const std::string&) { return nullptr; }
inline void register_logger(std::shared_ptr<logger>) {}
inline void drop(const std::string&) {}
inline void set_pattern(const std::string&) {}
template <typename... A>
void error(A&&...)
{
}
template <typename... A>
void warn(A&&...)
{
}
} // namespace spdlog
