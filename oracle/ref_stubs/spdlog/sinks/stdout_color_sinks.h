// No-op stand-in for spdlog's console sink (TEST INFRASTRUCTURE ONLY; see spdlog.h).
#pragma once
#include "../spdlog.h"
namespace spdlog::sinks
{
struct stdout_color_sink_st : sink {
    template <typename... A>
    explicit stdout_color_sink_st(A&&...)
    {
    }
};
using stdout_color_sink_mt = stdout_color_sink_st;
} // namespace spdlog::sinks
