// No-op stand-in for spdlog's file sink (TEST INFRASTRUCTURE ONLY; see spdlog.h).
#pragma once
#include "../spdlog.h"
namespace spdlog::sinks
{
struct basic_file_sink_st : sink {
    template <typename... A>
    explicit basic_file_sink_st(A&&...)
    {
    }
};
using basic_file_sink_mt = basic_file_sink_st;
} // namespace spdlog::sinks
