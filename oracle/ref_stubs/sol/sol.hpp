// Compile-only stand-in for sol2, so that the reference's translation units that also hold
// a from_lua reader compile unmodified into oracle/_ref (TEST INFRASTRUCTURE ONLY).  The
// readers are never called: oracle/ref_driver.cpp builds every object through its C++
// constructor.  Every lookup reports "not present".
#pragma once
#include "forward.hpp"

#include <optional>
#include <string>
#include <tuple>
#include <utility>

namespace sol
{
template <typename T>
using optional = std::optional<T>;

struct nil_t {
};
inline constexpr nil_t nil{};
enum class type { none, lua_nil, string, number, thread, boolean, function, userdata, table };
enum class lib { base, math, string, table, io, os, package };

struct proxy {
    template <typename K>
    proxy operator[](K&&) const
    {
        return {};
    }
    bool valid() const { return false; }
    type get_type() const { return type::lua_nil; }
    template <typename T>
    T get_or(T d) const
    {
        return d;
    }
    template <typename T, typename D>
    T get_or(D&& d) const
    {
        return T(std::forward<D>(d));
    }
    template <typename T>
    T get() const
    {
        return T{};
    }
    template <typename T>
    bool is() const
    {
        return false;
    }
    template <typename T>
    operator T() const
    {
        return T{};
    }
    template <typename... A>
    proxy operator()(A&&...) const
    {
        return {};
    }
};

using object = proxy;

class table : public proxy
{
public:
    table() = default;
    table(const proxy&) {}
    std::size_t size() const { return 0; }
    template <typename F>
    void for_each(F&&) const
    {
    }
};

class function : public proxy
{
};

class state : public table
{
public:
    template <typename... L>
    void open_libraries(L...)
    {
    }
    proxy script(const std::string&) { return {}; }
};
} // namespace sol
