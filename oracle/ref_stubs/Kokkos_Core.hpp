// Serial stand-in for the small part of Kokkos that the reference's hot-path translation
// units use (View, RangePolicy, TeamPolicy with team/vector ranges, parallel_for,
// parallel_reduce, deep_copy, mirrors, fence, graphs, profiling regions).
//
// TEST INFRASTRUCTURE ONLY: lets oracle/build_ref.sh compile the reference's own sources
// unmodified into oracle/_ref so that the oracle restatement can be pinned to them.
// Everything runs on the calling thread in index order, which is also the order in which
// the Kokkos host backends evaluate a sum inside one matrix row (ThreadVectorRange and the
// serial loop of a RangePolicy body), so results are the reference's own arithmetic.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [ =, *this ]
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_FORCEINLINE_FUNCTION inline

namespace Kokkos
{

struct HostSpace {
    using memory_space = HostSpace;
};

struct Serial {
    using memory_space = HostSpace;
    using execution_space = Serial;
    using size_type = std::size_t;
    static void fence(const std::string& = {}) {}
};

using DefaultHostExecutionSpace = Serial;
using DefaultExecutionSpace = Serial;

enum MemoryTraitsFlags : unsigned { Unmanaged = 1u, RandomAccess = 2u, Atomic = 4u };
template <unsigned F>
struct MemoryTraits {
    static constexpr unsigned flags = F;
};
using MemoryUnmanaged = MemoryTraits<Unmanaged>;

struct AUTO_t {
};
inline constexpr AUTO_t AUTO{};

inline void fence(const std::string& = {}) {}

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline bool is_initialized() { return true; }

struct ScopeGuard {
    ScopeGuard() = default;
    ScopeGuard(int&, char**) {}
    ScopeGuard(const ScopeGuard&) = delete;
};

template <typename T>
KOKKOS_INLINE_FUNCTION T abs(T x)
{
    return std::abs(x);
}

// ---------------------------------------------------------------------------
// View: rank-1 only (the reference's non-test sources use no other rank).
// ---------------------------------------------------------------------------
template <typename DataType, typename... Props>
class View;

template <typename T, typename... Props>
class View<T*, Props...>
{
    template <typename, typename...>
    friend class View;

public:
    using value_type = T;
    using non_const_value_type = std::remove_const_t<T>;
    using const_value_type = const non_const_value_type;
    using pointer_type = T*;
    using reference_type = T&;
    using data_type = T*;
    using memory_space = HostSpace;
    using execution_space = Serial;
    using HostMirror = View<T*, Props...>;
    using host_mirror_type = HostMirror;
    using size_type = std::size_t;

private:
    std::shared_ptr<non_const_value_type[]> owner_{};
    T* ptr_ = nullptr;
    std::size_t n_ = 0;
    std::string label_{};

public:
    View() = default;

    View(const std::string& label, std::size_t n)
        : owner_(n ? new non_const_value_type[n]() : nullptr), ptr_(owner_.get()), n_(n),
          label_(label)
    {
    }

    View(T* p, std::size_t n) : ptr_(p), n_(n) {}

    template <typename U, typename... P2>
        requires std::is_convertible_v<U*, T*>
    View(const View<U*, P2...>& o) : owner_(o.owner_), ptr_(o.ptr_), n_(o.n_), label_(o.label_)
    {
    }

    T& operator()(std::size_t i) const { return ptr_[i]; }
    T& operator[](std::size_t i) const { return ptr_[i]; }
    T* data() const { return ptr_; }
    std::size_t extent(int r) const { return r == 0 ? n_ : 1; }
    int extent_int(int r) const { return static_cast<int>(extent(r)); }
    std::size_t size() const { return n_; }
    std::size_t span() const { return n_; }
    bool is_allocated() const { return ptr_ != nullptr; }
    const std::string& label() const { return label_; }
    static constexpr int rank = 1;
    static constexpr int rank_dynamic = 1;
};

template <typename V>
V create_mirror_view(const V& v)
{
    return v;
}

template <typename Space, typename V>
V create_mirror_view(const Space&, const V& v)
{
    return v;
}

template <typename V>
V create_mirror_view_and_copy(const HostSpace&, const V& v)
{
    return v;
}

template <typename V>
V create_mirror(const V& v)
{
    V out(v.label(), v.size());
    for (std::size_t i = 0; i < v.size(); ++i) out(i) = v(i);
    return out;
}

template <typename T, typename... P1, typename U, typename... P2>
void deep_copy(const View<T*, P1...>& dst, const View<U*, P2...>& src)
{
    if (static_cast<const void*>(dst.data()) == static_cast<const void*>(src.data())) return;
    const std::size_t n = std::min(dst.size(), src.size());
    for (std::size_t i = 0; i < n; ++i) dst(i) = src(i);
}

template <typename T, typename... P1, typename S>
    requires std::is_arithmetic_v<S>
void deep_copy(const View<T*, P1...>& dst, S value)
{
    for (std::size_t i = 0; i < dst.size(); ++i) dst(i) = value;
}

template <typename ES, typename T, typename... P1, typename U, typename... P2>
void deep_copy(const ES&, const View<T*, P1...>& dst, const View<U*, P2...>& src)
{
    deep_copy(dst, src);
}

template <typename T, typename... P>
void realloc(View<T*, P...>& v, std::size_t n)
{
    v = View<T*, P...>(v.label(), n);
}

template <typename T, typename... P>
void resize(View<T*, P...>& v, std::size_t n)
{
    View<T*, P...> w(v.label(), n);
    const std::size_t m = std::min(n, v.size());
    for (std::size_t i = 0; i < m; ++i) w(i) = v(i);
    v = w;
}

// ---------------------------------------------------------------------------
// Execution policies
// ---------------------------------------------------------------------------
template <typename... Args>
struct IndexType {
};

template <typename... Args>
struct RangePolicy {
    std::int64_t b = 0, e = 0;
    RangePolicy() = default;
    template <typename I, typename J>
    RangePolicy(I begin, J end) : b(static_cast<std::int64_t>(begin)), e(static_cast<std::int64_t>(end))
    {
    }
    template <typename ES, typename I, typename J>
        requires(!std::is_integral_v<ES>)
    RangePolicy(const ES&, I begin, J end)
        : b(static_cast<std::int64_t>(begin)), e(static_cast<std::int64_t>(end))
    {
    }
};

struct TeamMember {
    int league_rank_ = 0;
    int league_size_ = 1;
    int league_rank() const { return league_rank_; }
    int league_size() const { return league_size_; }
    int team_rank() const { return 0; }
    int team_size() const { return 1; }
    void team_barrier() const {}
};

template <typename... Args>
struct TeamPolicy {
    using member_type = TeamMember;
    int league = 0;
    TeamPolicy() = default;
    template <typename A>
    TeamPolicy(int league_size, A) : league(league_size)
    {
    }
    template <typename A, typename B>
    TeamPolicy(int league_size, A, B) : league(league_size)
    {
    }
    template <typename... X>
    TeamPolicy& set_scratch_size(X&&...)
    {
        return *this;
    }
};

template <typename I>
struct NestedRange {
    I b, e;
};

template <typename I>
NestedRange<I> TeamThreadRange(const TeamMember&, I n)
{
    return {I(0), n};
}
template <typename I, typename J>
NestedRange<std::common_type_t<I, J>> TeamThreadRange(const TeamMember&, I b, J e)
{
    return {b, e};
}
template <typename I>
NestedRange<I> ThreadVectorRange(const TeamMember&, I n)
{
    return {I(0), n};
}
template <typename I, typename J>
NestedRange<std::common_type_t<I, J>> ThreadVectorRange(const TeamMember&, I b, J e)
{
    return {b, e};
}
template <typename I>
NestedRange<I> TeamVectorRange(const TeamMember&, I n)
{
    return {I(0), n};
}

struct PerThread_t {
};
struct PerTeam_t {
};
inline PerThread_t PerThread(const TeamMember&) { return {}; }
inline PerTeam_t PerTeam(const TeamMember&) { return {}; }

template <typename F>
void single(PerThread_t, F&& f)
{
    f();
}
template <typename F>
void single(PerTeam_t, F&& f)
{
    f();
}
template <typename F, typename T>
void single(PerThread_t, F&& f, T& v)
{
    f(v);
}

// ---------------------------------------------------------------------------
// parallel_for
// ---------------------------------------------------------------------------
namespace detail
{
template <typename F, typename... Args>
void run_range(const RangePolicy<Args...>& p, F&& f)
{
    for (std::int64_t i = p.b; i < p.e; ++i) f(i);
}
} // namespace detail

template <typename... Args, typename F>
void parallel_for(const RangePolicy<Args...>& p, F&& f)
{
    detail::run_range(p, f);
}

template <typename... Args, typename F>
void parallel_for(const std::string&, const RangePolicy<Args...>& p, F&& f)
{
    detail::run_range(p, f);
}

template <typename I, typename F>
    requires std::is_integral_v<I>
void parallel_for(I n, F&& f)
{
    for (I i = 0; i < n; ++i) f(i);
}

template <typename I, typename F>
    requires std::is_integral_v<I>
void parallel_for(const std::string&, I n, F&& f)
{
    for (I i = 0; i < n; ++i) f(i);
}

template <typename... Args, typename F>
void parallel_for(const TeamPolicy<Args...>& p, F&& f)
{
    for (int l = 0; l < p.league; ++l) f(TeamMember{l, p.league});
}

template <typename... Args, typename F>
void parallel_for(const std::string&, const TeamPolicy<Args...>& p, F&& f)
{
    parallel_for(p, f);
}

template <typename I, typename F>
void parallel_for(const NestedRange<I>& r, F&& f)
{
    for (I i = r.b; i < r.e; ++i) f(i);
}

// ---------------------------------------------------------------------------
// Reducers and parallel_reduce
// ---------------------------------------------------------------------------
template <typename T>
struct MinMaxScalar {
    T min_val, max_val;
};

template <typename T, typename I>
struct ValLocScalar {
    T val;
    I loc;
};

template <typename T, typename I>
struct MinMaxLocScalar {
    T min_val, max_val;
    I min_loc, max_loc;
};

template <typename T, typename S = HostSpace>
struct Sum {
    using value_type = T;
    T& ref;
    explicit Sum(T& r) : ref(r) {}
    void init(T& v) const { v = T(0); }
    void join(T& d, const T& s) const { d += s; }
    T& reference() const { return ref; }
};

template <typename T, typename S = HostSpace>
struct Max {
    using value_type = T;
    T& ref;
    explicit Max(T& r) : ref(r) {}
    void init(T& v) const { v = std::numeric_limits<T>::lowest(); }
    void join(T& d, const T& s) const
    {
        if (s > d) d = s;
    }
    T& reference() const { return ref; }
};

template <typename T, typename S = HostSpace>
struct Min {
    using value_type = T;
    T& ref;
    explicit Min(T& r) : ref(r) {}
    void init(T& v) const { v = std::numeric_limits<T>::max(); }
    void join(T& d, const T& s) const
    {
        if (s < d) d = s;
    }
    T& reference() const { return ref; }
};

template <typename T, typename S = HostSpace>
struct MinMax {
    using value_type = MinMaxScalar<T>;
    value_type& ref;
    explicit MinMax(value_type& r) : ref(r) {}
    void init(value_type& v) const
    {
        v.min_val = std::numeric_limits<T>::max();
        v.max_val = std::numeric_limits<T>::lowest();
    }
    void join(value_type& d, const value_type& s) const
    {
        if (s.min_val < d.min_val) d.min_val = s.min_val;
        if (s.max_val > d.max_val) d.max_val = s.max_val;
    }
    value_type& reference() const { return ref; }
};

template <typename T, typename I, typename S = HostSpace>
struct MaxLoc {
    using value_type = ValLocScalar<T, I>;
    value_type& ref;
    explicit MaxLoc(value_type& r) : ref(r) {}
    void init(value_type& v) const
    {
        v.val = std::numeric_limits<T>::lowest();
        v.loc = std::numeric_limits<I>::max();
    }
    void join(value_type& d, const value_type& s) const
    {
        if (s.val > d.val || (s.val == d.val && s.loc < d.loc)) d = s;
    }
    value_type& reference() const { return ref; }
};

template <typename T, typename I, typename S = HostSpace>
struct MinLoc {
    using value_type = ValLocScalar<T, I>;
    value_type& ref;
    explicit MinLoc(value_type& r) : ref(r) {}
    void init(value_type& v) const
    {
        v.val = std::numeric_limits<T>::max();
        v.loc = std::numeric_limits<I>::max();
    }
    void join(value_type& d, const value_type& s) const
    {
        if (s.val < d.val || (s.val == d.val && s.loc < d.loc)) d = s;
    }
    value_type& reference() const { return ref; }
};

namespace detail
{
template <typename R>
concept Reducer = requires(const R& r, typename R::value_type& v) {
    r.init(v);
    r.reference();
};

// Reduction into a reducer: the body sees a private accumulator that starts at the
// reducer's identity; the result is joined into the reducer's target.
template <typename R, typename Loop>
void reduce_into(const R& red, Loop&& loop)
{
    typename R::value_type acc;
    red.init(acc);
    loop(acc);
    red.reference() = acc;
}
} // namespace detail

template <typename... Args, typename F, typename R>
    requires detail::Reducer<R>
void parallel_reduce(const RangePolicy<Args...>& p, F&& f, const R& red)
{
    detail::reduce_into(red, [&](auto& acc) {
        for (std::int64_t i = p.b; i < p.e; ++i) f(i, acc);
    });
}

template <typename... Args, typename F, typename T>
    requires(!detail::Reducer<T>)
void parallel_reduce(const RangePolicy<Args...>& p, F&& f, T& result)
{
    T acc{};
    for (std::int64_t i = p.b; i < p.e; ++i) f(i, acc);
    result = acc;
}

template <typename... Args, typename F, typename R>
void parallel_reduce(const std::string&, const RangePolicy<Args...>& p, F&& f, R&& r)
{
    parallel_reduce(p, f, r);
}

template <typename I, typename F, typename R>
    requires std::is_integral_v<I> && detail::Reducer<R>
void parallel_reduce(I n, F&& f, const R& red)
{
    parallel_reduce(RangePolicy<>(I(0), n), f, red);
}

template <typename I, typename F, typename T>
    requires std::is_integral_v<I> && (!detail::Reducer<T>)
void parallel_reduce(I n, F&& f, T& result)
{
    parallel_reduce(RangePolicy<>(I(0), n), f, result);
}

template <typename I, typename F, typename T>
    requires(!detail::Reducer<T>)
void parallel_reduce(const NestedRange<I>& r, F&& f, T& result)
{
    T acc{};
    for (I i = r.b; i < r.e; ++i) f(i, acc);
    result = acc;
}

template <typename I, typename F, typename R>
    requires detail::Reducer<R>
void parallel_reduce(const NestedRange<I>& r, F&& f, const R& red)
{
    detail::reduce_into(red, [&](auto& acc) {
        for (I i = r.b; i < r.e; ++i) f(i, acc);
    });
}

struct Timer {
    void reset() {}
    double seconds() const { return 0.0; }
};

} // namespace Kokkos
