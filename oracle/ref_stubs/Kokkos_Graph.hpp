// Serial stand-in for Kokkos::Experimental graphs (create_graph, then_parallel_for,
// when_all, instantiate, submit).
//
// TEST INFRASTRUCTURE ONLY (see Kokkos_Core.hpp).  A node's body is recorded when the node
// is created and submit() runs the bodies in creation order.  A node can only be created
// after its predecessors, so creation order is a topological order of the graph; nodes
// without a path between them write disjoint buffers in the reference, so any order of
// them gives the same results.
#pragma once

#include "Kokkos_Core.hpp"

#include <functional>
#include <memory>
#include <string>
#include <vector>

namespace Kokkos::Experimental
{

namespace detail
{
struct graph_state {
    std::vector<std::function<void()>> bodies;
};
} // namespace detail

struct GraphNodeRef {
    std::shared_ptr<detail::graph_state> g;

    template <typename Policy, typename F>
    GraphNodeRef then_parallel_for(const std::string&, const Policy& p, F f) const
    {
        g->bodies.emplace_back([p, f]() { Kokkos::parallel_for(p, f); });
        return *this;
    }

    template <typename Policy, typename F>
    GraphNodeRef then_parallel_for(const Policy& p, F f) const
    {
        g->bodies.emplace_back([p, f]() { Kokkos::parallel_for(p, f); });
        return *this;
    }

    template <typename F>
    GraphNodeRef then(const std::string&, F f) const
    {
        g->bodies.emplace_back([f]() { f(); });
        return *this;
    }
};

template <typename... N>
GraphNodeRef when_all(const GraphNodeRef& first, const N&...)
{
    return first;
}

template <typename ES>
class Graph
{
    std::shared_ptr<detail::graph_state> g_ = std::make_shared<detail::graph_state>();

public:
    Graph() = default;

    GraphNodeRef root_node() const { return GraphNodeRef{g_}; }
    void instantiate() {}
    void submit() const
    {
        for (auto& b : g_->bodies) b();
    }
    void submit(const ES&) const { submit(); }
};

template <typename ES, typename Closure>
Graph<ES> create_graph(Closure&& c)
{
    Graph<ES> g;
    c(g.root_node());
    return g;
}

template <typename ES, typename Closure>
Graph<ES> create_graph(const ES&, Closure&& c)
{
    return create_graph<ES>(c);
}

} // namespace Kokkos::Experimental
