// ref_unbuilt.cpp -- placeholders for the two reference functions whose translation units
// need libraries absent here (src/io/xdmf.cpp: pugixml; src/operators/eigenvalue_visitor.cpp:
// lapackpp).  Other reference units refer to them (field output, the eigenvalue system), but
// nothing on the path that oracle/ref_driver.cpp drives calls them; if anything did, the
// call would throw instead of running.
//
// TEST INFRASTRUCTURE ONLY (compiled into oracle/_ref by oracle/build_ref.sh).
#include "io/xdmf.hpp"
#include "operators/eigenvalue_visitor.hpp"

#include <stdexcept>

namespace ccs
{
void xdmf::write(int, real, std::span<const std::string>, std::span<const std::string>,
                 std::array<std::span<const mesh_object_info>, 3>, const logs&) const
{
    throw std::logic_error("xdmf::write is not built into oracle/_ref (needs pugixml)");
}

void eigenvalue_visitor::visit(const derivative&)
{
    throw std::logic_error("eigenvalue_visitor is not built into oracle/_ref (needs lapackpp)");
}

std::span<const real> eigenvalue_visitor::eigenvalues_real() const
{
    throw std::logic_error("eigenvalue_visitor is not built into oracle/_ref (needs lapackpp)");
}

std::span<const real> eigenvalue_visitor::eigenvalues_imag() const
{
    throw std::logic_error("eigenvalue_visitor is not built into oracle/_ref (needs lapackpp)");
}
} // namespace ccs
