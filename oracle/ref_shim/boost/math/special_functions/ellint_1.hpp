// Stand-in: elliptic integrals appear only in potentials the cross-check
// never constructs; calling one throws.
#pragma once
#include <stdexcept>
namespace boost { namespace math {
template <class T> T ellint_1(T) { throw std::logic_error("ellint_1 is not available"); }
} }
