// Stand-in: Bessel functions appear only in potentials the cross-check never
// constructs; calling one throws.
#pragma once
#include <stdexcept>
namespace boost { namespace math {
template <class T1, class T2> double cyl_bessel_k(T1, T2) { throw std::logic_error("cyl_bessel_k is not available"); }
} }
