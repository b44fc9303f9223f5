// Declaration-only stand-in: Brent minimisation is used by potentials that
// the cross-check never constructs; calling it throws.
#pragma once
#include <stdexcept>
#include <utility>
namespace boost { namespace math { namespace tools {
template <class F, class T>
std::pair<T, T> brent_find_minima(F, T, T, int) { throw std::logic_error("brent_find_minima is not available"); }
template <class F, class T, class I>
std::pair<T, T> brent_find_minima(F, T, T, int, I&) { throw std::logic_error("brent_find_minima is not available"); }
} } }
