// Stand-in for boost::optional as setup.h uses it (an optional reference
// that tests false and dereferences).  Not Boost code.
#pragma once
#include <stdexcept>
namespace boost {
template <class T> class optional;
template <class T>
class optional<T&> {
    T* p_ = nullptr;
  public:
    optional() = default;
    optional(T& r) : p_(&r) {}
    explicit operator bool() const { return p_ != nullptr; }
    bool operator!() const { return p_ == nullptr; }
    T& operator*() const { if (!p_) throw std::logic_error("empty optional"); return *p_; }
};
}
