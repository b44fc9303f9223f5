// A minimal owning pointer vector with boost::ptr_vector's interface as the
// reference uses it (push_back of a raw pointer, element access and
// iteration by reference), for the cross-check build.  Not Boost code.
#pragma once
#include <cstddef>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <vector>

namespace boost {

template <class T>
class ptr_vector {
    std::vector<std::unique_ptr<T>> v_;

  public:
    template <class Base, class Ref>
    class iter_t {
        Base it_;
      public:
        using iterator_category = std::random_access_iterator_tag;
        using value_type = T;
        using difference_type = std::ptrdiff_t;
        using pointer = std::remove_reference_t<Ref>*;
        using reference = Ref;
        iter_t() = default;
        explicit iter_t(Base it) : it_(it) {}
        Ref operator*() const { return **it_; }
        pointer operator->() const { return it_->get(); }
        iter_t& operator++() { ++it_; return *this; }
        iter_t operator++(int) { iter_t t = *this; ++it_; return t; }
        iter_t& operator--() { --it_; return *this; }
        iter_t& operator+=(difference_type n) { it_ += n; return *this; }
        iter_t operator+(difference_type n) const { return iter_t(it_ + n); }
        iter_t operator-(difference_type n) const { return iter_t(it_ - n); }
        difference_type operator-(const iter_t& o) const { return it_ - o.it_; }
        bool operator==(const iter_t& o) const { return it_ == o.it_; }
        bool operator!=(const iter_t& o) const { return it_ != o.it_; }
        bool operator<(const iter_t& o) const { return it_ < o.it_; }
    };
    using iterator = iter_t<typename std::vector<std::unique_ptr<T>>::iterator, T&>;
    using const_iterator = iter_t<typename std::vector<std::unique_ptr<T>>::const_iterator, const T&>;
    using size_type = std::size_t;

    ptr_vector() = default;
    ptr_vector(const ptr_vector&) = delete;
    ptr_vector& operator=(const ptr_vector&) = delete;
    ptr_vector(ptr_vector&&) = default;
    ptr_vector& operator=(ptr_vector&&) = default;

    void push_back(T* p) { v_.emplace_back(p); }
    size_type size() const { return v_.size(); }
    bool empty() const { return v_.empty(); }
    T& operator[](size_type i) { return *v_[i]; }
    const T& operator[](size_type i) const { return *v_[i]; }
    T& at(size_type i) { if (i >= v_.size()) throw std::out_of_range("ptr_vector"); return *v_[i]; }
    const T& at(size_type i) const { if (i >= v_.size()) throw std::out_of_range("ptr_vector"); return *v_[i]; }
    T& front() { return *v_.front(); }
    const T& front() const { return *v_.front(); }
    T& back() { return *v_.back(); }
    const T& back() const { return *v_.back(); }
    iterator begin() { return iterator(v_.begin()); }
    iterator end() { return iterator(v_.end()); }
    const_iterator begin() const { return const_iterator(v_.begin()); }
    const_iterator end() const { return const_iterator(v_.end()); }
    void clear() { v_.clear(); }
};

}  // namespace boost
