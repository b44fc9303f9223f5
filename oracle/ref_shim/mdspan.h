// The subset of std::mdspan that the reference's include/dynamic_array.h
// uses, for compiling the reference's own sources in the cross-check build
// (dynamic_array.h includes "mdspan.h" when USE_REFERENCE_MDSPAN is defined;
// GCC 13 has no <mdspan>).  Dynamic extents only: std::dextents<I, R>,
// std::mdspan<T, E> with the row-major layout, std::mdspan<T, E,
// std::layout_stride> with explicit strides, and the members the reference
// calls (extent, rank, data_handle, mapping().stride, operator[] of rank 1).
// Written for this build; not a general implementation.
#pragma once
#include <array>
#include <cstddef>
#include <type_traits>

namespace std {

template <class I, size_t R>
class dextents_ref {
  public:
    using index_type = I;
    using rank_type = size_t;
    static constexpr size_t rank() { return R; }
    constexpr dextents_ref() : e_{} {}
    template <class... J, class = enable_if_t<sizeof...(J) == R && (is_convertible_v<J, I> && ...)>>
    constexpr dextents_ref(J... j) : e_{static_cast<I>(j)...} {}
    template <class J>
    constexpr explicit dextents_ref(const array<J, R>& a) : e_{} {
        for (size_t i = 0; i < R; ++i) e_[i] = static_cast<I>(a[i]);
    }
    constexpr I extent(size_t r) const { return e_[r]; }

  private:
    array<I, R> e_;
};

template <class I, size_t R>
using dextents = dextents_ref<I, R>;

struct layout_right {
    template <class E>
    class mapping {
      public:
        constexpr mapping() = default;
        constexpr mapping(const E& e) : e_(e) {}
        constexpr const E& extents() const { return e_; }
        constexpr size_t stride(size_t r) const {
            size_t s = 1;
            for (size_t k = r + 1; k < E::rank(); ++k) s *= e_.extent(k);
            return s;
        }
        template <class... J>
        constexpr size_t operator()(J... j) const {
            const array<size_t, sizeof...(J)> idx{static_cast<size_t>(j)...};
            size_t off = 0;
            for (size_t k = 0; k < sizeof...(J); ++k) off = off * e_.extent(k) + idx[k];
            return off;
        }

      private:
        E e_{};
    };
};

struct layout_stride {
    template <class E>
    class mapping {
      public:
        constexpr mapping() = default;
        template <class J>
        constexpr mapping(const E& e, const array<J, E::rank()>& s) : e_(e), s_{} {
            for (size_t k = 0; k < E::rank(); ++k) s_[k] = static_cast<size_t>(s[k]);
        }
        constexpr const E& extents() const { return e_; }
        constexpr size_t stride(size_t r) const { return s_[r]; }
        template <class... J>
        constexpr size_t operator()(J... j) const {
            const array<size_t, sizeof...(J)> idx{static_cast<size_t>(j)...};
            size_t off = 0;
            for (size_t k = 0; k < sizeof...(J); ++k) off += idx[k] * s_[k];
            return off;
        }

      private:
        E e_{};
        array<size_t, E::rank()> s_{};
    };
};

template <class T, class E, class L = layout_right>
class mdspan {
  public:
    using element_type = T;
    using value_type = remove_cv_t<T>;
    using extents_type = E;
    using layout_type = L;
    using mapping_type = typename L::template mapping<E>;
    using index_type = typename E::index_type;
    using reference = T&;
    static constexpr size_t rank() { return E::rank(); }

    constexpr mdspan() = default;
    constexpr mdspan(T* p, const E& e) : p_(p), m_(e) {}
    constexpr mdspan(T* p, const mapping_type& m) : p_(p), m_(m) {}
    template <class... J, class = enable_if_t<sizeof...(J) == E::rank() && (is_convertible_v<J, size_t> && ...)>>
    constexpr mdspan(T* p, J... j) : p_(p), m_(E(j...)) {}

    constexpr T* data_handle() const { return p_; }
    constexpr const mapping_type& mapping() const { return m_; }
    constexpr const E& extents() const { return m_.extents(); }
    constexpr index_type extent(size_t r) const { return m_.extents().extent(r); }
    constexpr size_t size() const {
        size_t n = 1;
        for (size_t k = 0; k < E::rank(); ++k) n *= extent(k);
        return n;
    }
    template <class J, class = enable_if_t<E::rank() == 1 && is_convertible_v<J, size_t>>>
    constexpr T& operator[](J i) const { return p_[m_(i)]; }

  private:
    T* p_ = nullptr;
    mapping_type m_{};
};

}  // namespace std
