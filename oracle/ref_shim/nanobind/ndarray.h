// Test infrastructure (oracle only): minimal ndarray stand-in. An ndarray is a non-owning
// strided view (data pointer, shape, strides in elements) plus an optional shared owner.
// view() returns an accessor with operator()(i, j, ...) using the strides.
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <vector>

namespace nanobind {

struct numpy {};
struct pytorch {};
struct c_contig {};
struct f_contig {};
template <int N> struct ndim {
    static constexpr int value = N;
};

namespace detail {
template <typename... Ts> struct ndim_of;
template <> struct ndim_of<> {
    static constexpr int value = -1;
};
template <int N, typename... Ts> struct ndim_of<ndim<N>, Ts...> {
    static constexpr int value = N;
};
template <typename T, typename... Ts> struct ndim_of<T, Ts...> {
    static constexpr int value = ndim_of<Ts...>::value;
};
} // namespace detail

template <typename T, int N> class ndarray_view {
  public:
    ndarray_view(T* data, const std::array<size_t, N>& shape, const std::array<int64_t, N>& strides)
        : data_(data), shape_(shape), strides_(strides) {}
    template <typename... Idx> T& operator()(Idx... idx) const {
        static_assert(sizeof...(Idx) == N, "wrong number of indices");
        const size_t ii[] = {static_cast<size_t>(idx)...};
        int64_t off = 0;
        for (int k = 0; k < N; ++k)
            off += static_cast<int64_t>(ii[k]) * strides_[k];
        return data_[off];
    }
    size_t shape(size_t i) const { return shape_[i]; }

  private:
    T* data_;
    std::array<size_t, N> shape_;
    std::array<int64_t, N> strides_;
};

template <typename Framework, typename T, typename... Args> class ndarray {
  public:
    static constexpr int N = detail::ndim_of<Args...>::value;
    static_assert(N > 0, "the shim needs an explicit nb::ndim<N>");

    ndarray() = default;

    // Row-major (C order) view over caller memory.
    ndarray(T* data, size_t ndim_, const size_t* shape, object owner = object(),
            const int64_t* strides = nullptr)
        : data_(data), owner_(owner.holder_) {
        if (static_cast<int>(ndim_) != N)
            throw std::runtime_error("ndarray shim: ndim mismatch");
        for (int k = 0; k < N; ++k)
            shape_[k] = shape[k];
        if (strides) {
            for (int k = 0; k < N; ++k)
                strides_[k] = strides[k];
        } else {
            int64_t s = 1;
            for (int k = N - 1; k >= 0; --k) {
                strides_[k] = s;
                s *= static_cast<int64_t>(shape_[k]);
            }
        }
    }
    ndarray(T* data, size_t ndim_, const size_t* shape, capsule owner)
        : ndarray(data, ndim_, shape, object(owner)) {}

    T* data() const { return data_; }
    size_t shape(size_t i) const { return shape_[i]; }
    int64_t stride(size_t i) const { return strides_[i]; }
    size_t ndim() const { return N; }
    size_t size() const {
        size_t s = 1;
        for (int k = 0; k < N; ++k)
            s *= shape_[k];
        return s;
    }
    ndarray_view<T, N> view() const { return ndarray_view<T, N>(data_, shape_, strides_); }
    object cast() const {
        object o;
        o.holder_ = owner_;
        return o;
    }

  private:
    T* data_ = nullptr;
    std::array<size_t, N> shape_{};
    std::array<int64_t, N> strides_{};
    std::shared_ptr<void> owner_;
};

} // namespace nanobind
