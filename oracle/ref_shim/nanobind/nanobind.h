// Test infrastructure (oracle only): a minimal stand-in for the nanobind headers so that
// the reference's hot-path C++ sources compile into a plain shared library without Python.
// Only the pieces those sources touch are provided: nb::capsule, nb::object and the
// ndarray template declared in ndarray.h. Nothing here is used by the GPU product.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <memory>

namespace nanobind {

/// Owner handle: keeps a deleter alive for arrays allocated by the reference.
class capsule {
  public:
    capsule() = default;
    capsule(void* p, void (*deleter)(void*) noexcept)
        : holder_(std::shared_ptr<void>(p, [deleter](void* q) { deleter(q); })) {}
    std::shared_ptr<void> holder_;
};

/// Generic owner object (the reference passes it along as an array owner).
class object {
  public:
    object() = default;
    object(const capsule& c) : holder_(c.holder_) {}
    std::shared_ptr<void> holder_;
};

} // namespace nanobind

#include "ndarray.h"
