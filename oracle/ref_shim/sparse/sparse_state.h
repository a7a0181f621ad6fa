// Test infrastructure (oracle only): stand-in for the reference's SparseState so that its
// sigma-builder translation unit compiles without the sparse-operator subsystem. The oracle
// never calls make_sparse_state; this type only has to support state[det] = value.
#pragma once

#include <unordered_map>

#include "determinant/determinant.h"

namespace forte2 {
class SparseState {
  public:
    double& operator[](const Determinant& d) { return map_[d]; }

  private:
    std::unordered_map<Determinant, double, Determinant::Hash> map_;
};
} // namespace forte2
