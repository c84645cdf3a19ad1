// TEST INFRASTRUCTURE -- stand-in header for compiling the reference's own
// sources into the oracle's checker (oracle/build_ref.py).
//
// The part of blitz++ that the reference's Riemann-solver adapters use
// (sourcecode/pure_RS_exact.cpp, sourcecode/mixed_RS_exact.cpp): a
// one-dimensional double array of a given length with element access and
// assignment.  Written for this project.
#pragma once

#include <vector>

namespace blitz {

template <typename T, int N>
class Array {
  static_assert(N == 1, "only one-dimensional arrays are used");

 public:
  Array() {}
  explicit Array(int n) : v_(n) {}
  T& operator()(int k) { return v_[k]; }
  const T& operator()(int k) const { return v_[k]; }
  int extent(int) const { return static_cast<int>(v_.size()); }
  const T* data() const { return v_.data(); }
  T* data() { return v_.data(); }

 private:
  std::vector<T> v_;
};

}  // namespace blitz
