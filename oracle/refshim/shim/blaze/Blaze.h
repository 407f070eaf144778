// Minimal stand-in for the Blaze types that NLMech's util/matrixBlaze.h names.
//
// TEST INFRASTRUCTURE ONLY (oracle/refshim): lets the reference's own
// RNPBond / Neighbor / Fracture sources compile without the Blaze library.
// Only what those sources touch is provided: element access on a 3x3 static
// matrix, a 3-vector built from an initializer list, and declarations of the
// dynamic types that appear in typedefs and unused inline helpers.
#pragma once

#include <math.h>
#include <stdint.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <initializer_list>
#include <vector>

namespace blaze {

constexpr bool columnVector = false;
constexpr bool rowVector = true;

template <class T, bool TF = columnVector>
class DynamicVector {
 public:
  DynamicVector() = default;
  explicit DynamicVector(std::size_t n) : v_(n) {}
  T &operator[](std::size_t i) { return v_[i]; }
  const T &operator[](std::size_t i) const { return v_[i]; }
  std::size_t size() const { return v_.size(); }

 private:
  std::vector<T> v_;
};

template <class T, bool TF>
T dot(const DynamicVector<T, TF> &a, const DynamicVector<T, TF> &b) {
  T s = T();
  for (std::size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}

template <class T, bool SO = false>
class DynamicMatrix {
 public:
  DynamicMatrix() = default;
  DynamicMatrix(std::size_t m, std::size_t n) : m_(m), n_(n), a_(m * n) {}
  T &operator()(std::size_t i, std::size_t j) { return a_[i * n_ + j]; }
  const T &operator()(std::size_t i, std::size_t j) const { return a_[i * n_ + j]; }

 private:
  std::size_t m_ = 0, n_ = 0;
  std::vector<T> a_;
};

template <class MT>
class SymmetricMatrix : public MT {};

template <class T, std::size_t M, std::size_t N, bool SO = false>
class StaticMatrix {
 public:
  StaticMatrix() : a_() {}
  T &operator()(std::size_t i, std::size_t j) { return a_[i * N + j]; }
  const T &operator()(std::size_t i, std::size_t j) const { return a_[i * N + j]; }

 private:
  T a_[M * N];
};

template <class T, std::size_t N, bool TF = columnVector>
class StaticVector {
 public:
  StaticVector() : a_() {}
  StaticVector(std::initializer_list<T> l) : a_() {
    std::size_t i = 0;
    for (const T &v : l)
      if (i < N) a_[i++] = v;
  }
  T &operator[](std::size_t i) { return a_[i]; }
  const T &operator[](std::size_t i) const { return a_[i]; }

 private:
  T a_[N];
};

template <class T>
class IdentityMatrix {};

}  // namespace blaze
