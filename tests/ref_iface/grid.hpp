// Test-only stand-in for the reference's host grid type (mworchel/fluid-2d
// src/grid.hpp:8-66), used to build include/fluid_solver_gb300.hpp where the
// reference checkout is absent. Same shape of interface: row-major storage,
// (rows, cols, init) constructor, rows()/cols()/data() and (i, j) element access.
#pragma once

#include <cstddef>
#include <vector>

template <typename T>
class grid {
public:
    grid(std::size_t rows, std::size_t cols, T init) : r_(rows), c_(cols), v_(rows * cols, init) {}
    std::size_t rows() const { return r_; }
    std::size_t cols() const { return c_; }
    T* data() { return v_.data(); }
    const T* data() const { return v_.data(); }
    T& operator()(std::size_t i, std::size_t j) { return v_[i * c_ + j]; }
    T operator()(std::size_t i, std::size_t j) const { return v_[i * c_ + j]; }

private:
    std::size_t r_, c_;
    std::vector<T> v_;
};
