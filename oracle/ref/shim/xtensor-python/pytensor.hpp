#pragma once
// Minimal stand-in for the few xt::pytensor members that the RBMonGPU headers use
// (shape(), data(), size(), operator[]), so that their Python-facing constructors
// can be called from the golden-vector harness without xtensor-python.
#include <array>
#include <cstddef>
#include <vector>

namespace xt {

template <typename T, std::size_t D>
struct pytensor {
    std::vector<T> values;
    std::array<long, D> dims{};

    pytensor() = default;
    explicit pytensor(std::array<long, D> shape) : dims(shape) {
        std::size_t n = 1;
        for (long x : shape) n *= static_cast<std::size_t>(x);
        values.resize(n);
    }
    pytensor(std::array<long, D> shape, std::vector<T> data) : values(std::move(data)), dims(shape) {}

    const std::array<long, D>& shape() const { return dims; }
    T* data() { return values.data(); }
    const T* data() const { return values.data(); }
    std::size_t size() const { return values.size(); }
    T& operator[](std::size_t i) { return values[i]; }
    const T& operator[](std::size_t i) const { return values[i]; }
};

}  // namespace xt
