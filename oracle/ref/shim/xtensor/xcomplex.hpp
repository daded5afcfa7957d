#pragma once
// Stand-in for xt::real / xt::imag on the pytensor shim (used by PsiPair's constructor).
#include <complex>
#include "xtensor-python/pytensor.hpp"

namespace xt {

template <std::size_t D>
pytensor<double, D> real(const pytensor<std::complex<double>, D>& x) {
    pytensor<double, D> r(x.shape());
    for (std::size_t i = 0; i < x.size(); i++) r[i] = x[i].real();
    return r;
}

template <std::size_t D>
pytensor<double, D> imag(const pytensor<std::complex<double>, D>& x) {
    pytensor<double, D> r(x.shape());
    for (std::size_t i = 0; i < x.size(); i++) r[i] = x[i].imag();
    return r;
}

}  // namespace xt
