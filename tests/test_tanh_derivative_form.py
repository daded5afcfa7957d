"""The derivative form of the activation's tanh used by the fused evaluation of f and tanh
(rbmongpu_gb300/csrc/device_math.cuh: lc_tanh_approx, in the serving kernel and the
gradient estimator pass): tanh(z) = s g'(u), u = s z, s = sign(Re z),
g(u) = A u + N(u) / D(u) - C, N = NA - NB u, D the quartic of the log-cosh denominator,
g'(u) = A + (-NB - N D' / D) / D.

Against the oracle's restatement of the reference's my_tanh
(include/quantum_state/psi_functions.hpp:97-114), whose rational form differs only in the
last digits of one constant: FP64 to 1e-10 relative, and the FP32 operation order of the
kernel (emulated with numpy float32, the approximate reciprocal as the rounded quotient)
to 1e-5 of |tanh|."""
import os
import re

import numpy as np
import pytest

from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))


def constants():
    src = open(os.path.join(HERE, "..", "rbmongpu_gb300", "csrc", "device_math.cuh")).read()
    c = dict(re.findall(r"constexpr float LC_(\w+) = ([0-9.]+)f;", src))
    return {k: float(v) for k, v in c.items()}


def tanh_derivative(z, c, dtype=np.float64):
    """The kernel's sequence of operations in the given precision."""
    f = dtype
    x, y = f(z.real), f(z.imag)
    s = f(1.0) if x > 0 else f(-1.0)
    p, q = s * x, s * y
    # D(u) = ((u + D3) u + D2) u + D1) u + D0
    t1r = p + f(c["D3"])
    t2r = p * t1r + (f(c["D2"]) - q * q)
    t2i = p * q + q * t1r
    t3r = p * t2r + (f(c["D1"]) - q * t2i)
    t3i = p * t2i + q * t2r
    dr = p * t3r + (f(c["D0"]) - q * t3i)
    di = p * t3i + q * t3r
    nr = f(c["NA"]) - f(c["NB"]) * p
    ni = -f(c["NB"]) * q
    inv = f(1.0) / (dr * dr + di * di)
    # D'(u) = ((4 u + 3 D3) u + 2 D2) u + D1
    ar, ai = f(4.0) * p + f(3.0) * f(c["D3"]), f(4.0) * q
    ar, ai = p * ar - q * ai, p * ai + q * ar
    ar = ar + f(2.0) * f(c["D2"])
    ar, ai = p * ar - q * ai, p * ai + q * ar
    ar = ar + f(c["D1"])
    ndr, ndi = nr * ar - ni * ai, nr * ai + ni * ar
    wr, wi = (ndr * dr + ndi * di) * inv, (ndi * dr - ndr * di) * inv
    mr, mi = -f(c["NB"]) - wr, -wi
    return complex(s * (f(c["A"]) + (mr * dr + mi * di) * inv), s * ((mi * dr - mr * di) * inv))


def points():
    rng = np.random.default_rng(12)
    z = list(rng.normal(0, 0.3, 400) + 1j * rng.normal(0, 0.3, 400))
    z += list(rng.normal(0, 3.0, 400) + 1j * rng.normal(0, 3.0, 400))
    z += [0.7 + 0.0j, -0.7 + 0.2j, 1e-3 - 2.0j, -5.0 + 5.0j, 12.0 - 0.5j]
    return z


def test_constants_are_the_reference_activation_constants():
    c = constants()
    assert set(c) >= {"A", "NA", "NB", "D0", "D1", "D2", "D3", "C"}
    # f(z) = g(s z) of the kernels is the oracle's restated my_logcosh
    for z in points()[:50]:
        s = 1.0 if z.real > 0 else -1.0
        u = s * z
        D = (((u + c["D3"]) * u + c["D2"]) * u + c["D1"]) * u + c["D0"]
        g = c["A"] * u + (c["NA"] - c["NB"] * u) / D - c["C"]
        assert abs(g - po.logcosh(z)) <= 1e-9 * max(1.0, abs(g))


def test_fp64_derivative_form_is_the_reference_tanh():
    c = constants()
    for z in points():
        ref = po.tanh(z)
        got = tanh_derivative(z, c)
        assert abs(got - ref) <= 1e-10 * max(abs(ref), 1e-3), (z, got, ref)


def test_fp32_operation_order_stays_within_tolerance():
    c = constants()
    worst = 0.0
    for z in points():
        ref = po.tanh(z)
        got = tanh_derivative(z, c, np.float32)
        worst = max(worst, abs(got - ref) / max(abs(ref), 1e-2))
    assert worst < 1e-5, worst
