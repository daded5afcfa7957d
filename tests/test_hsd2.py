"""Second-order Hilbert-space distance (HilbertSpaceDistance::distance_2nd_order): the CPU
restatement (oracle/pyoracle.py::hsd_2nd_order) against the reference's own value
(tests/golden/deep6_hsd2.npz, PsiDeep with ExactSummation, its only instantiation), the
CUDA path (rbmg_hsd_distance_2nd_order, FP64 per-sample terms) against both, and the
operator square (operators.product) against dense matrices.

Tolerance: d^2 within 1e-9 relative (every per-sample term is FP64); the square of an
operator table exact to rounding against the dense matrix product.
"""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po


def d2_close(d, ref, rtol=1e-9):
    assert abs(d * d - ref * ref) <= rtol * ref * ref + 1e-15, (d, ref)


def dense(op, N):
    P = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1, -1])]
    coef, types, idx = op
    H = np.zeros((2 ** N, 2 ** N), complex)
    for n in range(len(coef)):
        mats = [np.eye(2, dtype=complex) for _ in range(N)]
        for t, i in zip(types[n], idx[n]):
            if i < 0:
                break
            mats[i] = mats[i] @ P[t]
        m = mats[0]
        for q in range(1, N):
            m = np.kron(m, mats[q])
        H += coef[n] * m
    return H


def deep_pair(c):
    b, cn, w, fw = c.deep()
    bp, cnp, wp, fwp = c.deep("pp_")
    return (b, cn, w, fw), (bp, cnp, wp, fwp)


# ----------------------------------------------------------------------------- CPU
def test_restatement_matches_reference():
    c = Case("deep6_hsd2")
    a, p = deep_pair(c)
    psi, pp = po.Deep(c.N, *a, c.prefactor), po.Deep(c.N, *p, 1.0)
    sp = np.arange(2 ** c.N, dtype=np.uint64)[:, None]
    w = np.abs(po.psi_vector(psi)) ** 2
    d = po.hsd_2nd_order(psi, pp, po.Op(*c.op("h2a_")), po.Op(*c.op("h2b_")), sp, w)
    d2_close(d, c.s("hsd2_distance"))


def test_operator_product_matches_dense():
    from rbmongpu_gb300 import operators as ops
    A = ops.heisenberg_chain(4)
    B = ops.tfim_chain(4, 1.0, 0.7)
    C = ops.table([[(1, 0), (2, 0), (3, 1)], [(2, 2), (2, 2)], [(3, 1), (1, 1)], []], [0.3, 1j, -0.5, 2.0])
    for a, b in [(A, B), (B, A), (C, B), (A, C), (C, C)]:
        assert np.abs(dense(ops.product(a, b), 4) - dense(a, 4) @ dense(b, 4)).max() < 1e-13
    # the golden case's square, formed by the same function, is the dense square
    c = Case("deep6_hsd2")
    assert np.abs(dense(c.op("h2b_"), c.N) - np.linalg.matrix_power(dense(c.op("h2a_"), c.N), 2)).max() < 1e-15


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


@gpu
def test_deep_exact_vs_reference():
    import rbmongpu_gb300 as rg
    c = Case("deep6_hsd2")
    a, p = deep_pair(c)
    psi = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), *a, c.prefactor, False, True)
    pp = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), *p, 1.0, False, True)
    hsd = rg.HilbertSpaceDistance(c.N, pp.num_params)
    es = rg.ExactSummation(c.N)
    d2_close(hsd.distance_2nd_order(psi, pp, rg.Operator(*c.op("h2a_")), es), c.s("hsd2_distance"))
    # the square given explicitly (the reference's two operators) gives the same value
    d2_close(hsd.distance_2nd_order(psi, pp, c.op("h2a_"), es, c.op("h2b_")), c.s("hsd2_distance"))


def rbm_pair(seed, N, M, sigma=0.1):
    rng = np.random.default_rng(seed)
    b = sigma * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = sigma * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    bp = b + 1e-2 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    Wp = W + 1e-2 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    return (b, W), (bp, Wp)


@gpu
def test_rbm_exact_vs_restatement():
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300 import operators as ops
    N, M = 8, 16
    (b, W), (bp, Wp) = rbm_pair(5, N, M)
    cf, ty, ix = ops.tfim_chain(N, 1.0, 1.0)
    A = (-0.01j * cf, ty, ix)
    A2 = ops.product(A, A)
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    pp = rg.Psi(np.zeros(N), np.zeros(N), bp, Wp, 1.0, False, True)
    d = rg.HilbertSpaceDistance(N, pp.num_params).distance_2nd_order(psi, pp, A, rg.ExactSummation(N))
    opsi, opp = po.RBM(b, W, 1.0), po.RBM(bp, Wp, 1.0)
    sp = np.arange(2 ** N, dtype=np.uint64)[:, None]
    ref = po.hsd_2nd_order(opsi, opp, po.Op(*A), po.Op(*A2), sp, np.abs(po.psi_vector(opsi)) ** 2)
    d2_close(d, ref)


@gpu
def test_rbm_monte_carlo_vs_restatement_on_same_samples():
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300 import operators as ops
    N, M = 16, 32
    (b, W), (bp, Wp) = rbm_pair(6, N, M)
    cf, ty, ix = ops.tfim_chain(N, 1.0, 0.8)
    A = (-0.01j * cf, ty, ix)
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    pp = rg.Psi(np.zeros(N), np.zeros(N), bp, Wp, 1.0, False, True)
    mk = lambda: rg.MonteCarloLoop(1024, 1, 5, 256, True, seed=9)   # noqa: E731
    sp, _, _ = mk().samples(psi)
    d = rg.HilbertSpaceDistance(N, pp.num_params).distance_2nd_order(psi, pp, A, mk())
    ref = po.hsd_2nd_order(po.RBM(b, W, 1.0), po.RBM(bp, Wp, 1.0), po.Op(*A), po.Op(*ops.product(A, A)), sp)
    d2_close(d, ref)
