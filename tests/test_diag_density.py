"""DiagDensityOp: the CPU restatement (oracle/pyoracle.py::diag_density) against the
reference's own densities (tests/golden/deep6_hsd2.npz, PsiDeep with ExactSummation),
and the CUDA path (rbmg_diag_density) against both.

Tolerance: 1e-9 relative for the FP64 PsiDeep path; 1e-5 for the complex64 RBM path.
"""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def golden():
    c = Case("deep6_hsd2")
    return c, c.o("diag_density").view(np.float64)


# ----------------------------------------------------------------------------- CPU
def test_restatement_matches_reference():
    c, ref = golden()
    b, cn, w, fw = c.deep()
    psi = po.Deep(c.N, b, cn, w, fw, c.prefactor)
    sp = np.arange(2 ** c.N, dtype=np.uint64)[:, None]
    d = po.diag_density(psi, po.Op(*c.op()), sp, 3, np.abs(po.psi_vector(psi)) ** 2)
    assert rel(d, ref) < 1e-12


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


@gpu
def test_deep_exact_vs_reference():
    import rbmongpu_gb300 as rg
    c, ref = golden()
    b, cn, w, fw = c.deep()
    psi = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    d = rg.DiagDensityOp(3)(psi, rg.Operator(*c.op()), rg.ExactSummation(c.N))
    assert rel(d, ref) < 1e-9


@gpu
@pytest.mark.parametrize("na", [0, 4, 13])
def test_rbm_monte_carlo_vs_restatement(na):
    """13 spins: 8192 bins, beyond the shared-memory histogram (global atomics)."""
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300 import operators as ops
    rng = np.random.default_rng(17)
    N, M = 16, 32
    b = 0.1 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = 0.1 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    op = ops.tfim_chain(N, 1.0, 0.9)
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    mk = lambda: rg.MonteCarloLoop(2048, 1, 5, 512, True, seed=4)   # noqa: E731
    sp, _, _ = mk().samples(psi)
    d = rg.DiagDensityOp(na)(psi, rg.Operator(*op), mk())
    ref = po.diag_density(po.RBM(b, W, 1.0), po.Op(*op), sp, na)
    assert rel(d, ref) < 1e-5
    assert d.sum() == pytest.approx(ref.sum(), rel=1e-5)


@gpu
def test_rbm_exact_vs_restatement():
    import rbmongpu_gb300 as rg
    c = Case("c1_rbm_exact")
    b, W = c.rbm()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    opsi = po.RBM(b, W, c.prefactor)
    sp = np.arange(2 ** c.N, dtype=np.uint64)[:, None]
    d = rg.DiagDensityOp(5)(psi, rg.Operator(*c.op()), rg.ExactSummation(c.N))
    ref = po.diag_density(opsi, po.Op(*c.op()), sp, 5, np.abs(po.psi_vector(opsi)) ** 2)
    assert rel(d, ref) < 1e-5
