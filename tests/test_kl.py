"""KullbackLeibler: the CPU restatement (oracle/pyoracle.py::kl) against the reference's
own value and gradient (tests/golden/rbm6_smatrix.npz: the reference's
source/network_functions/KullbackLeibler.cu compiled in place and instantiated for two
complex RBMs over ExactSummation), and the CUDA path (rbmg_kl_gradient) against both.

Tolerance: value within 1e-9 relative (FP64 log psi); gradient within 1e-5 of its largest
entry (complex64 tanh rows of psi')."""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def setup_case():
    c = Case("rbm6_smatrix")
    b, W = c.rbm()
    bp, Wp = c.rbm("pp_")
    return c, (b, W), (bp, Wp)


# ----------------------------------------------------------------------------- CPU
def test_restatement_matches_reference():
    c, (b, W), (bp, Wp) = setup_case()
    psi, pp = po.RBM(b, W, c.prefactor), po.RBM(bp, Wp, 1.0)
    sp = np.arange(2 ** c.N, dtype=np.uint64)[:, None]
    g, v = po.kl(psi, pp, sp, np.abs(po.psi_vector(psi)) ** 2, nu=float(c.meta("hsd_nu")))
    assert v == pytest.approx(c.s("kl_value"), rel=1e-12)
    assert rel(g, c.o("kl_gradient")) < 1e-12


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


@gpu
def test_rbm_exact_vs_reference():
    import rbmongpu_gb300 as rg
    c, (b, W), (bp, Wp) = setup_case()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    pp = rg.Psi(np.zeros(c.N), np.zeros(c.N), bp, Wp, 1.0, False, True)
    kl = rg.KullbackLeibler(pp.num_params)
    es = rg.ExactSummation(c.N)
    assert kl(psi, pp, es) == pytest.approx(c.s("kl_value"), rel=1e-9)
    g, v = kl.gradient(psi, pp, es, float(c.meta("hsd_nu")))
    assert v == pytest.approx(c.s("kl_grad_value"), rel=1e-9)
    assert rel(g, c.o("kl_gradient")) < 1e-5


@gpu
def test_deep_monte_carlo_vs_restatement_on_same_samples():
    """PsiDeep psi' over an RBM psi's Monte Carlo samples (any pair of kinds)."""
    import rbmongpu_gb300 as rg
    c = Case("deep8_sparse")
    b, cn, w, fw = c.deep()
    pp = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, 1.0, False, True)
    opp = po.Deep(c.N, b, cn, w, fw, 1.0)
    rng = np.random.default_rng(8)
    rb = 0.2 * (rng.normal(size=16) + 1j * rng.normal(size=16))
    rW = 0.2 * (rng.normal(size=(c.N, 16)) + 1j * rng.normal(size=(c.N, 16)))
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), rb, rW, 1.0, False, True)
    mk = lambda: rg.MonteCarloLoop(512, 1, 5, 128, True, seed=21)   # noqa: E731
    sp, _, _ = mk().samples(psi)
    g, v = rg.KullbackLeibler(pp.num_params).gradient(psi, pp, mk(), 1.0)
    og, ov = po.kl(po.RBM(rb, rW, 1.0), opp, sp, None, 1.0)
    assert v == pytest.approx(ov, rel=1e-9)
    assert rel(g, og) < 1e-9    # FP64 O_k rows of the PsiDeep psi'
