"""The free-quantum-axis branch of HilbertSpaceDistance (source/network_functions/
HilbertSpaceDistance.cu:47-81, 109-122) on the GPU, against the reference's own outputs
(tests/golden/rbm6_hsd_fqa.npz, deep6_hsd_fqa.npz: a 6-spin RBM and a 6-spin PsiDeep with
random alpha angles, psi' with perturbed ones, beta = alpha as the reference's constructor
sets it), under exact summation, and against the FP64 restatement on Monte Carlo samples.

Tolerances: distances within 1e-6 relative; gradients (alpha, beta and network entries)
within 1e-5 of their largest entry.
"""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def gpu_psi(case, prefix=""):
    import rbmongpu_gb300 as rg
    alpha, fqa = case.quaxis(prefix)
    pf = case.prefactor if prefix == "" else 1.0
    if case.kind == "rbm":
        b, W = case.rbm(prefix)
        return rg.Psi(alpha, alpha, b, W, pf, fqa, True)
    b, c, w, fw = case.deep(prefix)
    return rg.PsiDeep(alpha, alpha, b, c, w, fw, pf, fqa, True)


def oracle_psi(case, prefix=""):
    alpha, fqa = case.quaxis(prefix)
    pf = case.prefactor if prefix == "" else 1.0
    if case.kind == "rbm":
        b, W = case.rbm(prefix)
        return po.RBM(b, W, pf, alpha=alpha, beta=alpha, free_quantum_axis=fqa)
    b, c, w, fw = case.deep(prefix)
    return po.Deep(case.N, b, c, w, fw, pf, alpha=alpha, beta=alpha, free_quantum_axis=fqa)


@pytest.mark.parametrize("name", ["rbm6_hsd_fqa", "deep6_hsd_fqa"])
def test_free_quantum_axis_distance_and_gradient_vs_reference(name):
    import rbmongpu_gb300 as rg
    c = Case(name)
    psi, pp = gpu_psi(c), gpu_psi(c, "pp_")
    assert psi.free_quantum_axis
    hop = rg.Operator(*c.op("hop_"))
    es = rg.ExactSummation(c.N)
    hsd = rg.HilbertSpaceDistance(c.N, psi.num_params)
    unitary = bool(c.meta("hsd_unitary"))
    d = hsd(psi, pp, hop, unitary, es)
    assert d == pytest.approx(c.s("hsd_distance"), rel=1e-6)
    g, d2 = hsd.gradient(psi, pp, hop, unitary, es, float(c.meta("hsd_nu")))
    assert d2 == pytest.approx(c.s("hsd_grad_distance"), rel=1e-6)
    ref = c.o("hsd_gradient")
    assert np.abs(g - ref).max() <= RTOL * np.abs(ref).max()
    # the alpha / beta entries are present and large: the branch is exercised
    assert np.abs(ref[:2 * c.N]).max() > 0.1
    # a copy keeps the flag and gives the same distance
    assert hsd(psi.copy(), pp, hop, unitary, es) == d


@pytest.mark.parametrize("name", ["rbm6_hsd_fqa", "deep6_hsd_fqa"])
def test_free_quantum_axis_on_monte_carlo_samples_vs_restatement(name):
    import rbmongpu_gb300 as rg
    c = Case(name)
    psi, pp = gpu_psi(c), gpu_psi(c, "pp_")
    hop_t = c.op("hop_")
    chains, samples, seed = 128, 4, 3
    mc = lambda: rg.MonteCarloLoop(chains * samples, 1, 4, chains, seed=seed)   # noqa: E731
    sp, _, _ = mc().samples(psi)
    hsd = rg.HilbertSpaceDistance(c.N, psi.num_params)
    unitary = bool(c.meta("hsd_unitary"))
    g, d = hsd.gradient(psi, pp, rg.Operator(*hop_t), unitary, mc(), 1.0)
    og, od = po.samples_hsd(oracle_psi(c), oracle_psi(c, "pp_"), po.Op(*hop_t), unitary, sp, 1.0)
    assert d == pytest.approx(od, rel=1e-6)
    assert np.abs(g - og).max() <= RTOL * np.abs(og).max()
