"""Parity of the PsiDeep / PsiPair CUDA path (through the C ABI) with the reference's
own outputs (tests/golden) and with the CPU restatement.

Tolerance: 1e-5 relative (complex64 compute; vectors relative to their largest entry).
"""
import numpy as np
import pytest

import rbmongpu_gb300 as rg
from golden_cases import Case
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def dist_close(d, ref):
    """d^2 = 1 - u/v within 1e-5 relative, floored at 1e-15 absolute: FP64 itself cannot
    resolve 1 - u/v below ~1e-16, so distances under ~1e-5 carry that floor."""
    assert abs(d * d - ref * ref) <= RTOL * ref * ref + 1e-15, (d, ref)


def vec_close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max() / scale
    assert err < rtol, f"max deviation {err:.3e} of scale {scale:.3e}"


def deep_gpu(case, prefix=""):
    b, c, w, fw = case.deep(prefix)
    cls = rg.PsiPair if case.kind == "pair" else rg.PsiDeep
    return cls(np.zeros(case.N), np.zeros(case.N), b, c, w, fw, case.prefactor if prefix == "" else 1.0, False, True)


def deep_oracle(case, prefix=""):
    b, c, w, fw = case.deep(prefix)
    return po.Deep(case.N, b, c, w, fw, case.prefactor if prefix == "" else 1.0, pair=case.kind == "pair")


@pytest.mark.parametrize("name", ["deep8_sparse", "deep10_dense", "pair3"])
def test_vector_norm_energy_vs_reference(name):
    c = Case(name)
    psi = deep_gpu(c)
    es = rg.ExactSummation(c.N)
    assert psi.norm(es) == pytest.approx(c.s("norm"), rel=RTOL)
    vec_close(psi.vector, c.o("vector"))
    E = rg.ExpectationValue()(psi, rg.Operator(*c.op()), es)
    E_ref = complex(c.s("E_re"), c.s("E_im"))
    assert abs(E - E_ref) <= RTOL * abs(E_ref)


@pytest.mark.parametrize("name", ["deep8_sparse", "deep10_dense"])
def test_gradient_vs_reference(name):
    c = Case(name)
    psi = deep_gpu(c)
    es = rg.ExactSummation(c.N)
    ev = rg.ExpectationValue()
    sig, E = ev.fluctuation(psi, rg.Operator(*c.op()), es)
    assert sig == pytest.approx(c.s("sigma"), rel=RTOL)
    g, E2 = ev.gradient(psi, rg.Operator(*c.op()), es)
    E_ref = complex(c.s("gradE_re"), c.s("gradE_im"))
    assert abs(E2 - E_ref) <= RTOL * abs(E_ref)
    vec_close(g, c.o("gradient"))


@pytest.mark.parametrize("name", ["deep8_sparse", "deep10_dense", "pair3"])
def test_hilbert_space_distance_vs_reference(name):
    c = Case(name)
    psi, pp = deep_gpu(c), deep_gpu(c, "pp_")
    hop = rg.Operator(*c.op("hop_"))
    es = rg.ExactSummation(c.N)
    hsd = rg.HilbertSpaceDistance(c.N, psi.num_params)
    unitary = bool(c.meta("hsd_unitary"))
    d = hsd(psi, pp, hop, unitary, es)
    dist_close(d, c.s("hsd_distance"))
    g, d2 = hsd.gradient(psi, pp, hop, unitary, es, float(c.meta("hsd_nu")))
    dist_close(d2, c.s("hsd_grad_distance"))
    # the gradient's numerator is the same FP64 difference as d^2: its relative error
    # floor is ~1e-16 / d^2 (2e-5 at the 8-spin PsiDeep's d = 3.3e-6)
    ref_d = c.s("hsd_distance")
    vec_close(g, c.o("hsd_gradient"), RTOL + 1e-16 / (ref_d * ref_d))


@pytest.mark.parametrize("name", ["deep8_sparse", "deep10_dense"])
def test_O_k_vector_vs_reference(name):
    c = Case(name)
    psi = deep_gpu(c)
    ref = c.o("ok_vectors").reshape(-1, psi.num_params)
    for t, conf in enumerate(c.i("ok_spins")):
        vec_close(rg.psi_O_k_vector(psi, int(conf)), ref[t])


def test_deep_mc_energy_and_gradient_vs_restatement_on_same_samples():
    c = Case("deep8_sparse")
    psi, opsi = deep_gpu(c), deep_oracle(c)
    op_t = c.op()
    chains, samples, seed = 64, 4, 17
    sp, lp, el = rg.MonteCarloLoop(chains * samples, 1, 3, chains, seed=seed).samples(psi, rg.Operator(*op_t))
    oel = np.array([po.local_energy(opsi, po.Op(*op_t), s) for s in sp])
    vec_close(el, oel)
    vec_close(lp, np.array([po.log_psi(opsi, s) for s in sp]))
    g, E = rg.ExpectationValue().gradient(psi, rg.Operator(*op_t),
                                          rg.MonteCarloLoop(chains * samples, 1, 3, chains, seed=seed))
    og, oE = po.samples_gradient(opsi, po.Op(*op_t), sp)
    assert abs(E - oE) <= RTOL * abs(oE)
    vec_close(g, og)


def test_deep_mc_converges_to_exact_energy():
    """Statistical check of the PsiDeep Metropolis chain against exact summation."""
    c = Case("deep8_sparse")
    psi = deep_gpu(c)
    op = rg.Operator(*c.op())
    mc = rg.MonteCarloLoop(512 * 40, 2, 20, 512, seed=4)
    _, _, el = mc.samples(psi, op)
    E_exact = complex(c.s("E_re"), c.s("E_im"))
    se = el.real.reshape(40, 512).mean(axis=1).std() / np.sqrt(40)
    assert abs(el.real.mean() - E_exact.real) < 5 * se + 1e-3
    assert 0.0 < mc.acceptance_rate < 1.0
