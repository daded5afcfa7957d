"""ExpectationValue's further methods: fluctuation_gradient, the operator-list call (one
pass), difference and corrected (source/network_functions/ExpectationValue.cu:76-127,
258-348, 350-446, 448-518; bound in pyRBMonGPU/main.cpp:295-339).

The CPU restatements (oracle/pyoracle.py) are pinned to the reference's own outputs from
its host build (tests/golden: o_fluct_gradient, o_ev_list, o_ev_difference,
s_corrected_*); the CUDA path is checked against those fixtures over ExactSummation and
against the restatement on the same Monte Carlo samples.

Tolerance: 1e-5 of the largest entry (complex64 compute), as for the gradient; difference,
a difference of two energies, 1e-5 of <E>; corrected's
weight exp(2 Im E + Re(E E - E)) turns a relative error dE of the FP32 local energy into
2 |E| dE, so it is held to 1e-4.
"""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po

RTOL = 1e-5
EXACT_CASES = ["c1_rbm_exact", "rbm8_mixed_operator", "deep8_sparse", "deep10_dense"]


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def oracle_of(c, prefix=""):
    if c.kind == "rbm":
        b, W = c.rbm(prefix)
        return po.RBM(b, W, c.prefactor if prefix == "" else 1.0)
    b, cn, w, fw = c.deep(prefix)
    return po.Deep(c.N, b, cn, w, fw, c.prefactor if prefix == "" else 1.0)


def gpu_of(rg, c, prefix=""):
    if c.kind == "rbm":
        b, W = c.rbm(prefix)
        return rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor if prefix == "" else 1.0, False, True)
    b, cn, w, fw = c.deep(prefix)
    return rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor if prefix == "" else 1.0, False, True)


# ----------------------------------------------------------------------------- CPU
@pytest.mark.parametrize("name", EXACT_CASES)
def test_restatements_match_reference(name):
    c = Case(name)
    psi = oracle_of(c)
    op, hop = po.Op(*c.op()), po.Op(*c.op("hop_"))
    s, w = po.exact_configs(psi)
    assert rel(po.fluctuation_gradient(psi, op, s, w), c.o("fluct_gradient")) < 1e-9
    assert np.abs(po.ev_list(psi, [op, hop], s, w) - c.o("ev_list")).max() < 1e-12
    if c.kind == "rbm":
        d = po.ev_difference(psi, oracle_of(c, "pp_"), [op, hop], s, w)
        assert np.abs(d - c.o("ev_difference")).max() < 1e-12
    else:
        v, a = po.ev_corrected(psi, op, s, w)
        assert v.real == pytest.approx(c.s("corrected_re"), rel=1e-10)
        assert a == pytest.approx(c.s("corrected_abs2"), rel=1e-10)


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


@gpu
@pytest.mark.parametrize("name", EXACT_CASES)
def test_exact_summation_vs_reference(name):
    import rbmongpu_gb300 as rg
    c = Case(name)
    psi = gpu_of(rg, c)
    op, hop = rg.Operator(*c.op()), rg.Operator(*c.op("hop_"))
    es = rg.ExactSummation(c.N)
    ev = rg.ExpectationValue()
    assert rel(ev.fluctuation_gradient(psi, op, es), c.o("fluct_gradient")) < RTOL
    vals = ev(psi, [op, hop], es)
    assert rel(vals, c.o("ev_list")) < RTOL
    if c.kind == "rbm":
        d = ev.difference(psi, gpu_of(rg, c, "pp_"), [op, hop], es)
        ref = c.o("ev_difference")
        # a difference of two energies of the size of <E>: held to the tolerance at that scale
        assert np.abs(np.asarray(d) - ref).max() < RTOL * np.abs(c.o("ev_list")).max()
    else:
        v, a = ev.corrected(psi, op, hop, es)
        assert v == pytest.approx(complex(c.s("corrected_re"), c.s("corrected_im")), rel=1e-4)
        assert a == pytest.approx(c.s("corrected_abs2"), rel=1e-4)


def mc_setup(rg, seed):
    c = Case("c2_rbm_mc")
    psi = gpu_of(rg, c)
    opsi = oracle_of(c)
    mk = lambda: rg.MonteCarloLoop(256 * 2, 1, 3, 256, seed=seed)   # noqa: E731
    sp, _, _ = mk().samples(psi)
    return c, psi, opsi, mk, sp


@gpu
def test_mc_fluctuation_gradient_vs_restatement_on_same_samples():
    import rbmongpu_gb300 as rg
    c, psi, opsi, mk, sp = mc_setup(rg, 21)
    g = rg.ExpectationValue().fluctuation_gradient(psi, rg.Operator(*c.op()), mk())
    og = po.fluctuation_gradient(opsi, po.Op(*c.op()), sp)
    assert rel(g, og) < RTOL


@gpu
def test_mc_operator_list_is_one_pass():
    """Both operators on the same samples: the list values equal the restatement's
    energies over the configurations one sampling call returns."""
    import rbmongpu_gb300 as rg
    c, psi, opsi, mk, sp = mc_setup(rg, 22)
    ops_t = [c.op(), c.op("hop_")]
    vals = rg.ExpectationValue()(psi, [rg.Operator(*o) for o in ops_t], mk())
    ref = po.ev_list(opsi, [po.Op(*o) for o in ops_t], sp)
    assert rel(vals, ref) < RTOL


@gpu
def test_mc_difference_vs_restatement_on_same_samples():
    import rbmongpu_gb300 as rg
    c, psi, opsi, mk, sp = mc_setup(rg, 23)
    b, W = c.rbm()
    rng = np.random.default_rng(3)
    Wp = W + 1e-2 * (rng.normal(size=W.shape) + 1j * rng.normal(size=W.shape))
    pp = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, Wp, 1.0, False, True)
    d = rg.ExpectationValue().difference(psi, pp, [rg.Operator(*c.op())], mk())
    ref = po.ev_difference(opsi, po.RBM(b, Wp, 1.0), [po.Op(*c.op())], sp)
    scale = abs(po.ev_list(opsi, [po.Op(*c.op())], sp)[0])
    assert abs(d[0] - ref[0]) < RTOL * scale


@gpu
def test_corrected_and_difference_argument_checks():
    import rbmongpu_gb300 as rg
    c = Case("deep8_sparse")
    psi = gpu_of(rg, c)
    op = rg.Operator(*c.op())
    with pytest.raises(rg.RbmgError):   # difference is instantiated for Psi only
        rg.ExpectationValue().difference(psi, psi, [op], rg.ExactSummation(c.N))
