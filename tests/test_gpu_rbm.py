"""Parity of the CUDA path (through the C ABI) with the reference's own outputs and
with the CPU restatement, for the complex RBM.

Tolerances: energies, gradients and distances within 1e-5 relative (complex64
compute; relative to the largest entry for vectors); spins, flip sites and accept
counts bit-exact against the restatement's FP32 replay with the same Philox streams.
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


def rbm_gpu(case, prefix=""):
    b, W = case.rbm(prefix)
    return rg.Psi(np.zeros(case.N), np.zeros(case.N), b, W, case.prefactor if prefix == "" else 1.0, False, True)


def rbm_oracle(case, prefix=""):
    b, W = case.rbm(prefix)
    return po.RBM(b, W, case.prefactor if prefix == "" else 1.0)


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm6_hsd_nonunitary", "rbm8_mixed_operator"])
def test_exact_summation_vs_reference(name):
    c = Case(name)
    psi = rbm_gpu(c)
    op = rg.Operator(*c.op())
    es = rg.ExactSummation(c.N)
    assert psi.norm(es) == pytest.approx(c.s("norm"), rel=RTOL)
    vec_close(psi.vector, c.o("vector"))
    ev = rg.ExpectationValue()
    E = ev(psi, op, es)
    E_ref = complex(c.s("E_re"), c.s("E_im"))
    assert abs(E - E_ref) <= RTOL * abs(E_ref)
    sigma, E2 = ev.fluctuation(psi, op, es)
    assert sigma == pytest.approx(c.s("sigma"), rel=RTOL)
    g, E3 = ev.gradient(psi, op, es)
    assert abs(E3 - E_ref) <= RTOL * abs(E_ref)
    vec_close(g, c.o("gradient"))


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm6_hsd_nonunitary", "rbm8_mixed_operator"])
def test_hilbert_space_distance_vs_reference(name):
    c = Case(name)
    psi, pp = rbm_gpu(c), rbm_gpu(c, "pp_")
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


@pytest.mark.parametrize("name", ["c1_rbm_exact", "c2_rbm_mc"])
def test_O_k_vector_vs_reference(name):
    c = Case(name)
    psi = rbm_gpu(c)
    ref = c.o("ok_vectors").reshape(-1, psi.num_params)
    for t, conf in enumerate(c.i("ok_spins")):
        vec_close(rg.psi_O_k_vector(psi, int(conf)), ref[t])


def test_activation_function_matches_reference():
    c = Case("c1_rbm_exact")
    got = np.array([rg.activation_function(z) for z in c.i("act_in")])
    np.testing.assert_allclose(got, c.o("logcosh"), rtol=1e-13, atol=1e-14)


def c2_setup():
    c = Case("c2_rbm_mc")
    return c, rbm_gpu(c), rbm_oracle(c), c.op()


def test_mc_chains_bit_exact_vs_restatement():
    """c2 shapes (N=64, M=128, 8x8 TFIM h=3): spins and accept counts of 64 chains."""
    c, psi, opsi, op_t = c2_setup()
    chains, samples, therm, seed = 64, 3, 2, 0xC0FFEE
    mc = rg.MonteCarloLoop(chains * samples, 1, therm, chains, seed=seed)
    op = rg.Operator(*op_t)
    sp, lp, el = mc.samples(psi, op)
    acc_gpu, props = mc.acceptance()
    ospins, olp, oel, oacc, orej = po.mc_run(opsi, po.Op(*op_t), chains, samples, 1, therm, seed=seed)
    assert np.array_equal(sp.reshape(samples, chains, -1), ospins)
    assert int(acc_gpu) == int(oacc.sum())
    assert int(props) == int((oacc + orej).sum())
    vec_close(el, oel.reshape(-1))
    vec_close(lp, olp.reshape(-1))


def test_mc_total_z_chains_bit_exact_vs_restatement():
    c = Case("c1_rbm_exact")
    psi, opsi = rbm_gpu(c), rbm_oracle(c)
    chains, samples, seed = 32, 4, 7
    mc = rg.MonteCarloLoop(chains * samples, 2, 3, chains, seed=seed)
    mc.set_total_z_symmetry(2)
    sp, _, _ = mc.samples(psi)
    ospins, _, _, oacc, _ = po.mc_run(opsi, None, chains, samples, 2, 3, seed=seed, total_z=True, sector=2,
                                     want_eloc=False)
    assert np.array_equal(sp.reshape(samples, chains, -1), ospins)
    assert all(2 * bin(int(x)).count("1") - c.N == 2 for x in sp[:, 0])
    assert int(mc.acceptance()[0]) == int(oacc.sum())


def test_mc_gradient_vs_restatement_on_same_samples():
    c, psi, opsi, op_t = c2_setup()
    chains, samples, seed = 256, 2, 99
    op = rg.Operator(*op_t)
    mc_a = rg.MonteCarloLoop(chains * samples, 1, 2, chains, seed=seed)
    sp, _, _ = mc_a.samples(psi)
    mc_b = rg.MonteCarloLoop(chains * samples, 1, 2, chains, seed=seed)
    g, E = rg.ExpectationValue().gradient(psi, op, mc_b)
    og, oE = po.samples_gradient(opsi, po.Op(*op_t), sp)
    assert abs(E - oE) <= RTOL * abs(oE)
    vec_close(g, og)


def test_mc_energy_and_fluctuation_vs_restatement():
    c, psi, opsi, op_t = c2_setup()
    chains, samples, seed = 512, 2, 5
    op = rg.Operator(*op_t)
    sp, _, _ = rg.MonteCarloLoop(chains * samples, 1, 3, chains, seed=seed).samples(psi)
    el = np.array([po.local_energy(opsi, po.Op(*op_t), s) for s in sp])
    ev = rg.ExpectationValue()
    E = ev(psi, op, rg.MonteCarloLoop(chains * samples, 1, 3, chains, seed=seed))
    assert abs(E - el.mean()) <= RTOL * abs(el.mean())
    sig, E2 = ev.fluctuation(psi, op, rg.MonteCarloLoop(chains * samples, 1, 3, chains, seed=seed))
    assert sig == pytest.approx(np.sqrt(np.mean(np.abs(el) ** 2) - abs(el.mean()) ** 2), rel=1e-4)


def test_mc_hsd_vs_restatement_on_same_samples():
    c = Case("c1_rbm_exact")
    psi, pp = rbm_gpu(c), rbm_gpu(c, "pp_")
    opsi, opp = rbm_oracle(c), rbm_oracle(c, "pp_")
    hop_t = c.op("hop_")
    chains, samples, seed = 128, 4, 3
    sp, _, _ = rg.MonteCarloLoop(chains * samples, 1, 4, chains, seed=seed).samples(psi)
    hsd = rg.HilbertSpaceDistance(c.N, psi.num_params)
    g, d = hsd.gradient(psi, pp, rg.Operator(*hop_t), True,
                        rg.MonteCarloLoop(chains * samples, 1, 4, chains, seed=seed), 1.0)
    og, od = po.samples_hsd(opsi, opp, po.Op(*hop_t), True, sp, 1.0)
    assert d == pytest.approx(od, rel=RTOL)
    vec_close(g, og)


def test_c2_full_size_walkers():
    """4096 walkers of the N=64 / M=128 chain: size-independent properties."""
    c, psi, opsi, op_t = c2_setup()
    mc = rg.MonteCarloLoop(4096 * 2, 1, 5, 4096, seed=2024)
    sp, lp, el = mc.samples(psi, rg.Operator(*op_t))
    rate = mc.acceptance_rate
    assert 0.0 < rate < 1.0
    assert sp.shape == (8192, 1)
    assert np.isfinite(el).all() and np.isfinite(lp).all()
    # spot-check walkers bit-exactly against the restatement (walkers are independent streams)
    for w in (0, 1777, 4095):
        ospins, _, _, _, _ = po.mc_run(opsi, None, 1, 2, 1, 5, seed=2024, chain_begin=w, total_chains=4096,
                                       want_eloc=False)
        assert np.array_equal(sp.reshape(2, 4096, 1)[:, w], ospins[:, 0])


def test_params_roundtrip_and_errors():
    c = Case("c1_rbm_exact")
    psi = rbm_gpu(c)
    p = psi.params
    assert p.shape == (2 * 12 + 24 + 12 * 24,)
    psi.params = p * 1.5
    np.testing.assert_array_equal(psi.params, p * 1.5)
    bad = p.copy()
    bad[30] = np.nan
    with pytest.raises(rg.RbmgError):
        psi.params = bad
    cp = psi.copy()
    np.testing.assert_array_equal(cp.params, psi.params)
    with pytest.raises(rg.RbmgError):
        rg.MonteCarloLoop(10, 1, 0, 3)   # samples not a multiple of chains
    with pytest.raises(rg.RbmgError):
        rg.ExpectationValue()(psi, rg.Operator(*rg.operators.tfim_chain(20)), rg.ExactSummation(12))


@pytest.mark.parametrize("N,M,chains", [(10, 20, 7), (40, 60, 16), (150, 100, 5), (70, 250, 16), (100, 400, 9),
                                        (200, 576, 6)])
def test_mc_chains_bit_exact_every_instantiation(N, M, chains):
    """Every hidden-units-per-lane count (K = 1, 2, 4, 8, 13, 18: odd ones with the paired
    form's zero unit), one to four spin words (N up to 200), walker counts that do not fill
    a block: spins and accept counts equal the restatement's bit for bit."""
    rng = np.random.default_rng(N * 1000 + M)
    b = 0.1 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = 0.1 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    samples, therm, seed = 2, 1, 31
    mc = rg.MonteCarloLoop(chains * samples, 1, therm, chains, seed=seed)
    sp, _, _ = mc.samples(psi)
    acc_gpu, props = mc.acceptance()
    ospins, _, _, oacc, orej = po.mc_run(po.RBM(b, W, 1.0), None, chains, samples, 1, therm, seed=seed,
                                         want_eloc=False)
    assert np.array_equal(sp.reshape(samples, chains, -1), ospins)
    assert int(acc_gpu) == int(oacc.sum()) > 0
    assert int(props) == int((oacc + orej).sum())


def test_local_energies_of_no_configurations():
    c = Case("c1_rbm_exact")
    psi = rbm_gpu(c)
    out = rg.local_energies(psi, rg.Operator(*c.op()), np.zeros((0, 1), np.uint64))
    assert out.shape == (0,)
