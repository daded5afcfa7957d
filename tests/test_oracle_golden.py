"""Pins the CPU restatement (oracle/) to outputs of the reference's own host path
(tests/golden/*.npz, generated by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po


def close(a, b, rtol, atol):
    np.testing.assert_allclose(np.asarray(a), np.asarray(b), rtol=rtol, atol=atol)


def rbm_of(case, prefix=""):
    b, W = case.rbm(prefix)
    alpha, fqa = case.quaxis(prefix)
    return po.RBM(b, W, case.prefactor if prefix == "" else 1.0, alpha=alpha, beta=alpha, free_quantum_axis=fqa)


def deep_of(case, prefix=""):
    b, c, w, fw = case.deep(prefix)
    alpha, fqa = case.quaxis(prefix)
    return po.Deep(case.N, b, c, w, fw, case.prefactor if prefix == "" else 1.0, pair=case.kind == "pair",
                   alpha=alpha, beta=alpha, free_quantum_axis=fqa)


def psi_of(case, prefix=""):
    return rbm_of(case, prefix) if case.kind == "rbm" else deep_of(case, prefix)


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm6_hsd_nonunitary"])
def test_activation_matches_reference(name):
    c = Case(name)
    z = c.i("act_in")
    lc = np.array([po.logcosh(x) for x in z])
    th = np.array([po.tanh(x) for x in z])
    close(lc, c.o("logcosh"), 1e-13, 1e-14)
    close(th, c.o("tanh"), 1e-12, 1e-14)


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm6_hsd_nonunitary", "rbm8_mixed_operator",
                                  "deep8_sparse", "deep10_dense", "pair3"])
def test_exact_summation_matches_reference(name):
    c = Case(name)
    psi = psi_of(c)
    op = po.Op(*c.op())
    # prefactor was normalised by the reference: the norm is then 1
    assert po.exact_norm(psi) == pytest.approx(c.s("norm"), rel=1e-12)
    close(po.psi_vector(psi), c.o("vector"), 1e-11, 1e-15)
    if c.kind == "pair":
        sig, E = po.exact_fluctuation(psi, op)
        assert E == pytest.approx(complex(c.s("E_re"), c.s("E_im")), rel=1e-11, abs=1e-13)
        return
    sig, E = po.exact_fluctuation(psi, op)
    assert E == pytest.approx(complex(c.s("E_re"), c.s("E_im")), rel=1e-11, abs=1e-13)
    assert sig == pytest.approx(c.s("sigma"), rel=1e-8, abs=1e-10)
    g, E2 = po.exact_gradient(psi, op)
    assert E2 == pytest.approx(complex(c.s("gradE_re"), c.s("gradE_im")), rel=1e-11, abs=1e-13)
    close(g, c.o("gradient"), 1e-9, 1e-12 * np.abs(c.o("gradient")).max())


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm6_hsd_nonunitary", "rbm8_mixed_operator",
                                  "deep8_sparse", "deep10_dense", "pair3", "rbm6_hsd_fqa", "deep6_hsd_fqa"])
def test_hilbert_space_distance_matches_reference(name):
    c = Case(name)
    psi, pp = psi_of(c), psi_of(c, "pp_")
    hop = po.Op(*c.op("hop_"))
    unitary = bool(c.meta("hsd_unitary"))
    nu = float(c.meta("hsd_nu"))
    g, d = po.exact_hsd(psi, pp, hop, unitary, nu)
    assert d == pytest.approx(c.s("hsd_distance"), rel=1e-8)
    assert d == pytest.approx(c.s("hsd_grad_distance"), rel=1e-8)
    ref = c.o("hsd_gradient")
    close(g, ref, 1e-6, 1e-9 * np.abs(ref).max())


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm6_hsd_nonunitary", "c2_rbm_mc", "deep8_sparse", "deep10_dense"])
def test_O_k_vector_matches_reference(name):
    c = Case(name)
    psi = psi_of(c)
    ref = c.o("ok_vectors").reshape(-1, psi.num_params)
    for t, conf in enumerate(c.i("ok_spins")):
        ok = po.O_k(psi, po.spins_array([conf], c.N)[0])
        close(ok, ref[t], 1e-12, 1e-14)


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm8_mixed_operator", "c2_rbm_mc", "deep8_sparse"])
def test_metropolis_chain_matches_reference_bit_exact(name):
    """mt19937(0) stream, FP64 reference arithmetic: identical spins and accept counts."""
    c = Case(name)
    psi = psi_of(c)
    op = po.Op(*c.op())
    samples = int(c.meta("mc_samples"))
    spins, lp, el, acc, rej = po.mc_run(psi, op, 1, samples, int(c.meta("mc_sweeps")), int(c.meta("mc_therm")),
                                        rng=po.OR_RNG_MT19937, prec=po.OR_PREC_REF64)
    ref_spins = c.o("mc_spins")
    assert np.array_equal(spins[:, 0, 0], ref_spins)
    assert int(acc[0]) == int(c.s("mc_accept"))
    assert int(rej[0]) == int(c.s("mc_reject"))
    close(lp[:, 0], c.o("mc_logpsi"), 1e-12, 1e-12)
    E = el[:, 0].mean()
    assert E == pytest.approx(complex(c.s("mc_E_re"), c.s("mc_E_im")), rel=1e-10, abs=1e-12)


@pytest.mark.parametrize("name", ["c1_rbm_exact", "rbm8_mixed_operator", "c2_rbm_mc", "deep8_sparse"])
def test_mc_gradient_estimator_matches_reference(name):
    """The E_k-term gradient estimator over the reference's own samples."""
    c = Case(name)
    psi = psi_of(c)
    op = po.Op(*c.op())
    spins = po.spins_array(c.o("mc_spins"), c.N)
    g, E = po.samples_gradient(psi, op, spins)
    assert E == pytest.approx(complex(c.s("mc_gradE_re"), c.s("mc_gradE_im")), rel=1e-10, abs=1e-12)
    ref = c.o("mc_gradient")
    close(g, ref, 1e-8, 1e-11 * np.abs(ref).max())


def test_mt19937_known_answer():
    # 10000th output of mt19937 seeded with 5489 (C++ standard [rand.predef])
    assert int(po.mt_words(5489, 10000)[-1]) == 4123659995


def test_philox_known_answer():
    # Philox4x32-10 known-answer vectors of the Random123 distribution (kat_vectors)
    import ctypes as C
    L = po.lib()
    out = (C.c_uint32 * 4)()
    L.or_philox4x32_10((C.c_uint32 * 4)(0, 0, 0, 0), (C.c_uint32 * 2)(0, 0), out)
    assert list(out) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    L.or_philox4x32_10((C.c_uint32 * 4)(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF),
                       (C.c_uint32 * 2)(0xFFFFFFFF, 0xFFFFFFFF), out)
    assert list(out) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    L.or_philox4x32_10((C.c_uint32 * 4)(0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344),
                       (C.c_uint32 * 2)(0xA4093822, 0x299F31D0), out)
    assert list(out) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_expf_det_error_bound():
    xs = np.linspace(-87.0, 0.0, 20001, dtype=np.float32)
    got = np.array([po.expf_det(float(x)) for x in xs], np.float64)
    ref = np.exp(xs.astype(np.float64))
    assert np.max(np.abs(got - ref) / ref) < 4e-7


def test_deterministic_log_of_the_restatement():
    """or_logf_det (the learned proposal's softmax log, replayed bit for bit on the device)
    is within 2e-7 relative of log over the range the softmax normalisers take."""
    xs = np.concatenate([np.linspace(1.0, 300.0, 5000), np.exp(np.linspace(-30, 30, 500))]).astype(np.float32)
    got = np.array([po.logf_det(float(x)) for x in xs], np.float64)
    ref = np.log(xs.astype(np.float64))
    assert np.all(np.abs(got - ref) <= 2e-7 * np.maximum(np.abs(ref), 1.0))


def test_div_pos_is_within_an_ulp_of_the_ieee_quotient():
    """div_pos (device_math.cuh; the Metropolis test's quotient, replayed here by the
    oracle bit for bit): within one ulp of the correctly rounded quotient for every
    denominator the activation produces (|D(u)|^2 >= 84) and numerators of any sign, and
    equal to it for all but a small fraction of inputs."""
    rng = np.random.default_rng(21)
    n = 1_000_000
    den = np.float32(84.0) * np.exp2(rng.uniform(0.0, 40.0, n)).astype(np.float32)
    num = (rng.normal(size=n) * np.exp2(rng.uniform(-20.0, 60.0, n))).astype(np.float32)
    got = po.div_pos_f32(num, den)
    ref = (num / den).astype(np.float32)       # IEEE division, correctly rounded
    ulp = np.spacing(np.abs(ref)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert np.all(err <= ulp), float((err / ulp).max())
    assert np.mean(got != ref) < 1e-3, float(np.mean(got != ref))


def test_reciprocal_seed_constant():
    """The integer seed 0x7EF311C2 - bits(den) of div_pos: its largest relative error over
    every mantissa is 5.05 %, the same in every binade, and no neighbouring constant does
    better; two Newton steps square it twice (to 6.5e-6)."""
    m = np.arange(0, 1 << 23, dtype=np.uint32)

    def worst(c, exponent=127):
        bits = (np.uint32(exponent) << 23) | m
        den = bits.view(np.float32).astype(np.float64)
        est = (np.uint32(c) - bits).view(np.float32).astype(np.float64)
        return float(np.abs(est * den - 1.0).max())

    e0 = worst(0x7EF311C2)
    assert 0.0505 < e0 < 0.0506
    assert worst(0x7EF311C2, 133) == pytest.approx(e0, abs=1e-9)
    for c in (0x7EF311C1, 0x7EF311C3, 0x7EF31000, 0x7EF31400):
        assert worst(c) > e0
    assert (e0 ** 2) ** 2 < 7e-6
