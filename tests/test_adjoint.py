"""Adjoint (reverse-mode) gradient of the local energy for PsiDeep, and the complex RBM's
derivative of <E_loc> from its estimator sums, behind a torch.autograd.Function: against
FP64 central finite differences on 32 seeded parameters, against the reference's O_k
estimator (rbmg_ev_gradient), and through torch's backward.

Tolerances: the adjoint runs its forward and reverse passes in FP32 (complex64) with FP64
sums; gradients agree with the FP64 references within 1e-4 of the gradient's largest
entry (FP32 round-off of log psi(s') - log psi(s) is ~1e-6 of |log psi|).

Finite differences: the reference's activation f(z) = g(sign(Re z) z) (a rational g,
include/quantum_state/psi_functions.hpp:49-57) is discontinuous across Re z = 0, and with
thousands of pre-activations per sample set a step of 1e-3 crosses that line for almost
every parameter (the central difference then measures the jump, not the derivative).
The checks therefore take FP64 central differences with steps 1e-5 and 2e-5 and use a
parameter only where the two agree (no pre-activation crossed the line); at least 24 of
the 32 seeded parameters must qualify.
"""
import numpy as np
import pytest

RTOL = 1e-4


def deep_net(N, sizes, seed, scale=0.1):
    """Dense complex PsiDeep N -> sizes[0] -> ..., weights complex Normal(0, scale / fan_in)
    (variance), biases likewise, final weights 1: the deep-net benchmark configuration
    at N=100, sizes (200, 100, 50)."""
    import rbmongpu_gb300 as rg
    rng = np.random.Generator(np.random.PCG64(seed))
    b, conn, W = [], [], []
    fan = N
    for m in sizes:
        sd = np.sqrt(scale / fan / 2)
        b.append(rng.normal(0, sd, m) + 1j * rng.normal(0, sd, m))
        conn.append(np.array([[c] * m for c in range(fan)]))
        W.append(rng.normal(0, sd, (fan, m)) + 1j * rng.normal(0, sd, (fan, m)))
        fan = m
    return rg.PsiDeep(np.zeros(N), np.zeros(N), b, conn, W, np.ones(sizes[-1]), 1.0, False, True)


def param_indices(psi, count, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(np.arange(2 * psi.N, psi.num_params), count, replace=False))


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def fd_check(psi, loss, grad, idx, h=1e-5, rtol=RTOL):
    """FP64 central differences of loss(params) in the real and imaginary direction of
    each parameter in idx at steps h and 2h; returns (usable indices, fd values)."""
    p0 = psi.params
    vals = {}
    for k in idx:
        d = []
        for hh in (h, 2 * h):
            v = []
            for step in (hh, 1j * hh):
                p = p0.copy()
                p[k] += step
                lp = loss(p)
                p[k] -= 2 * step
                v.append((lp - loss(p)) / (2 * hh))
            d.append(v[0] + 1j * v[1])
        vals[k] = d
    psi.params = p0
    scale = np.abs(grad).max()
    good = [k for k in idx if abs(vals[k][0] - vals[k][1]) <= 0.5 * rtol * scale]
    return np.array(good), np.array([vals[k][0] for k in good])


@pytest.mark.gpu
@pytest.mark.parametrize("N,sizes,walkers,rtol", [(12, (24, 12, 6), 128, RTOL), (100, (200, 100, 50), 8, 2e-3)])
def test_fixed_sample_adjoint_matches_fp64_finite_differences(N, sizes, walkers, rtol):
    """rtol 2e-3 for the N=100 net: its central differences carry FP64 round-off of an
    energy of ~1e2 over a step of 1e-5, ~1e-8 against gradient entries of ~1e-5, so their
    own noise is ~1e-3 of the largest entry (measured deviations 0.5e-3 to 1.1e-3 over the
    sample sets the sampler has drawn)."""
    import rbmongpu_gb300 as rg
    psi = deep_net(N, sizes, 103)
    H = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    mc = rg.MonteCarloLoop(walkers * 2, 1, 5, walkers, seed=31)
    sp, _, _ = mc.samples(psi)
    g, E = rg.ExpectationValue().eloc_gradient(psi, H, rg.MonteCarloLoop(walkers * 2, 1, 5, walkers, seed=31),
                                               score=False)
    el = rg.local_energies(psi, H, sp)
    assert abs(E - el.mean()) <= 1e-5 * np.abs(el).mean()
    def loss(p):
        psi.params = p
        return rg.local_energies(psi, H, sp).real.mean()

    good, fd = fd_check(psi, loss, g, param_indices(psi, 32, 7), rtol=rtol)
    assert len(good) >= 24, len(good)
    assert rel_err(g[good], fd) < rtol, (g[good][:4], fd[:4])


@pytest.mark.gpu
def test_adjoint_with_sampling_term_matches_reference_estimator():
    """score=True reproduces ExpectationValue.gradient (the reference's O_k estimator,
    ExpectationValue.cu:243-253) over ExactSummation of a normalised psi, except the
    final weights, whose O_k the reference scales by log psi.  (The two expressions differ
    by 2i Im<E> <O*>, which vanishes for a hermitian operator under exact summation.)"""
    import rbmongpu_gb300 as rg
    N, sizes = 10, (20, 10, 5)
    psi = deep_net(N, sizes, 5, scale=0.5)
    H = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    es = rg.ExactSummation(N)
    psi.prefactor = 1.0 / psi.norm(es)
    g, E = rg.ExpectationValue().eloc_gradient(psi, H, es, score=True)
    gr, Er = rg.ExpectationValue().gradient(psi, H, es)
    assert abs(E - Er) <= 1e-5 * abs(Er)
    last = sizes[-1]
    body = slice(2 * N, psi.num_params - last)
    assert rel_err(g[body], gr[body]) < RTOL
    assert np.all(g[:2 * N] == 0)


@pytest.mark.gpu
def test_exact_summation_gradient_matches_finite_differences_of_the_energy():
    """Normalised psi, ExactSummation: score=True is the gradient of <H>."""
    import rbmongpu_gb300 as rg
    N, sizes = 8, (16, 8, 4)
    psi = deep_net(N, sizes, 11, scale=0.5)
    H = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    es = rg.ExactSummation(N)

    def energy(p):
        psi.params = p
        return (rg.ExpectationValue()(psi, H, es) / psi.norm(es) ** 2).real

    p0 = psi.params
    psi.params = p0
    psi.prefactor = 1.0 / psi.norm(es)
    g, E = rg.ExpectationValue().eloc_gradient(psi, H, es, score=True)
    assert abs(E.real - energy(p0)) <= 1e-5 * abs(E)
    good, fd = fd_check(psi, energy, g, param_indices(psi, 32, 9))
    assert len(good) >= 24, len(good)
    assert rel_err(g[good], fd) < RTOL


@pytest.mark.gpu
def test_torch_backward_is_the_adjoint():
    import torch
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300.autograd import energy
    N, sizes = 12, (24, 12, 6)
    psi = deep_net(N, sizes, 2)
    H = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    params = torch.tensor(psi.params, requires_grad=True)
    E = energy(params, psi, H, rg.MonteCarloLoop(256, 1, 5, 128, seed=8))
    assert params.grad is None
    E.backward()
    # the backward pass ran on the forward pass's samples: the same gradient, bit for bit,
    # as the adjoint on the same (seeded) Monte Carlo pass; the forward value is the mean
    # of that pass's local energies
    g, E2 = rg.ExpectationValue().eloc_gradient(psi, H, rg.MonteCarloLoop(256, 1, 5, 128, seed=8), score=True)
    assert abs(E.item() - E2.real) <= 1e-6 * abs(E2)
    np.testing.assert_array_equal(params.grad.numpy(), g)


def test_autograd_function_follows_torchs_complex_convention():
    """CPU check of the convention the Function relies on: for a real loss L of a
    complex leaf z, backward returns dL/dRe z + i dL/dIm z."""
    torch = pytest.importorskip("torch")

    class Sq(torch.autograd.Function):
        @staticmethod
        def forward(ctx, z):
            ctx.save_for_backward(z)
            return (z * z).real.sum()

        @staticmethod
        def backward(ctx, g):
            (z,) = ctx.saved_tensors
            return g.to(z.dtype) * torch.conj(2 * z)

    z = torch.tensor([1 + 2j, 0.5 - 1j], dtype=torch.complex128, requires_grad=True)
    Sq.apply(z).backward()
    w = torch.tensor([1 + 2j, 0.5 - 1j], dtype=torch.complex128, requires_grad=True)
    (w * w).real.sum().backward()
    assert torch.equal(z.grad, w.grad)


# ----------------------------------------------------------------------------- complex RBM
# The RBM path computes local energies in FP32, whose round-off over a step of 1e-5 would
# swamp a finite difference; its derivative is checked against FP64 central differences
# of the CPU restatement (oracle/pyoracle.py) at the same parameters and samples.
def rbm_net(N, M, seed, sigma):
    import rbmongpu_gb300 as rg
    rng = np.random.Generator(np.random.PCG64(seed))
    b = sigma * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = sigma * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    return rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True), b, W


def oracle_rbm(p, N, M):
    from oracle import pyoracle as po
    return po.RBM(p[2 * N:2 * N + M], p[2 * N + M:].reshape(N, M), 1.0)


def fd_oracle(loss, p0, grad, idx, h=1e-5, rtol=RTOL):
    """fd_check on a loss of the parameter vector (FP64, no device)."""
    vals = {}
    for k in idx:
        d = []
        for hh in (h, 2 * h):
            v = []
            for step in (hh, 1j * hh):
                p = p0.copy()
                p[k] += step
                lp = loss(p)
                p[k] -= 2 * step
                v.append((lp - loss(p)) / (2 * hh))
            d.append(v[0] + 1j * v[1])
        vals[k] = d
    scale = np.abs(grad).max()
    good = [k for k in idx if abs(vals[k][0] - vals[k][1]) <= 0.5 * rtol * scale]
    return np.array(good), np.array([vals[k][0] for k in good])


@pytest.mark.gpu
@pytest.mark.parametrize("N,M", [(12, 24), (40, 80)])
def test_rbm_fixed_sample_derivative_matches_fp64_finite_differences(N, M):
    """Psi: score=False is the derivative of Re <E_loc> over the samples held fixed."""
    import rbmongpu_gb300 as rg
    from oracle import pyoracle as po
    psi, b, W = rbm_net(N, M, 41, 0.2)
    H_t = rg.operators.tfim_chain(N, 1.0, 1.0)
    H = rg.Operator(*H_t)
    mk = lambda: rg.MonteCarloLoop(64, 1, 5, 32, seed=13)   # noqa: E731
    sp, _, _ = mk().samples(psi)
    g, E = rg.ExpectationValue().eloc_gradient(psi, H, mk(), score=False)
    el = rg.local_energies(psi, H, sp)
    assert abs(E - el.mean()) <= 1e-5 * np.abs(el).mean()
    op = po.Op(*H_t)
    words = [np.asarray([s], np.uint64) for s in sp]

    def loss(p):
        o = oracle_rbm(p, N, M)
        return np.mean([po.local_energy(o, op, s).real for s in words])

    good, fd = fd_oracle(loss, psi.params, g, param_indices(psi, 32, 7))
    assert len(good) >= 24, len(good)
    assert rel_err(g[good], fd) < RTOL, (g[good][:4], fd[:4])
    assert np.all(g[:2 * N] == 0)


@pytest.mark.gpu
def test_rbm_exact_summation_gradient_matches_finite_differences_and_the_reference_estimator():
    """Psi, normalised, ExactSummation: score=True is the gradient of <H> and equals the
    reference's O_k estimator (ExpectationValue.cu:243-253) for the hermitian TFIM."""
    import rbmongpu_gb300 as rg
    from oracle import pyoracle as po
    N, M = 8, 16
    psi, b, W = rbm_net(N, M, 43, 0.3)
    H_t = rg.operators.tfim_chain(N, 1.0, 1.0)
    H = rg.Operator(*H_t)
    es = rg.ExactSummation(N)
    op = po.Op(*H_t)

    def energy(p):
        o = oracle_rbm(p, N, M)
        sig, E = po.exact_fluctuation(o, op)
        return E.real / po.exact_norm(o) ** 2

    p0 = psi.params
    psi.prefactor = 1.0 / psi.norm(es)
    g, E = rg.ExpectationValue().eloc_gradient(psi, H, es, score=True)
    assert abs(E.real - energy(p0)) <= 1e-5 * abs(E)
    gr, _ = rg.ExpectationValue().gradient(psi, H, es)
    assert rel_err(g, gr) < RTOL
    good, fd = fd_oracle(energy, p0, g, param_indices(psi, 32, 9))
    assert len(good) >= 24, len(good)
    assert rel_err(g[good], fd) < RTOL


@pytest.mark.gpu
def test_rbm_torch_backward():
    import torch
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300.autograd import energy
    N, M = 16, 32
    psi, _, _ = rbm_net(N, M, 47, 0.1)
    H = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    params = torch.tensor(psi.params, requires_grad=True)
    E = energy(params, psi, H, rg.MonteCarloLoop(256, 1, 5, 128, seed=8))
    assert params.grad is None
    E.backward()
    # the backward pass ran on the forward pass's samples: the same gradient, bit for bit,
    # as the adjoint on the same (seeded) Monte Carlo pass; the forward value is the mean
    # of that pass's local energies
    g, E2 = rg.ExpectationValue().eloc_gradient(psi, H, rg.MonteCarloLoop(256, 1, 5, 128, seed=8), score=True)
    assert abs(E.item() - E2.real) <= 1e-6 * abs(E2)
    np.testing.assert_array_equal(params.grad.numpy(), g)
