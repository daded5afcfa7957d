"""Learned cluster-flip proposal: the CPU restatement of its network (pinned by finite
differences), the CUDA forward / backward / Adam kernels against it, exactness of the
Metropolis-Hastings chain that uses it, and what training gains over the untrained
(uniform) proposal.

Tolerances: logits within 3e-3 of their largest magnitude and gradients within 1e-2 of
each tensor's largest entry (BF16 operands: a pre-activation that lands within FP32
round-off of a BF16 rounding boundary rounds the other way on one side); Adam within
1e-6 relative.
"""
import numpy as np
import pytest

from oracle import proposal_ref as pr


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1.0 + 2.0 ** -9], np.float32)
    np.testing.assert_array_equal(pr.bf16(x), np.array([1.0, 1.0, 1.0 + 2.0 ** -6, -2.5, 1.0], np.float32))


def test_restated_backward_is_the_derivative_of_the_forward():
    N, B = 12, 5
    rng = np.random.default_rng(11)
    lay, total = pr.layout(N)
    params = rng.normal(0, 0.15, total)
    words = rng.integers(0, 2 ** N, B, dtype=np.uint64).reshape(B, 1)
    dl = rng.normal(0, 1, (B, N + pr.LENGTHS))
    _, cache = pr.forward(params, words, N, exact=True)
    g = pr.backward(cache, dl, N, exact=True)
    loss = lambda q: float((pr.forward(q, words, N, exact=True)[0] * dl).sum())
    idx = np.concatenate([rng.choice(np.arange(o, o + int(np.prod(s))), 6, replace=False) for o, s in lay.values()])
    for k in idx:
        e = np.zeros(total)
        e[k] = 1e-5
        fd = (loss(params + e) - loss(params - e)) / 2e-5
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def random_params(N, seed):
    rng = np.random.default_rng(seed)
    lay, total = pr.layout(N)
    d = pr.unpack(np.zeros(total, np.float32), N)
    d["W1"][:] = rng.uniform(-1, 1, d["W1"].shape) * np.sqrt(6 / N)
    d["W2"][:] = rng.uniform(-1, 1, d["W2"].shape) * np.sqrt(6 / pr.HIDDEN)
    d["W3"][:] = rng.normal(0, 0.1, d["W3"].shape)
    for b in ("b1", "b2", "b3"):
        d[b][:] = rng.normal(0, 0.1, d[b].shape)
    return pr.pack(d, N)


def random_words(N, count, seed):
    rng = np.random.default_rng(seed)
    nw = (N + 63) // 64
    w = rng.integers(0, 2 ** 63, (count, nw), dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, (count, nw), dtype=np.uint64)
    if N % 64:
        w[:, -1] &= np.uint64((1 << (N % 64)) - 1)
    return w


def rel_err(a, b):
    return np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("N,count", [(20, 333), (100, 1000), (128, 300)])
def test_forward_and_backward_match_restatement(N, count):
    """eval without dlogits runs the inference kernel (tcgen05 for N + 8 <= 128, the fused
    mma.sync kernel above), with dlogits the layer-by-layer GEMMs and the backward pass."""
    import rbmongpu_gb300 as rg
    prop = rg.Proposal(N, seed=5)
    params = random_params(N, 17 + N)
    prop.params = params
    np.testing.assert_array_equal(prop.params, params)
    words = random_words(N, count, 3)
    dl = np.random.default_rng(4).normal(0, 1, (count, N + 8)).astype(np.float32)
    logits, grads = prop.eval(words, dl)
    ref_logits, cache = pr.forward(params, words, N)
    assert rel_err(logits, ref_logits) < 3e-3
    ref_g = pr.backward(cache, dl, N)
    lay, _ = pr.layout(N)
    for name, (o, s) in lay.items():
        n = int(np.prod(s))
        assert rel_err(grads[o:o + n], ref_g[o:o + n]) < 1e-2, name
    inf = prop.eval(words)
    if N + 8 > 128:
        np.testing.assert_array_equal(inf, logits)   # same k order and epilogue as the GEMMs
    else:
        assert rel_err(inf, ref_logits) < 3e-3       # tensor-core accumulation order differs
        assert rel_err(inf, logits) < 3e-3
    np.testing.assert_array_equal(prop.eval(words), inf)   # deterministic
    prop.status()


@pytest.mark.gpu
def test_adam_matches_restatement():
    import rbmongpu_gb300 as rg
    N = 16
    prop = rg.Proposal(N, seed=1, lr=1e-3)
    p0 = random_params(N, 2)
    prop.params = p0
    rng = np.random.default_rng(9)
    m = np.zeros(p0.size)
    v = np.zeros(p0.size)
    p = p0.astype(np.float64)
    for step in (1, 2, 3):
        g = rng.normal(0, 1, p0.size).astype(np.float32)
        prop.adam(g)
        p, m, v = pr.adam(p, g.astype(np.float64), m, v, step, 1e-3)
    got = prop.params.astype(np.float64)
    assert np.abs(got - p).max() <= 1e-6 * np.abs(p).max() + 1e-7


def small_rbm(N, M, sigma, seed):
    import rbmongpu_gb300 as rg
    rng = np.random.default_rng(seed)
    b = rng.normal(0, sigma, M) + 1j * rng.normal(0, sigma, M)
    W = rng.normal(0, sigma, (N, M)) + 1j * rng.normal(0, sigma, (N, M))
    return rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)


def chi_square(p, states, B):
    """Chi-square of B sampled states against the probabilities p, states grouped (in
    order of probability) to at least 20 expected counts; returns (chi2, dof)."""
    counts = np.bincount(np.asarray(states, np.int64), minlength=p.size)
    chi2, dof, e_acc, c_acc = 0.0, -1, 0.0, 0
    for s in np.argsort(p):
        e_acc += p[s] * B
        c_acc += counts[s]
        if e_acc >= 20:
            chi2 += (c_acc - e_acc) ** 2 / e_acc
            dof += 1
            e_acc, c_acc = 0.0, 0
    return chi2, dof


def chi_square_ok(chi2, dof):
    return chi2 < dof + 6 * np.sqrt(2 * dof)


EXACT_N, EXACT_M, EXACT_SIGMA, EXACT_STEPS = 10, 20, 0.15, 500


def exactness_setup():
    """N=10 RBM (sigma 0.15) and a random, clearly non-uniform proposal network."""
    from oracle import pyoracle as po
    rng = np.random.default_rng(5)
    b = rng.normal(0, EXACT_SIGMA, EXACT_M) + 1j * rng.normal(0, EXACT_SIGMA, EXACT_M)
    W = rng.normal(0, EXACT_SIGMA, (EXACT_N, EXACT_M)) + 1j * rng.normal(0, EXACT_SIGMA, (EXACT_N, EXACT_M))
    words = np.arange(2 ** EXACT_N, dtype=np.uint64)
    lp = np.array([po.log_psi(po.RBM(b, W, 1.0), int(w)) for w in words]).real
    p = np.exp(2 * (lp - lp.max()))
    return b, W, lp, p / p.sum(), random_params(EXACT_N, 8)


def test_chi_square_detects_a_chain_without_the_reverse_density():
    """CPU emulation of the learned chain: the chi-square statistic of the GPU test
    accepts the exact chain and rejects one that drops q(s|s') / q(s'|s)."""
    _, _, lp, p, params = exactness_setup()
    words = np.arange(2 ** EXACT_N, dtype=np.uint64).reshape(-1, 1)
    logits, _ = pr.forward(params, words, EXACT_N, exact=True)
    B = 8192
    good, _ = pr.emulate_chain(lp, logits, EXACT_N, B, EXACT_STEPS, 1)
    bad, _ = pr.emulate_chain(lp, logits, EXACT_N, B, EXACT_STEPS, 1, with_reverse=False)
    assert chi_square_ok(*chi_square(p, good, B))
    assert not chi_square_ok(*chi_square(p, bad, B))


@pytest.mark.gpu
def test_learned_chain_samples_psi_squared():
    """A frozen, non-uniform proposal: the final states of 16384 independent walkers
    follow |psi|^2 (chi-square over states grouped to >= 20 expected counts)."""
    import rbmongpu_gb300 as rg
    B = 16384
    b, W, _, p, params = exactness_setup()
    psi = rg.Psi(np.zeros(EXACT_N), np.zeros(EXACT_N), b, W, 1.0, False, True)
    prop = rg.Proposal(EXACT_N, seed=2)
    prop.params = params
    chain = rg.Chain(psi, B, seed=77)
    chain.learned_async(psi, None, prop, EXACT_STEPS, train=0)
    words, acc, props = chain.state()
    prop.status()
    assert props == EXACT_STEPS * B and 0.05 < acc / props < 1
    chi2, dof = chi_square(p, words[:, 0], B)
    assert dof > 100 and chi_square_ok(chi2, dof), (chi2, dof)


def lb_marginals(psi, words, N):
    """Seed and length marginals of the locally balanced proposal p*(i, l) propto
    exp(Re log psi(s') - Re log psi(s)) over all N x 8 contiguous cluster flips."""
    L = pr.LENGTHS
    masks = np.zeros((N, L), np.uint64)
    for i in range(N):
        for l in range(1, L + 1):
            masks[i, l - 1] = sum(1 << ((i + q) % N) for q in range(l))
    w = np.asarray(words, np.uint64).reshape(-1)
    lp0 = psi.log_psi_batch(w).real
    moved = (w[:, None, None] ^ masks[None]).reshape(-1)
    lp = psi.log_psi_batch(moved).real.reshape(len(w), N, L) - lp0[:, None, None]
    p = np.exp(lp - lp.max(axis=(1, 2), keepdims=True))
    p /= p.sum(axis=(1, 2), keepdims=True)
    return p.sum(axis=2), p.sum(axis=1)


def mean_kl(ps, pl, logits, N):
    ls = logits[:, :N] - np.logaddexp.reduce(logits[:, :N], axis=1, keepdims=True)
    ll = logits[:, N:] - np.logaddexp.reduce(logits[:, N:], axis=1, keepdims=True)
    kl = (ps * (np.log(ps + 1e-300) - ls)).sum(axis=1) + (pl * (np.log(pl + 1e-300) - ll)).sum(axis=1)
    return float(kl.mean())


@pytest.mark.gpu
def test_training_fits_the_locally_balanced_proposal():
    """N=20 RBM (sigma 0.25): online training brings the proposal's seed and length
    distributions to the locally balanced marginals (mean KL at the chain's states at
    most half the untrained one), and the frozen trained proposal accepts at least 1.5x
    as many moves as the untrained (uniform) one."""
    import rbmongpu_gb300 as rg
    N, B = 20, 4096
    psi = small_rbm(N, 40, 0.25, 6)

    def rate(chain, prop, steps):
        _, a0, p0 = chain.state()
        chain.learned_async(psi, None, prop, steps, train=0)
        _, a1, p1 = chain.state()
        return (a1 - a0) / (p1 - p0)

    prop = rg.Proposal(N, seed=3)
    chain = rg.Chain(psi, B, seed=5)
    chain.sweep_async(psi, None, 50)
    untrained = rate(chain, prop, 100)
    words = chain.state()[0][:256]
    ps, pl = lb_marginals(psi, words, N)
    kl0 = mean_kl(ps, pl, prop.eval(words), N)
    chain.learned_async(psi, None, prop, 600, train=1024)
    words = chain.state()[0][:256]
    ps, pl = lb_marginals(psi, words, N)
    kl1 = mean_kl(ps, pl, prop.eval(words), N)
    assert kl1 < 0.5 * kl0, (kl0, kl1)
    trained = rate(chain, prop, 100)
    assert trained >= 1.5 * untrained, (untrained, trained)


@pytest.mark.gpu
def test_trained_chain_energy_matches_exact_summation():
    """N=20 RBM with sigma 0.12 (where single-flip chains equilibrate within a few
    hundred sweeps): the frozen trained proposal's chain reproduces the exact energy
    within 5 standard errors of its walker means (walkers are independent chains)."""
    import rbmongpu_gb300 as rg
    import torch
    N, B, rows = 20, 4096, 40
    psi = small_rbm(N, 40, 0.12, 6)
    op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    prop = rg.Proposal(N, seed=4)
    chain = rg.Chain(psi, B, seed=9)
    chain.sweep_async(psi, None, 200)
    chain.learned_async(psi, None, prop, 300, train=1024)
    chain.learned_async(psi, None, prop, 500, train=0)
    el = torch.zeros((rows, B, 2), dtype=torch.float64, device="cuda")
    chain.learned_async(psi, op, prop, rows * 10, train=0, measure_every=10, d_eloc=el.data_ptr(),
                        stream=rg.library_stream())
    torch.cuda.synchronize()
    e = el[..., 0].cpu().numpy()
    es = rg.ExactSummation(N)
    E = rg.ExpectationValue()(psi, op, es) / psi.norm(es) ** 2
    se = e.mean(axis=0).std() / np.sqrt(B)
    assert abs(e.mean() - E.real) < 5 * se + 1e-3, (e.mean(), E.real, se)


@pytest.mark.gpu
def test_reinforce_objective_raises_the_acceptance():
    import rbmongpu_gb300 as rg
    N, B = 20, 4096
    psi = small_rbm(N, 40, 0.25, 6)
    prop = rg.Proposal(N, seed=3, objective=rg.Proposal.REINFORCE)
    chain = rg.Chain(psi, B, seed=5)
    chain.sweep_async(psi, None, 50)
    _, a0, p0 = chain.state()
    chain.learned_async(psi, None, prop, 100, train=0)
    _, a1, p1 = chain.state()
    chain.learned_async(psi, None, prop, 300, train=B)
    chain.learned_async(psi, None, prop, 100, train=0)
    _, a2, p2 = chain.state()
    assert (a2 - a1) / (p2 - p1) >= 1.5 * (a1 - a0) / (p1 - p0)
