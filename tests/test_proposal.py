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
@pytest.mark.parametrize("N,count", [(20, 333), (100, 1000)])
def test_forward_and_backward_match_restatement(N, count):
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
    np.testing.assert_array_equal(prop.eval(words), logits)   # forward alone, deterministic


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


def exact_probs(psi, N):
    words = np.arange(2 ** N, dtype=np.uint64)
    lp = psi.log_psi_batch(words)
    w = np.exp(2 * (lp.real - lp.real.max()))
    return w / w.sum()


@pytest.mark.gpu
def test_learned_chain_samples_psi_squared():
    """A frozen, non-uniform proposal: the final states of 16384 independent walkers
    follow |psi|^2 (chi-square over states grouped to >= 20 expected counts)."""
    import rbmongpu_gb300 as rg
    N, B = 10, 16384
    psi = small_rbm(N, 20, 0.3, 5)
    prop = rg.Proposal(N, seed=2)
    pv = random_params(N, 8)
    d = pr.unpack(pv, N)
    d["W3"] *= 10.0            # strongly non-uniform seeds and lengths
    prop.params = pr.pack(d, N)
    chain = rg.Chain(psi, B, seed=77)
    chain.learned_async(psi, None, prop, 400, train=0)
    words, acc, props = chain.state()
    assert props == 400 * B and 0 < acc < props
    p = exact_probs(psi, N)
    counts = np.bincount(words[:, 0].astype(np.int64), minlength=2 ** N)
    order = np.argsort(p)
    chi2, dof, e_acc, c_acc = 0.0, -1, 0.0, 0
    for s in order:
        e_acc += p[s] * B
        c_acc += counts[s]
        if e_acc >= 20:
            chi2 += (c_acc - e_acc) ** 2 / e_acc
            dof += 1
            e_acc, c_acc = 0.0, 0
    assert dof > 20, dof
    assert chi2 < dof + 6 * np.sqrt(2 * dof), (chi2, dof)


@pytest.mark.gpu
def test_training_raises_accepted_moves_and_keeps_the_energy():
    """N=20 RBM: after online training the frozen proposal accepts at least 1.5x as many
    moves per step as the untrained (uniform seed and length) one, and the learned
    chain's mean local energy agrees with exact summation."""
    import rbmongpu_gb300 as rg
    N, B = 20, 4096
    psi = small_rbm(N, 40, 0.25, 6)
    op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))

    def rate(chain, prop, steps):
        _, a0, p0 = chain.state()
        chain.learned_async(psi, None, prop, steps, train=0)
        _, a1, p1 = chain.state()
        return (a1 - a0) / (p1 - p0)

    prop = rg.Proposal(N, seed=3)
    chain = rg.Chain(psi, B, seed=5)
    chain.sweep_async(psi, None, 50)
    untrained = rate(chain, prop, 100)
    chain.learned_async(psi, None, prop, 400, train=B)
    trained = rate(chain, prop, 100)
    assert trained >= 1.5 * untrained, (untrained, trained)
    import torch
    rows = 40
    el = torch.zeros((rows, B, 2), dtype=torch.float64, device="cuda")
    chain.learned_async(psi, op, prop, rows * 10, train=0, measure_every=10, d_eloc=el.data_ptr(),
                        stream=rg.library_stream())
    torch.cuda.synchronize()
    e = el[..., 0].cpu().numpy()
    E = rg.ExpectationValue()(psi, op, rg.ExactSummation(N)) / psi.norm(rg.ExactSummation(N)) ** 2
    se = e.mean(axis=1).std() / np.sqrt(rows) + e.std() / np.sqrt(e.size)
    assert abs(e.mean() - E.real) < 6 * se + 1e-3, (e.mean(), E.real, se)
