"""CPU restatement of the learned proposal network (numpy).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA forward,
backward and Adam kernels.  The product package never imports it.

The proposal is an extension with no counterpart in the reference, so this module is
pinned by its own finite-difference check (``exact=True`` switches the BF16 roundings
off so that the backward pass is the exact derivative of the forward pass) rather than
by reference outputs.

With ``exact=False`` it mirrors the device's precision choices: operands of every
matrix product rounded to BF16 (round to nearest even), products accumulated in FP64
(the device accumulates in FP32), pre-activations and biases in FP32.
"""
import numpy as np

HIDDEN = 256
LENGTHS = 8


def bf16(x):
    """Round float32 values to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def layout(N):
    """Offsets of W1 [N][H], b1, W2 [H][H], b2, W3 [H][N+8], b3 in the parameter vector."""
    H, O = HIDDEN, N + LENGTHS
    sizes = [("W1", (N, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, O)), ("b3", (O,))]
    out, off = {}, 0
    for name, shape in sizes:
        n = int(np.prod(shape))
        out[name] = (off, shape)
        off += n
    return out, off


def unpack(params, N):
    lay, total = layout(N)
    assert params.shape == (total,)
    return {k: params[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def pack(d, N):
    lay, total = layout(N)
    out = np.zeros(total, np.float32)
    for k, (o, s) in lay.items():
        out[o:o + int(np.prod(s))] = np.asarray(d[k], np.float32).reshape(-1)
    return out


def spins_to_x(words, N):
    """uint64 words [B][nw] -> +-1 float [B][N] (bit i set <=> s_i = +1)."""
    words = np.asarray(words, np.uint64).reshape(len(words), -1)
    i = np.arange(N)
    bits = (words[:, i // 64] >> (i % 64).astype(np.uint64)) & np.uint64(1)
    return np.where(bits == 1, 1.0, -1.0)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def _rnd(x, exact):
    return np.asarray(x, np.float64) if exact else bf16(np.asarray(x, np.float32)).astype(np.float64)


def forward(params, words, N, exact=False):
    p = unpack(np.asarray(params, np.float64 if exact else np.float32), N)
    f32 = (lambda v: np.asarray(v, np.float64)) if exact else (lambda v: np.asarray(v, np.float32).astype(np.float64))
    x = spins_to_x(words, N)
    z1 = f32(x @ _rnd(p["W1"], exact) + p["b1"].astype(np.float64))
    h1 = _rnd(z1 * _sig(z1), exact)
    z2 = f32(h1 @ _rnd(p["W2"], exact) + p["b2"].astype(np.float64))
    h2 = _rnd(z2 * _sig(z2), exact)
    logits = f32(h2 @ _rnd(p["W3"], exact) + p["b3"].astype(np.float64))
    return logits, dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, p=p)


def backward(cache, dlogits, N, exact=False):
    """Gradient of sum(dlogits * logits) with respect to the parameters (packed)."""
    p = cache["p"]
    dl = np.asarray(dlogits, np.float64)
    dlr = _rnd(dl, exact)

    def dsilu(z):
        s = _sig(z)
        return s * (1.0 + z * (1.0 - s))

    g = {"W3": cache["h2"].T @ dlr, "b3": dl.sum(axis=0)}
    dz2 = (dlr @ _rnd(p["W3"], exact).T) * dsilu(cache["z2"])
    dz2r = _rnd(dz2, exact)
    g["W2"] = cache["h1"].T @ dz2r
    g["b2"] = dz2.sum(axis=0)
    dz1 = (dz2r @ _rnd(p["W2"], exact).T) * dsilu(cache["z1"])
    g["W1"] = cache["x"].T @ _rnd(dz1, exact)
    g["b1"] = dz1.sum(axis=0)
    return pack(g, N).astype(np.float64)


def adam(params, grads, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (Kingma & Ba 2015); step counts from 1."""
    m = b1 * m + (1 - b1) * grads
    v = b2 * v + (1 - b2) * grads * grads
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def log_q(logits, N, seed, length):
    """log of the proposal probability of (seed site, cluster length) under the logits."""
    ls = logits[:N] - np.logaddexp.reduce(logits[:N])
    ll = logits[N:] - np.logaddexp.reduce(logits[N:])
    return ls[seed] + ll[length - 1]


def emulate_chain(log_psi_re, logits_all, N, B, steps, seed, with_reverse=True):
    """Vectorised emulation of the learned Metropolis-Hastings chain over an enumerated
    state space (state = spin bit pattern, N <= 20): seed and length drawn by inverse
    CDF, the contiguous periodic cluster flipped, accepted with
    min(1, exp(2 dRe log psi) q(s|s') / q(s'|s)).  with_reverse=False drops the density
    ratio (a deliberately wrong chain, used to show that the tests detect it).
    Returns the final states of B independent walkers and the acceptance rate."""
    r = np.random.default_rng(seed)
    ls = logits_all[:, :N] - np.logaddexp.reduce(logits_all[:, :N], axis=1, keepdims=True)
    ll = logits_all[:, N:] - np.logaddexp.reduce(logits_all[:, N:], axis=1, keepdims=True)
    state = r.integers(0, 2 ** N, B)
    acc = 0
    for _ in range(steps):
        cs = np.cumsum(np.exp(ls[state]), axis=1)
        i = (cs < r.random(B)[:, None] * cs[:, -1:]).sum(axis=1).clip(0, N - 1)
        cl = np.cumsum(np.exp(ll[state]), axis=1)
        l = 1 + (cl < r.random(B)[:, None] * cl[:, -1:]).sum(axis=1).clip(0, LENGTHS - 1)
        mask = np.zeros(B, np.int64)
        for q in range(LENGTHS):
            mask |= np.where(q < l, 1 << ((i + q) % N), 0)
        new = state ^ mask
        loga = 2 * (log_psi_re[new] - log_psi_re[state])
        if with_reverse:
            loga = loga + ls[new, i] + ll[new, l - 1] - ls[state, i] - ll[state, l - 1]
        a = r.random(B) < np.exp(np.minimum(loga, 0.0))
        acc += int(a.sum())
        state = np.where(a, new, state)
    return state, acc / (B * steps)


def logcosh_ref(z):
    """The reference's rational activation in FP64, vectorised
    (include/quantum_state/psi_functions.hpp:49-57)."""
    z = np.asarray(z, np.complex128)
    sg = np.where(z.real > 0.0, 1.0, -1.0)
    t = z * (sg * 3.746646023906276 + z) + 7.771429504240965
    t = z * t + sg * 10.2180213465
    t = z * t + 9.19376335670885
    num = (5.49914721954 - sg * 2.16564366435 * z.real) - 1j * sg * 2.16564366435 * z.imag
    return sg * 0.9003320053750442 * z + num / t - 0.598139


def lb_target(W, b, words, logits, N):
    """The locally balanced training target of proposal.cu::lb_target_kernel in FP64:
    for every seed i and length l the cluster move's Re Delta = Re log psi(s') - Re log psi(s)
    (Zanella 2020: p*(i, l) propto exp(Re Delta) = |psi(s')/psi(s)|), the seed and length
    marginals of p*, and dl = (softmax(logits) - marginal) / count.
    W [N][M] and b [M] are the RBM's complex parameters as the device holds them."""
    x = spins_to_x(words, N)                              # [B][N] +-1
    count = len(x)
    theta = x @ W + b                                     # [B][M]
    base = logcosh_ref(theta).real.sum(axis=1)            # [B]
    delta = np.zeros((count, N, LENGTHS))
    for i in range(N):
        th = theta.copy()
        for q in range(LENGTHS):
            c = (i + q) % N
            th = th - 2.0 * x[:, c:c + 1] * W[c][None, :]
            delta[:, i, q] = logcosh_ref(th).real.sum(axis=1) - base
    m = delta.reshape(count, -1).max(axis=1)[:, None, None]
    p = np.exp(delta - m)
    p /= p.sum(axis=(1, 2), keepdims=True)
    lg = np.asarray(logits, np.float64)
    qs = np.exp(lg[:, :N] - np.logaddexp.reduce(lg[:, :N], axis=1, keepdims=True))
    ql = np.exp(lg[:, N:] - np.logaddexp.reduce(lg[:, N:], axis=1, keepdims=True))
    dl = np.concatenate([qs - p.sum(axis=2), ql - p.sum(axis=1)], axis=1) / count
    return dl
