"""The factorised E_k term the GPU estimators use (the serving kernel's tiles and the
gradient pass: rbmongpu_gb300/csrc/serving.cu, rbm_impl.cuh EST_GRADVEC with
reduce_kernels.cu vterm_kernel), checked in FP64 against the reference's definition
E_k(s) = sum_n e_n O_k(s'_n) (include/operator/Operator.hpp:145-179) evaluated term by
term with the oracle's O_k:

    E_k(b_j)  = U_j                  U_j  = sum_n e_n tanh(theta''_nj)
    E_k(W_ij) = s_i (U_j - 2 V_ij)   V_ij = sum over the strings n that flip i of e_n tanh(theta''_nj)

and the gradient assembled from it, <E O*> + conj<E_k> - 2 <E><O*>
(source/network_functions/ExpectationValue.cu:243-253), against the oracle's own
estimator on the same configurations.  Operators with single-flip strings, two-site
flips and several strings per site (the serving kernel's single-flip and general tiles)."""
import numpy as np

from oracle import pyoracle as po

X, Z = 1, 3


def operator(N):
    strings = [[(Z, i), (Z, (i + 1) % N)] for i in range(N)] + [[(X, i)] for i in range(N)]
    strings += [[(X, 2), (X, 3)], [(X, 7), (X, 8)], [(X, 5), (Z, 6)]]
    coefs = [-1.0] * N + [-0.8] * N + [0.3, -0.45 + 0.1j, 0.25]
    L = 3
    types = np.zeros((len(strings), L), np.int32)
    idx = -np.ones((len(strings), L), np.int32)
    for n, s in enumerate(strings):
        for c, (t, i) in enumerate(s):
            types[n, c], idx[n, c] = t, i
    return strings, np.asarray(coefs, np.complex128), types, idx


def test_factorised_ek_and_gradient():
    N, M = 10, 20
    rng = np.random.default_rng(31)
    b = 0.3 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = 0.3 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    psi = po.RBM(b, W, 1.0)
    strings, coef, types, idx = operator(N)
    op = po.Op(coef, types, idx)
    configs = rng.integers(0, 1 << N, 24)
    spins = po.spins_array([int(c) for c in configs], N)
    P = psi.num_params
    tanh = np.vectorize(po.tanh)

    def sgn(word, i):
        return 1.0 if (int(word) >> i) & 1 else -1.0

    Os, Es, Eks = [], [], []
    for row in spins:
        word = int(row[0])
        s = np.array([sgn(word, i) for i in range(N)])
        lp = po.log_psi(psi, row)
        O = po.O_k(psi, row)
        # the O_k layout of the reference: [alpha, beta, b, W], W row-major [i][j]
        theta = b + s @ W
        np.testing.assert_allclose(O[2 * N:2 * N + M], tanh(theta), rtol=1e-12)
        np.testing.assert_allclose(O[2 * N + M:].reshape(N, M), s[:, None] * tanh(theta)[None, :], rtol=1e-12)
        U = np.zeros(M, np.complex128)
        V = np.zeros((N, M), np.complex128)
        Ek_naive = np.zeros(P, np.complex128)
        E = 0.0
        for n, st in enumerate(strings):
            flips = [i for t, i in st if t == X]
            zf = np.prod([s[i] for t, i in st if t == Z]) if any(t == Z for t, _ in st) else 1.0
            w2 = word
            for i in flips:
                w2 ^= 1 << i
            row2 = np.array([w2], np.uint64)
            e = coef[n] * zf * np.exp(po.log_psi(psi, row2) - lp)
            E += e
            Ek_naive += e * po.O_k(psi, row2)
            s2 = np.array([sgn(w2, i) for i in range(N)])
            th2 = tanh(b + s2 @ W)
            U += e * th2
            for i in flips:
                V[i] += e * th2
        assert abs(E - po.local_energy(psi, op, row)) <= 1e-12 * abs(E)
        Ek = np.zeros(P, np.complex128)
        Ek[2 * N:2 * N + M] = U
        Ek[2 * N + M:] = (s[:, None] * (U[None, :] - 2.0 * V)).ravel()
        scale = np.abs(Ek_naive).max()
        assert np.abs(Ek - Ek_naive).max() <= 1e-12 * scale
        Os.append(O)
        Es.append(E)
        Eks.append(Ek)
    Os, Es, Eks = np.array(Os), np.array(Es), np.array(Eks)
    Em = Es.mean()
    g = (Es[:, None] * Os.conj()).mean(axis=0) + Eks.mean(axis=0).conj() - 2.0 * Em * Os.conj().mean(axis=0)
    og, oE = po.samples_gradient(psi, op, spins)
    assert abs(Em - oE) <= 1e-12 * abs(oE)
    assert np.abs(g - og).max() <= 1e-10 * np.abs(og).max()
