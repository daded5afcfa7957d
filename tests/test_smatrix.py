"""S matrix: the CPU restatement (oracle/pyoracle.py::s_matrix) against the reference's own
get_S_matrix (tests/golden/rbm6_smatrix.npz, from its host build), and the CUDA kernels
(rbmg_s_matrix) against both.

Tolerance: 1e-5 of the largest entry (complex64 tanh rows, FP32 products accumulated
over at most 1024 samples before the FP64 sum; the RBM path's tolerance elsewhere).  Both
product paths are held to it: the tensor cores (BF16 hi / mid / lo parts, the default) and
the FP32 CUDA-core tile kernel (simt=True).
"""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po

RTOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def all_states(N):
    return np.arange(2 ** N, dtype=np.uint64)[:, None]


def exact_weights(opsi, N):
    v = po.psi_vector(opsi)
    w = np.abs(v) ** 2
    return w / w.sum()


# ----------------------------------------------------------------------------- CPU
def test_restatement_matches_reference():
    c = Case("rbm6_smatrix")
    b, W = c.rbm()
    S = po.s_matrix(po.RBM(b, W, c.prefactor), all_states(c.N))
    ref = c.o("smatrix").reshape(S.shape)
    assert rel(S, ref) < 1e-13
    assert np.abs(ref[: 2 * c.N]).max() == 0.0


def test_restatement_centered_is_psd_and_hermitian():
    c = Case("rbm6_smatrix")
    b, W = c.rbm()
    opsi = po.RBM(b, W, c.prefactor)
    S = po.s_matrix(opsi, all_states(c.N), exact_weights(opsi, c.N), centered=True)
    assert np.abs(S - S.conj().T).max() < 1e-14
    assert np.linalg.eigvalsh(S).min() > -1e-12


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


paths = pytest.mark.parametrize("simt", [False, True], ids=["tensor", "simt"])


@gpu
@paths
def test_reference_golden(simt):
    import rbmongpu_gb300 as rg
    c = Case("rbm6_smatrix")
    b, W = c.rbm()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    S = rg.get_S_matrix(psi, rg.ExactSummation(c.N), simt=simt)
    assert rel(S, c.o("smatrix").reshape(S.shape)) < RTOL


@gpu
@paths
@pytest.mark.parametrize("weighted,centered", [(False, False), (True, False), (True, True), (False, True)])
def test_exact_rbm_vs_restatement(weighted, centered, simt):
    import rbmongpu_gb300 as rg
    c = Case("c1_rbm_exact")
    b, W = c.rbm()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    opsi = po.RBM(b, W, c.prefactor)
    S = rg.get_S_matrix(psi, rg.ExactSummation(c.N), weighted=weighted, centered=centered, simt=simt)
    ref = po.s_matrix(opsi, all_states(c.N), exact_weights(opsi, c.N) if weighted else None, centered)
    assert rel(S, ref) < RTOL


@gpu
@paths
@pytest.mark.parametrize("weighted", [False, True])
def test_exact_deep_vs_restatement(weighted, simt):
    import rbmongpu_gb300 as rg
    c = Case("deep8_sparse")
    b, cn, w, fw = c.deep()
    psi = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    opsi = po.Deep(c.N, b, cn, w, fw, c.prefactor)
    S = rg.get_S_matrix(psi, rg.ExactSummation(c.N), weighted=weighted, centered=weighted, simt=simt)
    ref = po.s_matrix(opsi, all_states(c.N), exact_weights(opsi, c.N) if weighted else None, weighted)
    assert rel(S, ref) < RTOL     # FP64 rows (centred in FP64), FP32 products


def _ragged_rbm():
    rng = np.random.default_rng(31)
    N, M = 32, 60
    b = 0.05 * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = 0.05 * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    return N, M, b, W


@gpu
@paths
@pytest.mark.parametrize("centered", [True, False])
@pytest.mark.parametrize("samples,chains", [(2048, 512), (1500, 500)])
def test_monte_carlo_ragged_size_vs_restatement(samples, chains, centered, simt):
    """N = 32, M = 60: L = 1980 is no multiple of the 64- or 128-wide tiles; MC samples on
    the same Philox streams as a restatement over the sampled configurations (1500: a
    second window of 476 samples, not a multiple of the 16-sample stages).  The diagonal,
    a sum of positive terms, is also held to the tolerance of its own size."""
    import rbmongpu_gb300 as rg
    N, M, b, W = _ragged_rbm()
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    mk = lambda: rg.MonteCarloLoop(samples, 1, 10, chains, True, seed=3)   # noqa: E731
    sp, _, _ = mk().samples(psi)
    assert len(sp) == samples
    S = rg.get_S_matrix(psi, mk(), centered=centered, simt=simt)
    O = np.array([po.O_k(po.RBM(b, W, 1.0), s) for s in sp])
    if centered:
        O = O - O.mean(axis=0)
    ref = O.T @ O.conj() / len(O)
    assert rel(S, ref) < RTOL
    d, dref = np.diag(S)[2 * N:].real, np.diag(ref)[2 * N:].real
    assert (np.abs(d - dref) / dref).max() < RTOL
    assert np.abs(S - S.conj().T).max() == 0.0


@gpu
def test_tensor_and_simt_paths_agree_over_windows():
    """4096 MC samples (four 1024-sample windows) of the ragged RBM: the tensor-core and
    FP32 CUDA-core products agree to the tolerance, and the centred matrix is positive
    semi-definite to rounding."""
    import rbmongpu_gb300 as rg
    N, M, b, W = _ragged_rbm()
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    mk = lambda: rg.MonteCarloLoop(4096, 1, 10, 512, True, seed=8)   # noqa: E731
    St = rg.get_S_matrix(psi, mk(), centered=True)
    Ss = rg.get_S_matrix(psi, mk(), centered=True, simt=True)
    assert rel(St, Ss) < RTOL
    ev = np.linalg.eigvalsh(St[2 * N:, 2 * N:])
    assert ev.min() > -1e-5 * ev.max()


@gpu
def test_pair_is_rejected():
    import rbmongpu_gb300 as rg
    c = Case("pair3")
    b, cn, w, fw = c.deep()
    psi = rg.PsiPair(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    with pytest.raises(rg.RbmgError):
        rg.get_S_matrix(psi, rg.ExactSummation(c.N))
