"""The PsiDeep adjoint kernel taking a sample's neighbours two, four or eight at a time against
the kernel taking them one at a time: every configuration's arithmetic and the local
energy's order of summation are the same, so the gradient and <E_loc> are identical, with
and without the sampling term, on Monte Carlo samples and on exact summation, for
operators whose strings flip one spin (TFIM) and two spins (Heisenberg exchange)."""
import os

import numpy as np
import pytest

import rbmongpu_gb300 as rg
from golden_cases import Case

pytestmark = pytest.mark.gpu


def dense_net(N, sizes, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    b, conn, W = [], [], []
    fan = N
    for m in sizes:
        sd = np.sqrt(0.3 / fan / 2)
        b.append(rng.normal(0, sd, m) + 1j * rng.normal(0, sd, m))
        conn.append(np.array([[c] * m for c in range(fan)]))
        W.append(rng.normal(0, sd, (fan, m)) + 1j * rng.normal(0, sd, (fan, m)))
        fan = m
    return rg.PsiDeep(np.zeros(N), np.zeros(N), b, conn, W, np.ones(sizes[-1]), 1.0, False, True)


def gradient(psi, op, ens, score, batch):
    old = os.environ.get("RBMG_DEEP_ADJOINT_BATCH")
    os.environ["RBMG_DEEP_ADJOINT_BATCH"] = str(batch)
    try:
        return rg.ExpectationValue().eloc_gradient(psi, op, ens(), score=score)
    finally:
        if old is None:
            del os.environ["RBMG_DEEP_ADJOINT_BATCH"]
        else:
            os.environ["RBMG_DEEP_ADJOINT_BATCH"] = old


@pytest.mark.parametrize("score", [False, True])
@pytest.mark.parametrize("batch", [2, 4, 8])
def test_tfim_n70_monte_carlo(batch, score):
    psi = dense_net(70, (90, 40, 20), 41)
    op = rg.Operator(*rg.operators.tfim_chain(70, 1.0, 0.8))
    ens = lambda: rg.MonteCarloLoop(96 * 2, 1, 3, 96, seed=9)   # noqa: E731
    g1, E1 = gradient(psi, op, ens, score, 1)
    gb, Eb = gradient(psi, op, ens, score, batch)
    assert np.array_equal(g1, gb) and E1 == Eb


@pytest.mark.parametrize("batch", [2, 4, 8])
def test_sparse_net_exact_summation_heisenberg(batch):
    c = Case("deep8_sparse")
    b, cn, w, fw = c.deep("")
    psi = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    op = rg.Operator(*rg.operators.heisenberg_chain(c.N, 1.0))
    ens = lambda: rg.ExactSummation(c.N)   # noqa: E731
    g1, E1 = gradient(psi, op, ens, True, 1)
    gb, Eb = gradient(psi, op, ens, True, batch)
    assert np.array_equal(g1, gb) and E1 == Eb
