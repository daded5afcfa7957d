"""The PsiDeep sampler's several-walkers-per-CTA kernel against its one-walker-per-CTA
kernel: single-flip chains of a complex net are the same chains (spins, log psi, local
energies and acceptance bit for bit) whatever the number of walkers per CTA, including
walker counts that leave the last CTA partly empty."""
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


def chains(psi, op, wpc, samples, sweeps, therm, walkers, seed):
    old = os.environ.get("RBMG_DEEP_WALKERS_PER_BLOCK")
    os.environ["RBMG_DEEP_WALKERS_PER_BLOCK"] = str(wpc)
    try:
        mc = rg.MonteCarloLoop(samples, sweeps, therm, walkers, seed=seed)
        sp, lp, el = mc.samples(psi, op)
        return np.asarray(sp), np.asarray(lp), np.asarray(el), mc.acceptance_rate
    finally:
        if old is None:
            del os.environ["RBMG_DEEP_WALKERS_PER_BLOCK"]
        else:
            os.environ["RBMG_DEEP_WALKERS_PER_BLOCK"] = old


@pytest.mark.parametrize("wpc", [2, 4, 8])
def test_sparse_net_chains_match_one_walker_per_block(wpc):
    c = Case("deep8_sparse")
    b, cn, w, fw = c.deep("")
    psi = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    op = rg.Operator(*c.op())
    ref = chains(psi, op, 1, 61 * 6, 2, 5, 61, 31)
    got = chains(psi, op, wpc, 61 * 6, 2, 5, 61, 31)
    for a, r in zip(got[:3], ref[:3]):
        assert np.array_equal(a, r)
    assert got[3] == ref[3]


@pytest.mark.parametrize("wpc", [2, 4, 8])
def test_dense_n100_chains_match_one_walker_per_block(wpc):
    psi = dense_net(100, (120, 60, 30), 33)
    op = rg.Operator(*rg.operators.tfim_chain(100, 1.0, 1.0))
    ref = chains(psi, op, 1, 203 * 3, 1, 2, 203, 5)
    got = chains(psi, op, wpc, 203 * 3, 1, 2, 203, 5)
    for a, r in zip(got[:3], ref[:3]):
        assert np.array_equal(a, r)
    assert got[3] == ref[3]
    assert 0.0 < got[3] < 1.0


def test_walkers_per_block_rejects_other_counts():
    psi = dense_net(12, (8,), 3)
    op = rg.Operator(*rg.operators.tfim_chain(12, 1.0, 1.0))
    with pytest.raises(rg.RbmgError):
        chains(psi, op, 3, 64, 1, 1, 32, 1)
