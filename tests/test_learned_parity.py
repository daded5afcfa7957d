"""Bit-level parity of the learned-proposal chain (rbmongpu_gb300/csrc/proposal.cu) with its
CPU replay (oracle/oracle.c::or_learned_replay), and the locally balanced training target
against an FP64 restatement.

The chain's frozen steps are traced on the GPU (Chain.learned_trace: the initial angles
and logits, the proposed states' logits of every step, every move and the spins after
every accept pass).  The replay is fed the device's initial angles and its logits -- the
tensor-core network's FP32 accumulation order is not restated -- and the same Philox
streams, and reproduces the draws (inverse-CDF over the deterministic softmax), the
acceptance ratios (cluster angle updates, Re f differences, fixed butterfly, forward and
reverse log q) and the decisions of the accept rule of
include/spin_ensembles/MonteCarloLoop.hpp:206-222.  Everything is compared bit for bit.

The training target dl = (q - p*) / n of lb_target_kernel (FP32 arithmetic) is compared with
the FP64 restatement to 1e-4 of its largest entry.
"""
import numpy as np
import pytest

from oracle import proposal_ref as pr
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

N, M, SIGMA, SEED = 100, 400, 0.1, 104     # the learned-proposal workload's RBM


def rbm():
    rng = np.random.Generator(np.random.PCG64(SEED))
    b = rng.normal(0, SIGMA, M) + 1j * rng.normal(0, SIGMA, M)
    W = rng.normal(0, SIGMA, (N, M)) + 1j * rng.normal(0, SIGMA, (N, M))
    return b, W


@pytest.mark.parametrize("walkers,steps,train", [(256, 50, 64), (128, 40, 0)])
def test_learned_chain_replays_bit_for_bit(walkers, steps, train):
    import rbmongpu_gb300 as rg
    b, W = rbm()
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    prop = rg.Proposal(N, seed=5, lr=1e-3)
    chain = rg.Chain(psi, walkers, seed=9)
    chain.sweep_async(psi, None, 200, 1, 0, None)
    if train:
        # a few online training steps, so that the logits are far from uniform
        chain.learned_async(psi, None, prop, 30, train, 1, 0, None)
    before = chain.checkpoint()
    tr = chain.learned_trace(psi, prop, steps)
    np.testing.assert_array_equal(tr["spins0"], before["spins"])
    np.testing.assert_array_equal(tr["rng0"], before["rng_index"])
    rep = po.learned_replay(W, tr, seed=9)
    np.testing.assert_array_equal(rep["site"], tr["site"])
    np.testing.assert_array_equal(rep["len"], tr["len"])
    np.testing.assert_array_equal(rep["logq"].view(np.uint32), tr["logq"].view(np.uint32))
    np.testing.assert_array_equal(rep["spins"], tr["spins"])
    gpu_acc = np.diff(np.concatenate([before["accepts"][None], tr["accepts"]]), axis=0)
    np.testing.assert_array_equal(rep["accepted"].astype(np.uint64), gpu_acc)
    np.testing.assert_array_equal(rep["rng_end"], tr["rng_end"])
    # the comparison is not vacuous: moves of several lengths, accepts and rejects
    assert len(np.unique(tr["len"])) >= 4
    assert 0 < rep["accepted"].sum() < rep["accepted"].size
    # and the chain state it leaves behind is the one the replay ends in
    after = chain.checkpoint()
    np.testing.assert_array_equal(after["spins"], rep["spins"][-1])


def test_locally_balanced_target_matches_fp64_restatement():
    import rbmongpu_gb300 as rg
    b, W = rbm()
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    prop = rg.Proposal(N, seed=5)
    chain = rg.Chain(psi, 64, seed=3)
    chain.sweep_async(psi, None, 100, 1, 0, None)
    words = chain.checkpoint()["spins"]
    logits = np.random.default_rng(4).normal(0, 1.5, (len(words), N + pr.LENGTHS)).astype(np.float32)
    dl = prop.lb_target(psi, words, logits)
    W32 = W.astype(np.complex64).astype(np.complex128)
    b32 = b.astype(np.complex64).astype(np.complex128)
    ref = pr.lb_target(W32, b32, words, logits, N)
    scale = np.abs(ref).max()
    assert np.abs(dl - ref).max() <= 1e-4 * scale, (np.abs(dl - ref).max(), scale)
    # the target is a distribution's marginals: each walker's dl rows sum to zero
    np.testing.assert_allclose(dl[:, :N].sum(axis=1), 0.0, atol=1e-6)
