"""Walker and proposal checkpoints: a chain restored from a checkpoint continues bit for
bit (spins, Philox positions, counters; the proposal's weights and Adam state)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rbm(N, M, seed, sigma=0.1):
    import rbmongpu_gb300 as rg
    rng = np.random.default_rng(seed)
    b = rng.normal(0, sigma, M) + 1j * rng.normal(0, sigma, M)
    W = rng.normal(0, sigma, (N, M)) + 1j * rng.normal(0, sigma, (N, M))
    return rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)


def test_plain_chain_resumes_bit_exactly(tmp_path):
    import rbmongpu_gb300 as rg
    psi = rbm(40, 80, 1)
    a = rg.Chain(psi, 512, seed=3)
    a.sweep_async(psi, None, 5)
    a.save(tmp_path / "walkers.npz")
    a.sweep_async(psi, None, 7)
    b = rg.Chain(psi, 512, seed=3)
    b.load(tmp_path / "walkers.npz")
    b.sweep_async(psi, None, 7)
    ca, cb = a.checkpoint(), b.checkpoint()
    for k in ca:
        np.testing.assert_array_equal(ca[k], cb[k])


def test_learned_chain_and_training_resume_bit_exactly():
    import rbmongpu_gb300 as rg
    N = 24
    psi = rbm(N, 48, 2, sigma=0.2)
    pa = rg.Proposal(N, seed=4)
    a = rg.Chain(psi, 1024, seed=5)
    a.sweep_async(psi, None, 3)
    a.learned_async(psi, None, pa, 20, train=256)
    ck_chain, ck_prop = a.checkpoint(), pa.checkpoint()
    a.learned_async(psi, None, pa, 20, train=256)
    pb = rg.Proposal(N, seed=99)
    pb.restore(ck_prop)
    b = rg.Chain(psi, 1024, seed=5)
    b.restore(ck_chain)
    b.learned_async(psi, None, pb, 20, train=256)
    for k, v in a.checkpoint().items():
        np.testing.assert_array_equal(v, b.checkpoint()[k])
    sa, sb = pa.checkpoint(), pb.checkpoint()
    for k in ("params", "m", "v"):
        np.testing.assert_array_equal(sa[k], sb[k])
    assert sa["steps"] == sb["steps"] == 40


def test_checkpoint_rejects_spins_beyond_n():
    import rbmongpu_gb300 as rg
    psi = rbm(10, 20, 3)
    c = rg.Chain(psi, 4, seed=1)
    c.sweep_async(psi, None, 1)
    ck = c.checkpoint()
    ck["spins"][0, 0] |= np.uint64(1 << 12)
    with pytest.raises(rg.RbmgError):
        c.restore(ck)


def test_sliced_frozen_steps_equal_one_stream():
    """The frozen learned steps of 8320 walkers as 2 or 4 slices on as many streams (4096 +
    4224; 2048 + 2048 + 2176 + 2048 walkers) give the chains, counters and measured local
    energies of one stream."""
    import torch
    import rbmongpu_gb300 as rg
    N, B, rows = 40, 8320, 3
    psi = rbm(N, 80, 7, sigma=0.15)
    op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    prop = rg.Proposal(N, seed=8)
    warm = rg.Chain(psi, 1024, seed=1)
    warm.learned_async(psi, None, prop, 30, train=512)
    runs = []
    for streams in (1, 2, 4):
        c = rg.Chain(psi, B, seed=12)
        c.set_learned_streams(streams)
        c.sweep_async(psi, None, 2)
        el = torch.zeros((rows, B, 2), dtype=torch.float64, device="cuda")
        c.learned_async(psi, op, prop, rows * 4 + 1, train=0, measure_every=4, d_eloc=el.data_ptr(),
                        stream=rg.library_stream())
        torch.cuda.synchronize()
        runs.append((c.checkpoint(), el.cpu().numpy()))
    ca, ea = runs[0]
    for cb, eb in runs[1:]:
        for k in ca:
            np.testing.assert_array_equal(ca[k], cb[k])
        np.testing.assert_array_equal(ea, eb)
    assert int(ca["accepts"].sum()) > 0
