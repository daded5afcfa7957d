"""Batched serving of uneven complex RBMs (one persistent launch replayed from a CUDA
graph): chains identical to the single-network chains with the same Philox streams, the
N=16 instances against FP64 exact summation, and the autotuner.

Tolerances: local energies within 1e-6 relative of the single-network pass (the same
FP32 operation order; the serving kernel only reads the angles from a runtime count of
hidden units per lane); every instance's gradient -- the reference's estimator
<E O*> + conj<E_k> - 2 <E> <O*> -- within 1e-5 of its largest entry of the single-network
gradient on the same configurations, and bit-identical between tile shapes (fixed-order
sums); Monte-Carlo energies within 5 standard errors of exact summation and the gradient
within 15 % (relative L2 norm, statistical) for 4096 walkers x 16 replays.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rbm(N, alpha, seed, sigma=0.05):
    import rbmongpu_gb300 as rg
    rng = np.random.Generator(np.random.PCG64(seed))
    M = alpha * N
    b = rng.normal(0, sigma, M) + 1j * rng.normal(0, sigma, M)
    W = rng.normal(0, sigma, (N, M)) + 1j * rng.normal(0, sigma, (N, M))
    return rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)


@pytest.mark.parametrize("regs", [255, 128, 96])
def test_batch_chains_match_single_network_chains(regs):
    """Under every register cap of the persistent kernel the chains equal single-network
    chains (energies and accept counts)."""
    import torch
    import rbmongpu_gb300 as rg
    specs = [(16, 1, 0.7, 64), (24, 2, 1.3, 96), (40, 4, 1.9, 128), (72, 2, 1.0, 32), (136, 1, 0.5, 48)]
    inst, nets = [], []
    for q, (N, a, h, B) in enumerate(specs):
        psi = rbm(N, a, 105_000 + q)
        op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, h))
        nets.append((psi, op, B, 900 + q))
        inst.append((psi, op, B, 900 + q))
    batch = rg.Batch(inst)
    batch.register_cap = regs
    therm, sweeps = 7, 3
    batch.run(therm, sweeps)
    total_acc = 0
    for q, (psi, op, B, seed) in enumerate(nets):
        chain = rg.Chain(psi, B, seed=seed)
        el = torch.zeros((1, B, 2), dtype=torch.float64, device="cuda")
        chain.sweep_async(psi, op, therm + sweeps, therm + sweeps, el.data_ptr(), rg.library_stream())
        torch.cuda.synchronize()
        ref = el[0].cpu().numpy().view(np.complex128)[:, 0]
        _, _, got = batch.result(q, want_eloc=True)
        assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max(), q
        total_acc += chain.state()[1]
    assert batch.accepts() == total_acc


def test_served_gradient_is_the_reference_estimator_on_the_same_configurations():
    import rbmongpu_gb300 as rg
    specs = [(16, 1, 0.7, 64), (24, 2, 1.3, 96), (40, 4, 1.9, 300), (72, 2, 1.0, 32), (136, 1, 0.5, 520)]
    results = []
    for rows in (16, 8):
        inst = []
        for q, (N, a, h, B) in enumerate(specs):
            inst.append((rbm(N, a, 105_200 + q), rg.Operator(*rg.operators.tfim_chain(N, 1.0, h)), B, 300 + q))
        batch = rg.Batch(inst)
        batch.set_shape(4, rows)
        batch.run(20, 2)
        results.append([batch.result(q) for q in range(len(inst))])
        if rows == 16:
            for q, (psi, op, B, _) in enumerate(inst):
                E, g, _ = results[-1][q]
                g_ref, E_ref = rg.ExpectationValue().gradient(psi, op, rg.FixedSamples(psi.N, batch.spins(q)))
                assert abs(E - E_ref) <= 1e-6 * abs(E_ref), (q, E, E_ref)
                assert np.abs(g - g_ref).max() <= 1e-5 * np.abs(g_ref).max(), (q, np.abs(g - g_ref).max())
    # the sums are fixed-order: another tile height gives the same bits
    for (E1, g1, _), (E2, g2, _) in zip(*results):
        assert E1 == E2
        np.testing.assert_array_equal(g1, g2)


def mixed_chain(N, h):
    """TFIM chain plus an X X bond on sites 2, 3 and a Y field on site 5: sites flipped by
    one single-site string (the single-flip tiles) beside sites flipped by several strings
    or by a two-site string (the general tiles)."""
    import rbmongpu_gb300 as rg
    X, Y, Z = rg.operators.X, rg.operators.Y, rg.operators.Z
    strings = [[(Z, i), (Z, (i + 1) % N)] for i in range(N)] + [[(X, i)] for i in range(N)]
    strings += [[(X, 2), (X, 3)], [(Y, 5)]]
    return rg.operators.table(strings, [-1.0] * N + [-h] * N + [0.3, 0.2])


def test_served_gradient_with_multi_flip_strings():
    """Operators whose strings flip several sites, or several strings per site (Heisenberg
    chain; TFIM with an extra bond and a Y field): the general reduction tiles, alone and
    beside single-flip tiles of the same instance, give the reference estimator on the same
    configurations, and the same bits for both tile heights."""
    import rbmongpu_gb300 as rg
    specs = [(16, 2, "heis", 64), (24, 1, "mixed", 96), (40, 2, "mixed", 130), (20, 4, "tfim", 48)]
    results = []
    for rows in (16, 8):
        inst = []
        for q, (N, a, kind, B) in enumerate(specs):
            if kind == "heis":
                op = rg.operators.heisenberg_chain(N, 1.0)
            elif kind == "mixed":
                op = mixed_chain(N, 0.9 + 0.1 * q)
            else:
                op = rg.operators.tfim_chain(N, 1.0, 1.2)
            inst.append((rbm(N, a, 105_400 + q), rg.Operator(*op), B, 700 + q))
        batch = rg.Batch(inst)
        batch.set_shape(4, rows)
        batch.run(15, 2)
        results.append([batch.result(q) for q in range(len(inst))])
        if rows == 16:
            for q, (psi, op, B, _) in enumerate(inst):
                E, g, _ = results[-1][q]
                g_ref, E_ref = rg.ExpectationValue().gradient(psi, op, rg.FixedSamples(psi.N, batch.spins(q)))
                assert abs(E - E_ref) <= 1e-6 * abs(E_ref), (q, E, E_ref)
                assert np.abs(g - g_ref).max() <= 1e-5 * np.abs(g_ref).max(), (q, np.abs(g - g_ref).max())
    for (E1, g1, _), (E2, g2, _) in zip(*results):
        assert E1 == E2
        np.testing.assert_array_equal(g1, g2)


def test_n16_instances_match_exact_summation():
    import rbmongpu_gb300 as rg
    N, B, reps = 16, 4096, 16
    inst = []
    for q, a in enumerate((1, 2, 4)):
        psi = rbm(N, a, 105_100 + q, sigma=0.1)
        op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 0.5 + 0.5 * q))
        inst.append((psi, op, B, 70 + q))
    batch = rg.Batch(inst + [(rbm(48, 2, 7), rg.Operator(*rg.operators.tfim_chain(48, 1.0, 1.0)), 512, 5)])
    batch.run(50, 2)
    E_acc = [[] for _ in inst]
    g_acc = [0 for _ in inst]
    for r in range(reps):
        batch.run(0, 2)
        for q in range(len(inst)):
            E, g, el = batch.result(q, want_eloc=True)
            E_acc[q].append(el)
            g_acc[q] = g_acc[q] + g / reps
    es = rg.ExactSummation(N)
    for q, (psi, op, _, _) in enumerate(inst):
        psi.prefactor = 1.0 / psi.norm(es)
        gx, Ex = rg.ExpectationValue().gradient(psi, op, es)
        el = np.array(E_acc[q])
        se = el.real.mean(axis=0).std() / np.sqrt(B)
        assert abs(el.real.mean() - Ex.real) < 5 * se + 1e-4, (q, el.real.mean(), Ex.real, se)
        err = np.linalg.norm(g_acc[q] - gx) / np.linalg.norm(gx)
        assert err < 0.15, (q, err)


def test_autotune_keeps_the_fastest_shape():
    import rbmongpu_gb300 as rg
    rng = np.random.default_rng(105)
    inst = []
    for q in range(12):
        N = int(rng.choice(np.arange(16, 145, 8)))
        a = int(rng.choice([1, 2, 4]))
        op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, float(rng.uniform(0.5, 2.0))))
        inst.append((rbm(N, a, 105_000 + q), op, 256 * N // 16 // 4, q))
    batch = rg.Batch(inst)
    times = batch.autotune(sweeps=1, reps=2)
    assert len(times) == 18 and all(t > 0 for t in times.values())
    w, r, blocks = batch.shape
    assert times[(batch.register_cap, w, r)] == min(times.values()) and blocks > 0
    batch.run(0, 1)
    E, g, _ = batch.result(0)
    assert np.isfinite(E) and np.all(np.isfinite(g))


def test_a_wait_that_runs_out_is_reported_and_the_device_stays_usable():
    """Failure detection without a GPU fault: the reduction tasks wait for one walker more
    than each instance has, so the bounded wait (0.2 s) runs out; the replay reports
    RBMG_ETIMEOUT, and the next replay with the ordinary wait succeeds."""
    import rbmongpu_gb300 as rg
    inst = [(rbm(16, 1, 106_000 + q), rg.Operator(*rg.operators.tfim_chain(16, 1.0, 1.0)), 64, q) for q in range(3)]
    batch = rg.Batch(inst)
    batch.set_wait(0.2, extra_walkers=1)
    with pytest.raises(rg.RbmgError) as err:
        batch.run(0, 1)
    assert err.value.code == 4   # RBMG_ETIMEOUT
    batch.set_wait(20.0, extra_walkers=0)
    batch.run(0, 2)
    for q in range(3):
        E, g, _ = batch.result(q)
        assert np.isfinite(E) and np.all(np.isfinite(g))
