"""Fast sweep (MonteCarloLoop::set_fast_sweep, include/spin_ensembles/MonteCarloLoop.hpp:
108-113, 139-151, 162-171, 288-291): the proposal flips the spins of a mask that is the AND
of num_tries random configurations; a thermalisation sweep is N such updates, a sampling
sweep one.

The reference's PsiDeep recomputes log psi from the spins for these moves (a Metropolis
chain of |psi|^2); its Psi keeps its angles unchanged, so its RBM chain accepts every move.
Here both networks follow the flipped sites (a Metropolis chain of |psi|^2 for both).
Checks: the RBM chains equal the restatement's FP32 replay bit for bit (spins, accept
counts) with the same Philox streams; the restated chain samples |psi|^2 (chi-square over
all states of a small RBM); the GPU chains of both networks reproduce exact energies.
"""
import numpy as np
import pytest

from golden_cases import Case
from oracle import pyoracle as po


def small_rbm(N, M, sigma, seed):
    rng = np.random.default_rng(seed)
    b = sigma * (rng.normal(size=M) + 1j * rng.normal(size=M))
    W = sigma * (rng.normal(size=(N, M)) + 1j * rng.normal(size=(N, M)))
    return b, W


def chi_square(p, states, n_bins_min=20):
    """chi-square of observed states against probabilities p over all states, states
    grouped (in order of p) so that every group expects at least n_bins_min counts"""
    n = len(states)
    counts = np.bincount(states.astype(np.int64), minlength=len(p)).astype(np.float64)
    order = np.argsort(p)
    chi2, dof, e_acc, o_acc = 0.0, -1, 0.0, 0.0
    for i in order:
        e_acc += n * p[i]
        o_acc += counts[i]
        if e_acc >= n_bins_min:
            chi2 += (o_acc - e_acc) ** 2 / e_acc
            dof += 1
            e_acc, o_acc = 0.0, 0.0
    return chi2, dof


# ----------------------------------------------------------------------------- CPU
def test_restated_fast_chain_samples_psi_squared():
    """N = 10, M = 20 RBM: the final states of 8192 independent restated fast-sweep chains
    (2 tries) follow |psi|^2 within a 5-sigma chi-square band."""
    N, M = 10, 20
    b, W = small_rbm(N, M, 0.15, 12)
    opsi = po.RBM(b, W, 1.0)
    chains = 8192
    spins, _, _, acc, rej = po.mc_run(opsi, None, chains, 1, 40, 3, seed=5, fast_sweep_tries=2, want_eloc=False)
    v = po.psi_vector(opsi)
    p = np.abs(v) ** 2
    p /= p.sum()
    chi2, dof = chi_square(p, spins[0, :, 0])
    assert dof > 50
    assert abs(chi2 - dof) < 5 * np.sqrt(2 * dof), (chi2, dof)
    assert 0 < acc.sum() < (acc + rej).sum()
    # control: the reference's own RBM fast sweep (restated with its FP64 arithmetic) keeps
    # the angles, accepts every move and does not sample |psi|^2
    spins, _, _, acc, rej = po.mc_run(opsi, None, chains, 1, 40, 3, seed=5, fast_sweep_tries=2, want_eloc=False,
                                      prec=po.OR_PREC_REF64)
    chi2, dof = chi_square(p, spins[0, :, 0])
    assert rej.sum() == 0
    assert chi2 > dof + 50 * np.sqrt(2 * dof), (chi2, dof)


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


@gpu
@pytest.mark.parametrize("N,M,tries", [(64, 128, 1), (64, 100, 3), (100, 200, 2), (150, 64, 4)])
def test_fast_sweep_chains_bit_exact_vs_restatement(N, M, tries):
    """Spins and accept counts of 64 chains equal the restatement's replay, one- to
    three-word spin sets, and the proposal count is N per thermalisation sweep and one
    per sampling sweep."""
    import rbmongpu_gb300 as rg
    b, W = small_rbm(N, M, 0.05, N + tries)
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    opsi = po.RBM(b, W, 1.0)
    chains, samples, sweeps, therm, seed = 64, 3, 7, 2, 41
    mc = rg.MonteCarloLoop(chains * samples, sweeps, therm, chains, seed=seed)
    mc.set_fast_sweep(tries)
    sp, _, _ = mc.samples(psi)
    ospins, _, _, oacc, orej = po.mc_run(opsi, None, chains, samples, sweeps, therm, seed=seed,
                                         fast_sweep_tries=tries, want_eloc=False)
    assert np.array_equal(sp.reshape(samples, chains, -1), ospins)
    acc, props = mc.acceptance()
    assert int(acc) == int(oacc.sum())
    assert int(props) == int((oacc + orej).sum()) == chains * (therm * N + samples * sweeps)


@gpu
def test_fast_sweep_rbm_energy_matches_exact_summation():
    import rbmongpu_gb300 as rg
    N, M = 12, 24
    b, W = small_rbm(N, M, 0.15, 3)
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    op = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    mc = rg.MonteCarloLoop(512 * 40, 2 * N, 20, 512, seed=6)
    mc.set_fast_sweep(2)
    _, _, el = mc.samples(psi, op)
    es = rg.ExactSummation(N)
    E = (rg.ExpectationValue()(psi, op, es) / psi.norm(es) ** 2).real
    se = el.real.reshape(40, 512).mean(axis=0).std() / np.sqrt(512)
    assert abs(el.real.mean() - E) < 5 * se + 1e-3, (el.real.mean(), E, se)
    assert 0.0 < mc.acceptance_rate < 1.0


@gpu
def test_fast_sweep_deep_energy_matches_exact():
    """PsiDeep (the reference's fast sweep is a Metropolis chain here too)."""
    import rbmongpu_gb300 as rg
    c = Case("deep8_sparse")
    b, cn, w, fw = c.deep()
    psi = rg.PsiDeep(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    op = rg.Operator(*c.op())
    mc = rg.MonteCarloLoop(512 * 40, 2 * c.N, 20, 512, seed=4)
    mc.set_fast_sweep(2)
    _, _, el = mc.samples(psi, op)
    E_exact = complex(c.s("E_re"), c.s("E_im"))
    se = el.real.reshape(40, 512).mean(axis=0).std() / np.sqrt(512)
    assert abs(el.real.mean() - E_exact.real) < 5 * se + 1e-3
    assert 0.0 < mc.acceptance_rate < 1.0


@gpu
def test_fast_sweep_with_total_z_is_rejected():
    import rbmongpu_gb300 as rg
    c = Case("c1_rbm_exact")
    b, W = c.rbm()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    mc = rg.MonteCarloLoop(64, 1, 1, 16, seed=1)
    mc.set_total_z_symmetry(0)
    mc.set_fast_sweep(2)
    with pytest.raises(rg.RbmgError):
        mc.samples(psi)
