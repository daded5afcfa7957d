"""The plain Metropolis configuration at its own size: 4096 walkers of the N=64, M=128 complex
RBM (sigma 0.05) on the periodic 8x8 transverse-field Ising model (J = 1, h = 3), 200
thermalisation sweeps, then 1000 measured sweeps of 64 single-flip proposals with E_loc and
O_k of every walker after every sweep (include/spin_ensembles/MonteCarloLoop.hpp:55-138).

* Chains: every sampled configuration and the accept count of 64 walkers spread over the
  4096 equal the FP32 replay of the restatement (oracle/oracle.c, the CUDA sampler's
  operation order, the same Philox streams) bit for bit -- 1000 configurations each.
* Estimators on the GPU's own samples: <E> and the reference O_k gradient
  <E O_k*> + conj<E_k> - 2<E><O_k*> (source/network_functions/ExpectationValue.cu:177-256)
  of 2048 of the run's samples against the FP64 restatement (1e-5 relative; vectors
  relative to their largest entry), and over all 4 096 000 samples: the sums the sampler
  pass accumulates chunk by chunk equal those of the same configurations evaluated as a
  fixed sample set (a different chunking), and <E> equals the mean of the per-sample local
  energies.
"""
import numpy as np
import pytest

import rbmongpu_gb300 as rg
from golden_cases import Case
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

CHAINS, SWEEPS, THERM, SEED = 4096, 1000, 200, 2024
RTOL = 1e-5


def vec_close(g, og, rtol=RTOL):
    scale = np.abs(og).max()
    assert np.abs(g - og).max() <= rtol * scale, (np.abs(g - og).max(), scale)


@pytest.fixture(scope="module")
def run():
    c = Case("c2_rbm_mc")
    b, W = c.rbm()
    psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    op_t = c.op()
    op = rg.Operator(*op_t)
    mc = rg.MonteCarloLoop(CHAINS * SWEEPS, 1, THERM, CHAINS, seed=SEED)
    sp, _, el = mc.samples(psi, op, log_psi=False)
    acc, props, per_chain = mc.acceptance(per_chain=True)
    return dict(c=c, b=b, W=W, psi=psi, op_t=op_t, op=op, spins=sp, eloc=el, acc=acc, props=props,
                per_chain=per_chain)


def test_full_size_chains_bit_exact(run):
    assert run["spins"].shape == (CHAINS * SWEEPS, 1)
    assert run["props"] == CHAINS * (THERM + SWEEPS) * 64
    assert 0.0 < run["acc"] / run["props"] < 1.0
    walkers = np.linspace(0, CHAINS - 1, 64).astype(int)
    ospins, oacc, orej = po.mc_run_walkers(run["b"], run["W"], run["c"].prefactor, walkers, SWEEPS, THERM, SEED,
                                           CHAINS)
    gpu = run["spins"].reshape(SWEEPS, CHAINS, 1)[:, walkers]
    np.testing.assert_array_equal(gpu, ospins)
    np.testing.assert_array_equal(run["per_chain"][walkers], oacc)
    assert np.all(oacc + orej == (THERM + SWEEPS) * 64)
    assert int(run["per_chain"].sum()) == run["acc"]


def test_estimators_on_the_runs_samples_vs_restatement(run):
    rng = np.random.default_rng(7)
    rows = rng.choice(CHAINS * SWEEPS, 2048, replace=False)
    sub = run["spins"][rows]
    c = run["c"]
    g, E = rg.ExpectationValue().gradient(run["psi"], run["op"], rg.FixedSamples(c.N, sub))
    og, oE = po.samples_gradient(po.RBM(run["b"], run["W"], c.prefactor), po.Op(*run["op_t"]), sub)
    assert abs(E - oE) <= RTOL * abs(oE)
    vec_close(g, og)
    # the per-sample local energies the sampler pass returned, for these samples
    oel = np.array([po.local_energy(po.RBM(run["b"], run["W"], c.prefactor), po.Op(*run["op_t"]), s)
                    for s in sub[:256]])
    vec_close(run["eloc"][rows[:256]], oel)


def test_full_size_accumulation_equals_fixed_sample_sums(run):
    c = run["c"]
    ev = rg.ExpectationValue()
    g_mc, E_mc = ev.gradient(run["psi"], run["op"], rg.MonteCarloLoop(CHAINS * SWEEPS, 1, THERM, CHAINS, seed=SEED))
    g_fx, E_fx = ev.gradient(run["psi"], run["op"], rg.FixedSamples(c.N, run["spins"]))
    assert abs(E_mc - E_fx) <= RTOL * abs(E_fx)
    vec_close(g_mc, g_fx)
    assert abs(E_mc - run["eloc"].mean()) <= RTOL * abs(E_mc)
    assert np.all(np.isfinite(g_mc))
