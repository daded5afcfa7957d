"""Optimisers: the CPU restatement (oracle/optim_ref.py) against the reference's own
generators (tests/golden/optim_golden.npz, from pyRBMonGPU/gradient_descent.py), the
device kernels against both, and the fused ground-state step against the host loop the
reference runs (ExpectationValue.gradient, then the optimiser on the host).

Tolerances: the update kernels round every operation as numpy does, so the generators
match the reference within 1e-13 relative (the only library function is padam's pow);
the fused step forms the same FP64 gradient on the device and matches the host loop
within 1e-9 relative over several steps (FMA contraction of the host's complex products
differs between compilers).
"""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN, Case
from oracle import optim_ref as orf

GOLD = np.load(os.path.join(GOLDEN, "optim_golden.npz"))
STEPS = int(GOLD["steps"])


def golden_gradient(step, params):
    return GOLD["scale"] * (np.asarray(params) - GOLD["target"]) + 0.01 * step


def golden_kw(method):
    return {k: float(v) for k, v in GOLD[method + "_kw"]}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


# ----------------------------------------------------------------------------- CPU
@pytest.mark.parametrize("method", orf.METHODS)
def test_restatement_matches_reference_generators(method):
    traj = orf.run(method, GOLD["p0"], golden_gradient, STEPS, golden_kw(method))
    assert np.array_equal(traj, GOLD[method])


def test_restatement_detects_a_planted_mistake():
    """Adam with the standard bias correction is not the reference's Adam: the golden
    trajectory tells them apart."""
    traj = orf.run("adam", GOLD["p0"], golden_gradient, STEPS, golden_kw("adam"), bias_correction="standard")
    assert rel(traj, GOLD["adam"]) > 1e-3


def test_standard_bias_first_step_is_sign_step():
    """With 1 - beta^t the first Adam step is eta g / (|g| + eps) per component."""
    g = np.array([0.3 - 2j, -1.5 + 0.1j])
    p = orf.step("adam", np.zeros(2, complex), g, {}, dict(beta1=0.9, beta2=0.999, eta=0.1, epsilon=1e-8), 0,
                 "standard")
    want = -0.1 * (g.real / (np.abs(g.real) + 1e-8) + 1j * g.imag / (np.abs(g.imag) + 1e-8))
    assert np.allclose(p, want, rtol=1e-12, atol=0)


# ----------------------------------------------------------------------------- GPU
gpu = pytest.mark.gpu


@gpu
@pytest.mark.parametrize("method", orf.METHODS)
def test_device_generators_match_reference(method):
    from rbmongpu_gb300 import gradient_descent as gd
    kw = golden_kw(method)
    p0 = GOLD["p0"].copy()
    if method in ("momentum", "adagrad", "adadelta"):
        traj = np.array(getattr(gd, method)(p0, STEPS, golden_gradient, **kw))
    elif method == "padam":
        seen = []

        def gc(step, params):
            seen.append(np.array(params))
            return golden_gradient(step, params), 0.0
        list(__import__("itertools").islice(gd.padam_generator(p0, gc, **kw), STEPS + 1))
        traj = np.array(seen[1:STEPS + 1])
    else:
        gen = getattr(gd, f"{method}_generator")(p0, golden_gradient, **kw)
        traj = np.array([next(gen) for _ in range(STEPS)])
    assert rel(traj, GOLD[method]) < 1e-13, method


@gpu
def test_device_adam_standard_bias_and_callable_eta():
    from rbmongpu_gb300 import Optimizer
    hp = dict(beta1=0.9, beta2=0.999, eta=lambda k: 0.01 / (1 + k), epsilon=1e-8)
    opt = Optimizer("adam", GOLD["p0"].size, bias_correction="standard", **hp)
    p, state, q = GOLD["p0"].copy(), {}, GOLD["p0"].copy()
    for k in range(STEPS):
        p = opt.update(p, golden_gradient(k, p))
        q = orf.step("adam", q, golden_gradient(k, q), state, hp, k, "standard")
    assert rel(p, q) < 1e-13
    assert opt.num_steps == STEPS
    opt.reset()
    assert opt.num_steps == 0


def _psi_and_op(name):
    import rbmongpu_gb300 as rg
    c = Case(name)
    if c.kind == "rbm":
        b, W = c.rbm()
        psi = rg.Psi(np.zeros(c.N), np.zeros(c.N), b, W, c.prefactor, False, True)
    else:
        b, cn, w, fw = c.deep()
        cls = rg.PsiPair if c.kind == "pair" else rg.PsiDeep
        psi = cls(np.zeros(c.N), np.zeros(c.N), b, cn, w, fw, c.prefactor, False, True)
    return c, psi, rg.Operator(*c.op())


def _host_loop(method, psi, op, ens, steps, hp, bias="reference"):
    """The reference's loop: gradient from ExpectationValue, update on the host."""
    import rbmongpu_gb300 as rg
    ev = rg.ExpectationValue()
    params, state, energies = psi.params, {}, []
    for k in range(steps):
        at = orf.lookahead(params, state, hp) if method == "nag" else params
        psi.params = at
        g, E = ev.gradient(psi, op, ens)
        energies.append(E)
        params = orf.step(method, params, g, state, hp, k, bias)
    psi.params = params
    return np.array(energies), params


FUSED = [("c1_rbm_exact", "adam", dict(beta1=0.9, beta2=0.999, eta=4e-3, epsilon=1e-3)),
         ("c1_rbm_exact", "nag", dict(eta=0.05, gamma=0.9)),
         ("c1_rbm_exact", "rmsprop", dict(eta=1e-3, gamma=0.9, epsilon=1e-3)),
         ("deep8_sparse", "padam", dict(beta1=0.9, beta2=0.999, eta=1e-2, epsilon=1e-4, p=0.25)),
         ("deep10_dense", "momentum", dict(eta=0.02, gamma=0.9))]


@gpu
@pytest.mark.parametrize("name,method,hp", FUSED)
def test_fused_step_matches_host_loop_exact(name, method, hp):
    import rbmongpu_gb300 as rg
    c, psi_a, op = _psi_and_op(name)
    _, psi_b, _ = _psi_and_op(name)
    es = rg.ExactSummation(c.N)
    steps = 5
    E_host, p_host = _host_loop(method, psi_b, op, es, steps, hp)
    opt = rg.Optimizer(method, psi_a.num_params, **hp)
    E_dev = opt.run(psi_a, op, es, steps)
    assert rel(E_dev, E_host) < 1e-9
    assert rel(psi_a.params, p_host) < 1e-9
    # the device parameters are the ones the kernels read: the next energy agrees too
    ev = rg.ExpectationValue()
    assert abs(ev(psi_a, op, es) - ev(psi_b, op, es)) <= 1e-9 * abs(ev(psi_b, op, es))


@gpu
def test_fused_step_monte_carlo_matches_host_loop():
    import rbmongpu_gb300 as rg
    c, psi_a, op = _psi_and_op("c2_rbm_mc")
    _, psi_b, _ = _psi_and_op("c2_rbm_mc")
    hp = dict(beta1=0.9, beta2=0.999, eta=4e-3, epsilon=1e-3)
    mk = lambda: rg.MonteCarloLoop(1024, 1, 20, 256, True, seed=7)   # noqa: E731
    E_host, p_host = _host_loop("adam", psi_b, op, mk(), 3, hp)
    opt = rg.Optimizer("adam", psi_a.num_params, **hp)
    E_dev = opt.run(psi_a, op, mk(), 3)
    assert rel(E_dev, E_host) < 1e-9
    assert rel(psi_a.params, p_host) < 1e-9


@gpu
def test_set_params_between_fused_steps():
    """Parameters set from the host replace the device copy the optimiser updates."""
    import rbmongpu_gb300 as rg
    c, psi, op = _psi_and_op("c1_rbm_exact")
    es = rg.ExactSummation(c.N)
    opt = rg.Optimizer("vanilla", psi.num_params, eta=0.01)
    p0 = psi.params
    opt.step(psi, op, es)
    assert rel(psi.params, p0) > 0
    psi.params = p0
    g, E = rg.ExpectationValue().gradient(psi, op, es)
    E1 = opt.step(psi, op, es)
    assert abs(E1 - E) <= 1e-12 * abs(E)
    assert rel(psi.params, p0 - 0.01 * g) < 1e-12
