"""Host logic of the autograd wrapper (rbmongpu_gb300/autograd.py), with the library's
estimators replaced by fakes that count their calls: when autograd records the call, the
forward pass runs the adjoint once and the backward pass returns its gradient; under
no_grad (or for a tensor without requires_grad) the forward pass evaluates the energy only
and no gradient work is done; the backward pass without a stored gradient evaluates it on
the forward pass's own samples."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import rbmongpu_gb300.autograd as ag   # noqa: E402


class FakePsi:
    N = 4

    def __init__(self):
        self.params = np.zeros(3, np.complex128)


class FakeMC:
    pass


class Calls:
    def __init__(self):
        self.grad = 0
        self.energy = 0
        self.samples = 0
        self.grad_ensembles = []


@pytest.fixture
def fakes(monkeypatch):
    calls = Calls()
    g = np.array([1.0 + 2.0j, -0.5j, 3.0])

    class FakeEV:
        def eloc_gradient(self, psi, op, ensemble, score):
            calls.grad += 1
            calls.grad_ensembles.append(ensemble)
            return g * (1.0 + float(np.abs(psi.params).sum())), complex(-2.5, 0.1)

        def __call__(self, psi, op, ensemble):
            calls.energy += 1
            return complex(-2.5, 0.0)

    class FakeFixed:
        def __init__(self, N, spins):
            self.spins = spins

    def samples(self, psi, op, log_psi=False):
        calls.samples += 1
        return np.zeros((8, 1), np.uint64), None, np.full(8, -2.5 + 0j)

    monkeypatch.setattr(ag, "ExpectationValue", FakeEV)
    monkeypatch.setattr(ag, "FixedSamples", FakeFixed)
    monkeypatch.setattr(ag, "MonteCarloLoop", FakeMC)
    monkeypatch.setattr(FakeMC, "samples", samples, raising=False)
    return calls, g


def test_recorded_call_runs_the_adjoint_once_in_the_forward_pass(fakes):
    calls, g = fakes
    params = torch.tensor(np.array([0.1, 0.2j, 0.0]), requires_grad=True)
    E = ag.energy(params, FakePsi(), None, FakeMC())
    assert E.item() == -2.5
    assert (calls.grad, calls.energy, calls.samples) == (1, 0, 0)
    assert params.grad is None
    E.backward()
    assert calls.grad == 1          # the stored gradient, no second pass
    np.testing.assert_allclose(params.grad.numpy(), g * 1.3)


def test_no_grad_forward_does_no_gradient_work(fakes):
    calls, _ = fakes
    params = torch.tensor(np.array([0.1, 0.2j, 0.0]), requires_grad=True)
    with torch.no_grad():
        E = ag.energy(params, FakePsi(), None, FakeMC())
    assert E.item() == -2.5
    assert (calls.grad, calls.energy, calls.samples) == (0, 0, 1)
    E2 = ag.energy(torch.tensor(np.zeros(3, np.complex128)), FakePsi(), None, object())
    assert E2.item() == -2.5
    assert (calls.grad, calls.energy) == (0, 1)


def test_backward_without_a_stored_gradient_uses_the_forward_samples(fakes):
    calls, g = fakes
    params = torch.tensor(np.array([0.1, 0.2j, 0.0]), requires_grad=True)
    psi = FakePsi()
    E = ag.LocalEnergy.apply(params, psi, None, FakeMC(), True, False)
    assert (calls.grad, calls.samples) == (0, 1)
    psi.params = np.full(3, 9.0 + 0j)   # the backward pass restores the forward's parameters
    E.backward()
    assert calls.grad == 1
    assert hasattr(calls.grad_ensembles[0], "spins")   # the forward pass's samples
    np.testing.assert_allclose(params.grad.numpy(), g * 1.3)


def test_params_must_be_complex(fakes):
    with pytest.raises(TypeError):
        ag.energy(torch.zeros(3, dtype=torch.float64), FakePsi(), None, FakeMC())
