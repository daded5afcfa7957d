"""The reference's gradient-descent methods (pyRBMonGPU/gradient_descent.py) with their
update and state on the device (``csrc/optim.cu``), and the fused ground-state step.

The generators and list functions keep the reference's names, arguments, defaults and
results: each step calls ``gradient_function(step, params)`` on the host, as the
reference does, and applies the method's update in a device kernel (the same rounding
as the reference's numpy expressions).  ``vanilla``, ``momentum`` and ``nag`` update the
caller's array in place, as the reference's ``params -= ...`` does.

``Optimizer`` is the extension that removes the host from the loop: ``step`` forms the
energy gradient on the device from the sampler's sums, updates the device copy of the
network's parameters and rewrites the parameters the kernels read; only the energy
returns to the host.
"""
import ctypes as C
from itertools import islice

import numpy as np

from ._lib import call, lib

_dp = C.POINTER(C.c_double)

METHODS = {"vanilla": 0, "momentum": 1, "nag": 2, "adagrad": 3, "adadelta": 4, "rmsprop": 5, "adam": 6,
           "padam": 7, "adamax": 8}
STANDARD_BIAS = 1

# the reference's defaults per method (gradient_descent.py signatures)
_DEFAULTS = {
    "vanilla": dict(eta=1e-3),
    "momentum": dict(eta=None, gamma=0.9),
    "nag": dict(eta=1e-1, gamma=0.9),
    "adagrad": dict(eta=None, epsilon=None),
    "adadelta": dict(gamma=None, epsilon=None),
    "rmsprop": dict(eta=None, gamma=0.9, epsilon=1e-3),
    "adam": dict(beta1=0.9, beta2=0.999, eta=4e-3, epsilon=1e-3),
    "padam": dict(beta1=0.9, beta2=0.999, eta=1e-1, epsilon=1e-4, p=1 / 4),
    "adamax": dict(beta1=0.9, beta2=0.999, eta=1e-3, epsilon=1e-4),
}


def pack(array):
    """gradient_descent.py:5-7: real vector [re, im] -> complex."""
    N = len(array) // 2
    return array[:N] + 1j * array[N:]


def unpack(array):
    """gradient_descent.py:10-11: complex -> real vector [re, im]."""
    return np.hstack((array.real, array.imag))


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Optimizer:
    """One of the reference's methods with its state (velocities, moments) on the device.

    ``method`` is a name of ``METHODS``; hyperparameters by the reference's names (``eta``,
    ``gamma``, ``beta1``, ``beta2``, ``epsilon``, ``p``), defaults as in the reference.
    ``eta`` may be a callable of the step count (the reference's rmsprop, padam, adamax).
    ``bias_correction="reference"`` divides Adam's moments by 1 - beta as the reference
    does (gradient_descent.py:147-148); ``"standard"`` by 1 - beta^t."""

    def __init__(self, method, num_params, bias_correction="reference", **hyper):
        if method not in METHODS:
            raise ValueError(f"unknown method {method!r}")
        if bias_correction not in ("reference", "standard"):
            raise ValueError("bias_correction is 'reference' or 'standard'")
        kw = dict(_DEFAULTS[method])
        kw.update(hyper)
        missing = [k for k, v in kw.items() if v is None]
        if missing:
            raise TypeError(f"{method} needs {', '.join(missing)}")
        self.method = method
        self.num_params = int(num_params)
        self.eta = kw.get("eta", 0.0)
        g = kw.get("gamma", kw.get("beta1", 0.0))
        h = np.array([0.0 if callable(self.eta) else float(self.eta), float(g), float(kw.get("beta2", 0.0)),
                      float(kw.get("epsilon", 0.0)), float(kw.get("p", 0.0))])
        flags = STANDARD_BIAS if bias_correction == "standard" else 0
        self._h = C.c_void_p()
        call("rbmg_optimizer_create", METHODS[method], self.num_params, _ptr(h), 5, flags, C.byref(self._h))

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            try:
                lib().rbmg_optimizer_destroy(h)
            except Exception:
                pass

    def _eta(self):
        return float(self.eta(self.num_steps)) if callable(self.eta) else -1.0

    @property
    def num_steps(self):
        n = C.c_uint64()
        call("rbmg_optimizer_num_steps", self._h, C.byref(n))
        return n.value

    def reset(self):
        call("rbmg_optimizer_reset", self._h)

    def update(self, params, gradient):
        """One step with a host gradient -> the new parameters (complex128 copy)."""
        p = np.array(params, dtype=np.complex128, copy=True).reshape(-1)
        g = np.ascontiguousarray(np.asarray(gradient, dtype=np.complex128).reshape(-1))
        if p.size != self.num_params or g.size != self.num_params:
            raise ValueError("params / gradient have the wrong length")
        call("rbmg_optimizer_update", self._h, _ptr(p.view(np.float64)), _ptr(g.view(np.float64)), self._eta())
        return p

    def lookahead(self, params):
        """NAG's evaluation point params - gamma velocity."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.complex128).reshape(-1))
        out = np.empty_like(p)
        call("rbmg_optimizer_lookahead", self._h, _ptr(p.view(np.float64)), _ptr(out.view(np.float64)))
        return out

    def step(self, psi, operator_, spin_ensemble):
        """Fused ground-state step: <H> and its gradient at psi's parameters, the update
        applied on the device.  -> the energy (complex) before the update."""
        e = np.zeros(2)
        call("rbmg_optimizer_step_energy", self._h, psi._h, operator_._h, spin_ensemble._h, self._eta(), _ptr(e))
        return complex(e[0], e[1])

    def run(self, psi, operator_, spin_ensemble, num_steps):
        """num_steps fused steps -> the energies (complex array)."""
        return np.array([self.step(psi, operator_, spin_ensemble) for _ in range(int(num_steps))])


# ------------------------------------------------------------------ the reference's generators
def _device(method, params, **kw):
    return Optimizer(method, np.asarray(params).size, **kw)


def _inplace(params, new):
    if isinstance(params, np.ndarray) and params.dtype == np.complex128:
        params[...] = new
        return params
    return new


def vanilla_generator(params, gradient_function, eta=1e-3):
    opt, step = _device("vanilla", params, eta=eta), 0
    while True:
        params = _inplace(params, opt.update(params, gradient_function(step, params)))
        yield +params
        step += 1


def vanilla(params, num_steps, gradient_function, eta):
    return list(islice(vanilla_generator(params, gradient_function, eta), num_steps))


def momentum(params, num_steps, gradient_function, eta, gamma=0.9):
    opt, history = _device("momentum", params, eta=eta, gamma=gamma), []
    for step in range(num_steps):
        params = _inplace(params, opt.update(params, gradient_function(step, params)))
        history.append(+params)
    return history


def nag_generator(params, gradient_function, eta=1e-1, gamma=0.9, **kwargs):
    opt, step = _device("nag", params, eta=eta, gamma=gamma), 0
    while True:
        gradient = gradient_function(step, opt.lookahead(params))
        params = _inplace(params, opt.update(params, gradient))
        yield +params
        step += 1


def nag(params, num_steps, gradient_function, eta=1e-1, gamma=0.9):
    return list(islice(nag_generator(params, gradient_function, eta, gamma), num_steps))


def _generic(method, params, gradient_function, with_cost=False, params_filter=None, **kw):
    opt = _device(method, params, **kw)
    p, step = np.array(params, dtype=np.complex128, copy=True), 0
    while True:
        res = gradient_function(step, p)
        gradient, cost = res if with_cost else (res, None)
        p = opt.update(p, gradient)
        if params_filter is not None:
            p = np.asarray(params_filter(step, p), dtype=np.complex128)
        yield cost if with_cost else p
        step += 1


def adagrad(params, num_steps, gradient_function, eta, epsilon):
    return list(islice(_generic("adagrad", params, gradient_function, eta=eta, epsilon=epsilon), num_steps))


def adadelta(params, num_steps, gradient_function, gamma, epsilon):
    return list(islice(_generic("adadelta", params, gradient_function, gamma=gamma, epsilon=epsilon), num_steps))


def rmsprop_generator(params, gradient_function, eta, gamma=0.9, epsilon=1e-3, **kwargs):
    return _generic("rmsprop", params, gradient_function, eta=eta, gamma=gamma, epsilon=epsilon)


def rmsprop(params, num_steps, gradient_function, eta, gamma, epsilon):
    return list(islice(rmsprop_generator(params, gradient_function, eta, gamma, epsilon), num_steps))


def adam_generator(params, gradient_function, beta1=0.9, beta2=0.999, eta=4e-3, epsilon=1e-3, **kwargs):
    return _generic("adam", params, gradient_function, beta1=beta1, beta2=beta2, eta=eta, epsilon=epsilon,
                    bias_correction=kwargs.get("bias_correction", "reference"))


def adam(params, num_steps, gradient_function, beta1=0.9, beta2=0.999, eta=4e-3, epsilon=1e-3):
    return list(islice(adam_generator(params, gradient_function, beta1, beta2, eta, epsilon), num_steps))


def padam_generator(params, gradient_function, beta1=0.9, beta2=0.999, eta=1e-1, epsilon=1e-4, p=1 / 4, **kwargs):
    """gradient_function returns (gradient, cost); yields the cost, as the reference does."""
    return _generic("padam", params, gradient_function, with_cost=True, beta1=beta1, beta2=beta2, eta=eta,
                    epsilon=epsilon, p=p)


def padam(params, num_steps, gradient_function, beta1=0.9, beta2=0.999, eta=1e-1, epsilon=1e-4, p=1 / 4):
    return list(islice(padam_generator(params, gradient_function, beta1, beta2, eta, epsilon, p), num_steps))


def adamax_generator(params, gradient_function, beta1=0.9, beta2=0.999, eta=1e-3, epsilon=1e-4, params_filter=None,
                     **kwargs):
    return _generic("adamax", params, gradient_function, params_filter=params_filter, beta1=beta1, beta2=beta2,
                    eta=eta, epsilon=epsilon)


def adamax(params, num_steps, gradient_function, beta1=0.9, beta2=0.999, eta=1e-3, epsilon=1e-4, params_filter=None):
    return list(islice(adamax_generator(params, gradient_function, beta1, beta2, eta, epsilon, params_filter),
                       num_steps))
