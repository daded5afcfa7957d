"""CPU restatement of the reference's gradient-descent optimisers (numpy, FP64).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the device optimiser
kernels (``csrc/optim.cu``).  The product package never imports it.

One step of each method, following ``pyRBMonGPU/gradient_descent.py`` of the reference
(line numbers cite that file).  Every method there works elementwise on the real vector
``hstack(params.real, params.imag)`` (``unpack``, :10-11), so it is stated here on the
real and imaginary parts separately, which is the same arithmetic.  Pinned against the
reference's own generators by ``tests/golden/optim_golden.npz``.

``step(method, params, grad, state, hp, k)`` returns the new parameters; ``state`` is a
dict updated in place; ``k`` counts steps from 0.
"""
import numpy as np

METHODS = ("vanilla", "momentum", "nag", "adagrad", "adadelta", "rmsprop", "adam", "padam", "adamax")


def _re(z):
    z = np.asarray(z, np.complex128)
    return np.concatenate([z.real, z.imag])


def _cx(x):
    n = len(x) // 2
    return x[:n] + 1j * x[n:]


def lookahead(params, state, hp):
    """NAG evaluates the gradient at params - gamma * velocity (:56)."""
    v = state.get("velocity", 0.0)
    return params - hp["gamma"] * v


def step(method, params, grad, state, hp, k=0, bias_correction="reference"):
    p = _re(params)
    g = _re(grad)
    eta = hp.get("eta", 0.0)
    eta = eta(k) if callable(eta) else eta
    if method == "vanilla":                       # :19
        p = p - eta * g
    elif method in ("momentum", "nag"):           # :42-44, :56-58
        v = state.get("v", 0.0)
        v = hp["gamma"] * v + eta * g
        state["v"] = v
        state["velocity"] = _cx(v)
        p = p - v
    elif method == "adagrad":                     # :77-80
        G = state.get("G", 0.0) + g ** 2
        state["G"] = G
        p = p - eta / (G + hp["epsilon"]) * g
    elif method == "adadelta":                    # :96-105
        gm, eps = hp["gamma"], hp["epsilon"]
        dp = state.get("dp", 0.0)
        Edp2 = gm * state.get("Edp2", 0.0) + (1 - gm) * dp ** 2
        Eg2 = gm * state.get("Eg2", 0.0) + (1 - gm) * g ** 2
        dp = -((Edp2 + eps) ** 0.5) / ((Eg2 + eps) ** 0.5) * g
        state.update(dp=dp, Edp2=Edp2, Eg2=Eg2)
        p = p + dp
    elif method == "rmsprop":                     # :119-123
        G = hp["gamma"] * state.get("G", 0.0) + (1 - hp["gamma"]) * g ** 2
        state["G"] = G
        p = p - eta / (G + hp["epsilon"]) * g
    elif method == "adam":                        # :144-150
        b1, b2 = hp["beta1"], hp["beta2"]
        m = b1 * state.get("m", 0.0) + (1 - b1) * g
        v = b2 * state.get("v", 0.0) + (1 - b2) * g ** 2
        state.update(m=m, v=v)
        if bias_correction == "reference":        # :147-148: no power of the step count
            mh, vh = m / (1 - b1), v / (1 - b2)
        else:                                     # Kingma & Ba (2015)
            mh, vh = m / (1 - b1 ** (k + 1)), v / (1 - b2 ** (k + 1))
        p = p - eta / (vh ** 0.5 + hp["epsilon"]) * mh
    elif method == "padam":                       # :170-179
        b1, b2 = hp["beta1"], hp["beta2"]
        m = b1 * state.get("m", 0.0) + (1 - b1) * g
        v = b2 * state.get("v", 0.0) + (1 - b2) * g ** 2
        vhat = np.maximum(state.get("vhat", 0.0), v)
        state.update(m=m, v=v, vhat=vhat)
        p = p - eta / (vhat ** hp["p"] + hp["epsilon"]) * m
    elif method == "adamax":                      # :200-206
        b1, b2 = hp["beta1"], hp["beta2"]
        m = b1 * state.get("m", 0.0) + (1 - b1) * g
        mh = m / (1 - b1)
        u = np.maximum(b2 * state.get("u", 0.0), np.abs(g))
        state.update(m=m, u=u)
        p = p - eta / (u + hp["epsilon"]) * mh
    else:
        raise ValueError(method)
    return _cx(p)


def run(method, p0, gradient, steps, hp, bias_correction="reference"):
    """Parameters after each of `steps` steps with gradient(step, params)."""
    params, state, out = np.asarray(p0, np.complex128).copy(), {}, []
    for k in range(steps):
        at = lookahead(params, state, hp) if method == "nag" else params
        params = step(method, params, gradient(k, at), state, hp, k, bias_correction)
        out.append(params.copy())
    return np.array(out)
