"""Generate ``optim_golden.npz``: parameter trajectories of the reference's optimisers.

Loads ``pyRBMonGPU/gradient_descent.py`` from the reference sources by path (it needs
only numpy and itertools, not the compiled module) and runs every generator for a few
steps on a fixed complex gradient function, storing the parameters after each step.

    python tests/golden/make_optim_golden.py [reference root]

Needs the reference sources; the committed .npz is what the tests read.
"""
import importlib.util
import os
import sys
from itertools import islice

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STEPS = 6
P = 7


def load(root):
    path = os.path.join(root, "pyRBMonGPU", "gradient_descent.py")
    spec = importlib.util.spec_from_file_location("reference_gradient_descent", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def problem():
    rng = np.random.default_rng(2024)
    p0 = rng.normal(size=P) + 1j * rng.normal(size=P)
    target = rng.normal(size=P) + 1j * rng.normal(size=P)
    scale = rng.uniform(0.5, 2.0, size=P) + 1j * rng.uniform(-0.5, 0.5, size=P)
    return p0, target, scale


def gradient(target, scale):
    def g(step, params):
        return scale * (params - target) + 0.01 * step
    return g


CASES = {
    "vanilla": dict(eta=0.05),
    "nag": dict(eta=0.05, gamma=0.9),
    "rmsprop": dict(eta=0.01, gamma=0.9, epsilon=1e-3),
    "adam": dict(beta1=0.9, beta2=0.999, eta=4e-3, epsilon=1e-3),
    "padam": dict(beta1=0.9, beta2=0.999, eta=1e-2, epsilon=1e-4, p=0.25),
    "adamax": dict(beta1=0.9, beta2=0.999, eta=1e-2, epsilon=1e-4),
}
LISTS = {
    "momentum": dict(eta=0.05, gamma=0.9),
    "adagrad": dict(eta=0.05, epsilon=1e-3),
    "adadelta": dict(gamma=0.9, epsilon=1e-6),
}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RBMONGPU_REF")
    if not root:
        sys.exit("usage: %s <RBMonGPU checkout>  (or set RBMONGPU_REF)" % sys.argv[0])
    gd = load(root)
    p0, target, scale = problem()
    g = gradient(target, scale)
    out = dict(p0=p0, target=target, scale=scale, steps=STEPS)
    for name, kw in CASES.items():
        if name == "padam":
            traj, params = [], p0.copy()
            def gc(step, params, g=g):
                traj.append(params.copy())
                return g(step, params), 0.0
            list(islice(getattr(gd, "padam_generator")(params, gc, **kw), STEPS + 1))
            hist = traj[1:STEPS + 1]
        else:
            hist = list(islice(getattr(gd, f"{name}_generator")(p0.copy(), g, **kw), STEPS))
        out[name] = np.array(hist)
    for name, kw in LISTS.items():
        out[name] = np.array(getattr(gd, name)(p0.copy(), STEPS, g, **kw))
    for name, kw in {**CASES, **LISTS}.items():
        out[name + "_kw"] = np.array(list(kw.items()), dtype=object).astype(str)
    np.savez(os.path.join(HERE, "optim_golden.npz"), **out)
    print("wrote", ", ".join(k for k in out if not k.endswith("_kw")))


if __name__ == "__main__":
    main()
