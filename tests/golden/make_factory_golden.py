"""Golden networks of the reference's factories (pyRBMonGPU/new_neural_network.py), for
tests/test_factories.py: the reference module is loaded from an RBMonGPU checkout with its
Psi / PsiDeep / PsiPair replaced by recorders of their constructor arguments, numpy is
seeded, and the arrays the factories pass are stored in factory_golden.npz.

    python tests/golden/make_factory_golden.py <RBMonGPU checkout>   (or set RBMONGPU_REF)
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (name, factory, args, kwargs, numpy seed)
CASES = [
    ("rbm", "new_neural_network", (8, 16), {}, 1),
    ("deep1d", "new_deep_neural_network", (8, [16, 8], [4, 8]), {}, 2),
    ("pair1d", "new_deep_neural_network", (6, [12, 6], [3, 6]), {"pair": True}, 3),
    ("deep2d", "new_deep_neural_network", ((4, 4), [(4, 4), (2, 2)], [(2, 2), (4, 4)]), {}, 4),
    ("deep2d_rect", "new_deep_neural_network", ((4, 2), [(4, 2), (2, 2)], [(3, 2), (4, 2)]), {"final_weights": 3.0}, 5),
]


class Recorder:
    def __init__(self, *args):
        self.args = args


def flatten(name, rec, out):
    kind = "rbm" if len(rec.args) == 7 else "deep"
    a = rec.args
    out[f"{name}_alpha"] = np.asarray(a[0])
    out[f"{name}_beta"] = np.asarray(a[1])
    if kind == "rbm":
        out[f"{name}_b"] = np.asarray(a[2])
        out[f"{name}_W"] = np.asarray(a[3])
        return
    for l, (b, c, w) in enumerate(zip(a[2], a[3], a[4])):
        out[f"{name}_b{l}"] = np.asarray(b)
        out[f"{name}_conn{l}"] = np.asarray(c)
        out[f"{name}_W{l}"] = np.asarray(w)
    out[f"{name}_fw"] = np.asarray(a[5])


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RBMONGPU_REF")
    if not root:
        sys.exit("usage: %s <RBMonGPU checkout>  (or set RBMONGPU_REF)" % sys.argv[0])
    spec = importlib.util.spec_from_file_location("reference_factories",
                                                  os.path.join(root, "pyRBMonGPU", "new_neural_network.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.Psi = mod.PsiDeep = mod.PsiPair = Recorder
    out = {}
    for name, fn, args, kw, seed in CASES:
        np.random.seed(seed)
        flatten(name, getattr(mod, fn)(*args, **kw), out)
    np.savez(os.path.join(HERE, "factory_golden.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
