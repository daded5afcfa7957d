"""The network factories (rbmongpu_gb300.api.new_neural_network / new_deep_neural_network,
pyRBMonGPU/new_neural_network.py:29-153) give the reference's networks for the same numpy
seed: every array they pass to the Psi / PsiDeep / PsiPair constructors equals the one the
reference's own factories pass (tests/golden/factory_golden.npz, written by
tests/golden/make_factory_golden.py), 1D and 2D connection patterns included."""
import os

import numpy as np
import pytest

from rbmongpu_gb300 import api

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "factory_golden.npz")
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


@pytest.mark.parametrize("name,fn,args,kw,seed", CASES)
def test_factory_builds_the_reference_network(name, fn, args, kw, seed, monkeypatch):
    for cls in ("Psi", "PsiDeep", "PsiPair"):
        monkeypatch.setattr(api, cls, Recorder)
    g = np.load(GOLDEN)
    np.random.seed(seed)
    a = getattr(api, fn)(*args, **kw).args
    np.testing.assert_array_equal(a[0], g[f"{name}_alpha"])
    np.testing.assert_array_equal(a[1], g[f"{name}_beta"])
    if name == "rbm":
        np.testing.assert_array_equal(a[2], g["rbm_b"])
        np.testing.assert_array_equal(a[3], g["rbm_W"])
        return
    for l, (b, c, w) in enumerate(zip(a[2], a[3], a[4])):
        np.testing.assert_array_equal(b, g[f"{name}_b{l}"])
        np.testing.assert_array_equal(c, g[f"{name}_conn{l}"])
        np.testing.assert_array_equal(w, g[f"{name}_W{l}"])
    np.testing.assert_array_equal(a[5], g[f"{name}_fw"])
