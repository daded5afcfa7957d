"""Loads the golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py
from the reference itself) into plain numpy structures shared by the tests."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class Case:
    def __init__(self, name):
        self.name = name
        self.z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
        self.kind = str(self.z["m_kind"])
        self.N = int(self.z["m_N"])

    def meta(self, k, default=None):
        return self.z["m_" + k].item() if ("m_" + k) in self.z else default

    def s(self, k):
        return float(self.z["s_" + k])

    def o(self, k):
        return self.z["o_" + k]

    def i(self, k):
        return self.z["i_" + k]

    def has(self, k):
        return k in self.z

    def op(self, prefix="op_"):
        return self.i(prefix + "coef"), self.i(prefix + "types"), self.i(prefix + "idx")

    @property
    def prefactor(self):
        return self.s("prefactor") if self.has("s_prefactor") else 1.0

    # free quantum axis: (alpha angles [N], flag); the reference sets beta = alpha
    def quaxis(self, prefix=""):
        if self.meta("fqa", 0):
            return self.i(prefix + "alpha"), True
        return np.zeros(self.N), False

    # RBM parameters
    def rbm(self, prefix=""):
        N, M = self.N, int(self.meta("M"))
        return self.i(prefix + "b"), self.i(prefix + "W").reshape(N, M)

    # PsiDeep / PsiPair parameters: (biases, connections, weights, final_weights)
    def deep(self, prefix=""):
        L = int(self.meta("layers"))
        b, c, w = [], [], []
        for l in range(L):
            size, conn = int(self.meta(f"size{l}")), int(self.meta(f"conn{l}"))
            b.append(self.i(f"{prefix}b{l}"))
            c.append(self.i(f"{prefix}conn{l}").reshape(conn, size))
            w.append(self.i(f"{prefix}W{l}").reshape(conn, size))
        return b, c, w, self.i(prefix + "fw")


ALL = ["c1_rbm_exact", "rbm6_hsd_nonunitary", "rbm8_mixed_operator", "c2_rbm_mc", "deep8_sparse",
       "deep10_dense", "pair3", "rbm6_hsd_fqa", "deep6_hsd_fqa"]
